"""Shared test helpers: workload generators and comparison metrics."""
from __future__ import annotations

import numpy as np


# Per-entry floors (fractions of max|ref|) of the entry-wise metric.  With the
# FP64 bar 1e-12 the floor 1e-2 gives every entry the tolerance
# max(1e-12 |ref_i|, 1e-14 max|ref|): relative 1e-12 for entries down to 1% of
# the largest, and an absolute floor of 1e-14 max|ref| (about 90 ulps of the
# largest entry) below that.  A floor on the relative error itself cannot be
# smaller: assembled matrices hold entries that are rounding residue of
# analytically zero sums (23% of the 32^3 Poisson CSC entries have
# |ref_i| <= 1.7e-15 max|ref|), which any two correct FP64 computations
# reproduce only to about 1e-16 max|ref| in absolute terms.  The FP32-element
# bar 1e-5 uses 1e-1 (absolute floor 1e-6 max|ref|, about 17 FP32 ulps).
FLOOR64 = 1e-2
FLOOR32 = 1e-1


def rel_err(a, b, floor: float = FLOOR64) -> tuple[float, float, float]:
    """(max |a-b| / max |b|,  ||a-b||_2 / ||b||_2,  max_i |a_i-b_i| / max(|b_i|, floor max|b|)).

    The third is the entry-wise relative error: every entry is held to the bar
    relative to its own size, entries smaller than floor * max|b| relative to
    that floor."""
    a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
    if not b.size:
        return 0.0, 0.0, 0.0
    d = np.abs(a - b)
    s = np.abs(b).max()
    n = np.linalg.norm(b)
    s = s if s > 0 else 1.0
    n = n if n > 0 else 1.0
    per = d / np.maximum(np.abs(b), floor * s)
    return float(d.max() / s), float(np.linalg.norm(a - b) / n), float(per.max())


def residual_err(a, b, abs_sum, floor: float = FLOOR64) -> tuple[float, float, float]:
    """rel_err for an assembled residual.  Its entries come out of cancelling
    sums -- element forces near equilibrium, stress components that vanish
    (uniaxial stress), and displacement gradients formed from nodal
    displacements much larger than their differences -- so the entry-wise term
    holds entry i to the bar relative to max(|b_i|, floor * abs_sum_i), with
    abs_sum_i the summed magnitude of every term the entry is formed from,
    down to the nodal values (the oracle's abs_out): relative to the entry
    itself, with an absolute floor of bar * floor (1e-14 for FP64) times the
    terms it sums."""
    a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
    m, n2, _ = rel_err(a, b)
    if not b.size:
        return m, n2, 0.0
    per = np.abs(a - b) / np.maximum(np.maximum(np.abs(b), floor * np.asarray(abs_sum, dtype=np.float64)), 1e-300)
    return m, n2, float(per.max())


def entry_err(a, b, floor: float) -> float:
    """Entry-wise relative error with the given floor (informational output)."""
    return rel_err(a, b, floor)[2]


from fec_gb300.workloads import stretch_field  # noqa: F401  (re-exported for the tests)


def blocks_of(mesh):
    return [(mesh.element_types[b], mesh.element_conns[b]) for b in mesh.element_block_names]


def adjacent_elements(conns, nodes):
    """{node (0-based): [(element, local index), ...]} for the given nodes, elements ascending.
    conns: (NE, NNPE) 1-based."""
    nodes = np.asarray(nodes, dtype=np.int64)
    out = {int(n): [] for n in nodes}
    hit = np.isin(conns, nodes + 1)
    for e, a in zip(*np.nonzero(hit)):
        out[int(conns[e, a]) - 1].append((int(e), int(a)))
    return out


def sampled_columns(orc, blocks, X, U, phys, props, nodes, dof_to_unknown, nf, states=None):
    """Expected CSC columns (and residual entries) of the given nodes from the
    oracle's element matrices of their adjacent elements.

    blocks: [(elem type, conns (NE, NNPE) 1-based)], U the full field, states a
    list (per block) of (NS, NQ, NE) state_old arrays or None.  Returns
    {unknown column (0-based): {unknown row (0-based): value}} and
    {unknown dof (0-based): residual value} for the nodes' unknown dofs, the
    matrix in the reference's storage convention (entry (I, J) = sum over
    elements of dR_J / du_I, K_el stored column-major)."""
    U = np.asarray(U).reshape(-1, nf)
    dtu = np.asarray(dof_to_unknown)
    cols, res = {}, {}
    for bi, (et, conns) in enumerate(blocks):
        adj = adjacent_elements(conns, nodes)
        st = None if states is None else states[bi]
        for n, pairs in adj.items():
            for e, a in pairs:
                c = conns[e] - 1
                so = None
                if st is not None:
                    nq = orc.NQ[orc.ELEM[et]]
                    so = st[e * 7 * nq:(e + 1) * 7 * nq]
                Re, Ke, _ = orc.element(et, phys, props, X[c], U[c].ravel(), so)
                for k in range(nf):
                    col = dtu[nf * n + k] - 1
                    if col < 0:
                        continue
                    res[col] = res.get(col, 0.0) + Re[nf * a + k]
                    cc = cols.setdefault(col, {})
                    for b, m in enumerate(c):
                        for i in range(nf):
                            row = dtu[nf * m + i] - 1
                            if row >= 0:
                                cc[row] = cc.get(row, 0.0) + Ke[nf * a + k, nf * b + i]
    return cols, res


def compare_sampled_columns(K, nzval, R, cols, res):
    """GPU columns/residual entries (K a CSCMatrix on the host pattern, nzval and
    R device or host arrays) against sampled_columns(); returns (rel_err of the
    columns, rel_err of the residual entries) after checking the row structure."""
    got, exp = [], []
    nz = nzval
    for col in sorted(cols):
        s, t = int(K.colptr[col]) - 1, int(K.colptr[col + 1]) - 1
        rows = (K.rowval[s:t] - 1).tolist()
        assert rows == sorted(cols[col]), f"rows of column {col}"
        v = nz[s:t]
        got.append(v.cpu().numpy() if hasattr(v, "cpu") else np.asarray(v))
        exp.append(np.array([cols[col][r] for r in rows]))
    idx = np.array(sorted(res), dtype=np.int64)
    Rh = R.cpu().numpy() if hasattr(R, "cpu") else np.asarray(R)
    Rg = Rh[idx]
    Re = np.array([res[i] for i in idx])
    return rel_err(np.concatenate(got), np.concatenate(exp)), rel_err(Rg, Re)
