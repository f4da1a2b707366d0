"""The 128^3 Neo-Hookean workload at full size (2,097,152 hex8 elements,
6,440,067 dofs, 513,599,625 CSC entries), checked through properties that do
not need a full-size oracle run:

  * entry count and the structure of sampled columns;
  * sampled CSC columns and residual entries against the oracle's element
    matrices of the adjacent elements, summed in element order (<= 1e-12);
  * exact symmetry of sampled entries;
  * translation invariance: K t = 0 for a rigid translation t;
  * bitwise determinism of two calls;
  * the FP32-element variant against the FP64 result (<= 1e-5 relative)."""
import numpy as np
import pytest

from helpers import rel_err, stretch_field

pytestmark = pytest.mark.gpu
N = 128


@pytest.fixture(scope="module")
def full(fec):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (N + 1,) * 3)
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    p = fec.create_parameters(mesh, asm, phys)
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    return dict(mesh=mesh, asm=asm, p=p, U=U, Uu=Uu, R=R.clone(), nz=K.nzval.clone(), K=K, phys=phys)


def test_pattern_size(full):
    K = full["K"]
    assert K.nnz == 513_599_625
    assert K.shape == (6_440_067, 6_440_067)
    # an interior node couples to 27 nodes x 3 components
    n = (N // 2) + (N + 1) * (N // 2) + (N + 1) ** 2 * (N // 2)   # 0-based interior node
    col = 3 * n
    assert K.colptr[col + 1] - K.colptr[col] == 81


def _adjacent(conns, nodes):
    """(element, local index) pairs of each node, elements ascending."""
    out = {int(n): [] for n in nodes}
    hit = np.isin(conns, nodes + 1)
    for e, a in zip(*np.nonzero(hit)):
        out[int(conns[e, a]) - 1].append((int(e), int(a)))
    return out


def test_sampled_columns_and_residual_against_oracle(full, orc):
    mesh, K = full["mesh"], full["K"]
    conns = mesh.element_conns["block_1"]
    X = mesh.nodal_coords
    U = full["U"].reshape(-1, 3)
    rng = np.random.default_rng(7)
    nodes = np.unique(np.concatenate([rng.integers(0, mesh.num_nodes, 40), [0, mesh.num_nodes - 1]]))
    adj = _adjacent(conns, nodes)
    props = full["phys"].create_properties()
    cache = {}
    R = full["R"].cpu().numpy()
    got_all, exp_all, R_got, R_exp = [], [], [], []
    for n in nodes:
        cols = {}
        rres = np.zeros(3)
        for e, a in adj[int(n)]:
            if e not in cache:
                c = conns[e] - 1
                cache[e] = orc.element("HEX8", "neohookean", props, X[c], U[c].ravel())
            Re, Ke, _ = cache[e]
            rres += Re[3 * a:3 * a + 3]
            for b, m in enumerate(conns[e] - 1):
                for k in range(3):
                    for i in range(3):
                        key = (k, 3 * m + i)
                        cols[key] = cols.get(key, 0.0) + Ke[3 * a + k, 3 * b + i]
        for k in range(3):
            col = 3 * n + k
            s, t = K.colptr[col] - 1, K.colptr[col + 1] - 1
            rows = K.rowval[s:t] - 1
            expect_rows = sorted(r for (kk, r) in cols if kk == k)
            assert rows.tolist() == expect_rows
            got = full["nz"][s:t].cpu().numpy()
            exp = np.array([cols[(k, r)] for r in rows])
            got_all.append(got)
            exp_all.append(exp)
        R_got.append(R[3 * n:3 * n + 3])
        R_exp.append(rres)
    # entry-wise: every sampled entry within 1e-12 of its own size (absolute
    # floor 1e-14 of the largest sampled entry), and normwise
    e_k = rel_err(np.concatenate(got_all), np.concatenate(exp_all))
    e_r = rel_err(np.concatenate(R_got), np.concatenate(R_exp))
    print("128^3 sampled columns:", e_k, "sampled residual entries:", e_r)
    assert max(e_k) <= 1e-12, e_k
    assert max(e_r) <= 1e-12, e_r


def test_symmetry_of_sampled_entries(full):
    K = full["K"]
    rng = np.random.default_rng(3)
    cols = rng.integers(0, K.shape[0], 2000)
    nz = full["nz"]
    for c in cols:
        s, t = K.colptr[c] - 1, K.colptr[c + 1] - 1
        j = rng.integers(s, t)
        r = K.rowval[j] - 1
        s2, t2 = K.colptr[r] - 1, K.colptr[r + 1] - 1
        k = s2 + np.searchsorted(K.rowval[s2:t2] - 1, c)
        assert K.rowval[k] - 1 == c
        a, b = float(nz[j]), float(nz[k])
        assert a == b or abs(a - b) <= 1e-12 * max(abs(a), abs(b))


def test_translation_invariance(full):
    import torch
    K = full["K"]
    nz = full["nz"]
    colptr = torch.from_numpy(K.colptr - 1).cuda()
    rowval = torch.from_numpy(K.rowval - 1).cuda()
    counts = colptr[1:] - colptr[:-1]
    colidx = torch.repeat_interleave(torch.arange(K.shape[0], device="cuda"), counts)
    for comp in range(3):
        t = (torch.arange(K.shape[0], device="cuda") % 3 == comp).double()
        Kt = torch.zeros(K.shape[0], dtype=torch.float64, device="cuda")
        Kt.index_add_(0, rowval, nz * t[colidx])
        absrow = torch.zeros_like(Kt).index_add_(0, rowval, nz.abs())
        assert float((Kt.abs() / absrow.max()).max()) <= 1e-12
    del colidx


def test_determinism_and_fp32_variant(full, fec):
    import torch
    asm, p, Uu = full["asm"], full["p"], full["Uu"]
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    assert torch.equal(R, full["R"]) and torch.equal(K.nzval, full["nz"])
    R32, K32 = fec.assemble_residual_and_stiffness(asm, Uu, p, precision="fp32_element")
    torch.cuda.synchronize()
    ek = float((K32.nzval - full["nz"]).norm() / full["nz"].norm())
    er = float((R32 - full["R"]).norm() / full["R"].norm())
    print(f"fp32-element vs fp64 at 128^3: stiffness {ek:.3e}, residual {er:.3e}")
    assert ek <= 1e-5 and er <= 1e-5
