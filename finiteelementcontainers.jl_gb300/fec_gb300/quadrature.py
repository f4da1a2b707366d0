"""Reference-element tables: quadrature rule, shape-function values and their
reference-coordinate gradients at the points -- what ReferenceFiniteElements.jl's
ReferenceFE(elem{Lagrange, p}(), q_type(q_degree)) holds for the element types
on the assembly path (built per block in src/FunctionSpaces.jl:104-126 and read
by the physics through _cell_interpolants, src/assemblers/Assemblers.jl:129-131).

The tables go to the library with fec_block_reference_set, so the kernels
integrate with the rule the caller chose.  The reference's default q_type is
GaussLobattoLegendre (src/FunctionSpaces.jl:187) with q_degree 2
(src/FunctionSpaces.jl:15-29); here q_degree is the number of points per
direction of the tensor rules.  The workloads of this project use the
Gauss-Legendre rule (the default of FunctionSpace below).

Layouts (row-major, as the C ABI takes them):
  N  [nq][nnpe]       dN [nq][nnpe][dim]       w [nq]
Point order of the tensor rules: x fastest, then y, then z.  Node orders: the
Exodus orders of QUAD4/HEX8/TETRA4/TETRA10 and, for HEX27, i + 3j + 9k over the
1D nodes (-1, 0, 1)."""
from __future__ import annotations

import math

import numpy as np

RULES = ("GaussLegendre", "GaussLobattoLegendre")

# built point counts of the library's kernels per element type
KERNEL_NQ = {"HEX8": 8, "QUAD4": 4, "TETRA4": 1, "TETRA10": 4, "HEX27": 27}

_HEX8_NODES = ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1))
_QUAD4_NODES = ((-1, -1), (1, -1), (1, 1), (-1, 1))


def gauss_legendre_1d(n: int) -> tuple[np.ndarray, np.ndarray]:
    """n-point Gauss-Legendre rule on [-1, 1]; the 2- and 3-point rules in closed form."""
    if n == 1:
        return np.array([0.0]), np.array([2.0])
    if n == 2:
        g = 1.0 / math.sqrt(3.0)
        return np.array([-g, g]), np.array([1.0, 1.0])
    if n == 3:
        p = math.sqrt(0.6)
        return np.array([-p, 0.0, p]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


def gauss_lobatto_1d(n: int) -> tuple[np.ndarray, np.ndarray]:
    """n-point Gauss-Lobatto-Legendre rule on [-1, 1] (end points included):
    interior points are the roots of P'_{n-1}, weights 2 / (n (n-1) P_{n-1}(x)^2)."""
    if n < 2:
        raise ValueError("a Lobatto rule has at least 2 points")
    if n == 2:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    if n == 3:
        return np.array([-1.0, 0.0, 1.0]), np.array([1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0])
    P = np.polynomial.legendre.Legendre.basis(n - 1)
    inner = np.sort(P.deriv().roots().real)
    x = np.concatenate([[-1.0], inner, [1.0]])
    w = 2.0 / (n * (n - 1) * P(x) ** 2)
    return x, w


def _rule_1d(q_type: str, n: int):
    if q_type == "GaussLegendre":
        return gauss_legendre_1d(n)
    if q_type == "GaussLobattoLegendre":
        return gauss_lobatto_1d(n)
    raise ValueError(f"q_type must be one of {RULES}")


def _quad4(xs, ws):
    n = xs.size
    nq = n * n
    N = np.empty((nq, 4)); dN = np.empty((nq, 4, 2)); w = np.empty(nq)
    for q in range(nq):
        qx, qy = q % n, q // n
        s, t = xs[qx], xs[qy]
        w[q] = ws[qx] * ws[qy]
        for a, (xa, ya) in enumerate(_QUAD4_NODES):
            N[q, a] = 0.25 * (1 + xa * s) * (1 + ya * t)
            dN[q, a, 0] = 0.25 * xa * (1 + ya * t)
            dN[q, a, 1] = 0.25 * ya * (1 + xa * s)
    return N, dN, w


def _hex8(xs, ws):
    n = xs.size
    nq = n ** 3
    N = np.empty((nq, 8)); dN = np.empty((nq, 8, 3)); w = np.empty(nq)
    for q in range(nq):
        qx, qy, qz = q % n, (q // n) % n, q // (n * n)
        s, t, u = xs[qx], xs[qy], xs[qz]
        w[q] = ws[qx] * ws[qy] * ws[qz]
        for a, (xa, ya, za) in enumerate(_HEX8_NODES):
            fs, ft, fu = 1 + xa * s, 1 + ya * t, 1 + za * u
            N[q, a] = 0.125 * fs * ft * fu
            dN[q, a, 0] = 0.125 * xa * ft * fu
            dN[q, a, 1] = 0.125 * ya * fs * fu
            dN[q, a, 2] = 0.125 * za * fs * ft
    return N, dN, w


def _lag2(x):
    """1D quadratic Lagrange basis on nodes -1, 0, 1 and its derivative."""
    return (np.array([0.5 * x * (x - 1.0), 1.0 - x * x, 0.5 * x * (x + 1.0)]),
            np.array([x - 0.5, -2.0 * x, x + 0.5]))


def _hex27(xs, ws):
    n = xs.size
    nq = n ** 3
    N = np.empty((nq, 27)); dN = np.empty((nq, 27, 3)); w = np.empty(nq)
    for q in range(nq):
        qx, qy, qz = q % n, (q // n) % n, q // (n * n)
        w[q] = ws[qx] * ws[qy] * ws[qz]
        vx, dx = _lag2(xs[qx]); vy, dy = _lag2(xs[qy]); vz, dz = _lag2(xs[qz])
        for a in range(27):
            i, j, k = a % 3, (a // 3) % 3, a // 9
            N[q, a] = vx[i] * vy[j] * vz[k]
            dN[q, a, 0] = dx[i] * vy[j] * vz[k]
            dN[q, a, 1] = vx[i] * dy[j] * vz[k]
            dN[q, a, 2] = vx[i] * vy[j] * dz[k]
    return N, dN, w


_TET_DL = ((-1.0, -1.0, -1.0), (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))
_TET10_EDGES = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))


def tet_points_rule(nq: int) -> tuple[np.ndarray, np.ndarray]:
    """Barycentric-free tet rules on the unit tetrahedron: 1 point (centroid,
    exact for degree 1) or 4 points (exact for degree 2)."""
    if nq == 1:
        return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
    if nq == 4:
        al = (5.0 + 3.0 * math.sqrt(5.0)) / 20.0
        be = (5.0 - math.sqrt(5.0)) / 20.0
        return (np.array([[be, be, be], [al, be, be], [be, al, be], [be, be, al]]),
                np.full(4, 1.0 / 24.0))
    raise ValueError("tet rules here have 1 or 4 points")


def tet_tables(nnpe: int, pts: np.ndarray, ws: np.ndarray):
    """P1 (4 nodes) or P2 (10 nodes, Exodus TETRA10 order) tables at the given
    points of the unit tetrahedron."""
    nq = pts.shape[0]
    N = np.empty((nq, nnpe)); dN = np.empty((nq, nnpe, 3))
    for q in range(nq):
        lam = (1.0 - pts[q, 0] - pts[q, 1] - pts[q, 2], pts[q, 0], pts[q, 1], pts[q, 2])
        if nnpe == 4:
            for a in range(4):
                N[q, a] = lam[a]
                dN[q, a] = _TET_DL[a]
        else:
            for v in range(4):
                N[q, v] = lam[v] * (2 * lam[v] - 1)
                for k in range(3):
                    dN[q, v, k] = (4 * lam[v] - 1) * _TET_DL[v][k]
            for e, (i, j) in enumerate(_TET10_EDGES):
                N[q, 4 + e] = 4 * lam[i] * lam[j]
                for k in range(3):
                    dN[q, 4 + e, k] = 4 * (_TET_DL[i][k] * lam[j] + lam[i] * _TET_DL[j][k])
    return N, dN, np.asarray(ws, dtype=np.float64).copy()


def reference_tables(elem_type: str, q_type: str = "GaussLegendre", q_degree: int | None = None):
    """(N, dN, w) of ReferenceFE(elem_type, q_type(q_degree)).

    Tensor elements: q_degree points per direction (default 2 for QUAD4/HEX8, 3
    for HEX27).  Tets: the Gauss rules the kernels are built for (1 point for
    TETRA4, 4 for TETRA10); a Lobatto rule is not defined for them here."""
    et = elem_type.upper()
    if q_type not in RULES:
        raise ValueError(f"q_type must be one of {RULES}")
    if et in ("QUAD4", "HEX8", "HEX27"):
        n = q_degree if q_degree is not None else (3 if et == "HEX27" else 2)
        xs, ws = _rule_1d(q_type, n)
        return {"QUAD4": _quad4, "HEX8": _hex8, "HEX27": _hex27}[et](xs, ws)
    if et in ("TETRA4", "TETRA10"):
        if q_type != "GaussLegendre":
            raise NotImplementedError(f"{q_type} is not defined for {et} here; pass tables directly")
        pts, ws = tet_points_rule(KERNEL_NQ[et])
        return tet_tables(4 if et == "TETRA4" else 10, pts, ws)
    raise ValueError(f"unknown element type {elem_type}")
