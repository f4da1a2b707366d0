"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle (oracle/fec_oracle.cpp).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product never imports it.  Each function names the reference code
it restates; see the header of fec_oracle.cpp for the parity pins."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libfec_oracle.so"

PHYS = {"poisson": 1, "neohookean": 2, "j2": 3}
ELEM = {"HEX8": 1, "QUAD4": 2, "TETRA4": 6, "TETRA10": 7, "HEX27": 8}
NNPE = {1: 8, 2: 4, 6: 4, 7: 10, 8: 27}
NQ = {1: 8, 2: 4, 6: 1, 7: 4, 8: 27}

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "fec_oracle.cpp").stat().st_mtime:
            build()
        _lib = C.CDLL(str(LIB))
        vp, i64 = C.c_void_p, C.c_int64
        sig = {
            "orc_structured_hex8": (None, [i64, i64, i64, vp, vp, vp, vp]),
            "orc_structured_quad4": (None, [i64, i64, vp, vp, vp, vp]),
            "orc_hex8_nodeset": (i64, [i64, i64, i64, C.c_int, vp]),
            "orc_update_dofs": (i64, [i64, vp, i64, vp, vp]),
            "orc_pattern_count": (i64, [C.c_int, vp, vp, vp, C.c_int, vp]),
            "orc_pattern_fill": (None, [C.c_int, vp, vp, vp, C.c_int, vp, vp, vp, vp]),
            "orc_sparse_csc": (i64, [i64, i64, i64, vp, vp, vp, vp, vp, vp]),
            "orc_element": (C.c_int, [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp]),
            "orc_assemble": (C.c_int, [C.c_int, vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp, vp, i64, vp, vp,
                                       C.c_int]),
            "orc_num_qp": (C.c_int, [C.c_int]),
            "orc_neohookean_PA": (None, [vp, C.c_double, C.c_double, vp, vp]),
            "orc_j2_update": (None, [vp, vp, vp, vp, vp, vp]),
            "orc_max_threads": (C.c_int, []),
            "orc_set_reference": (C.c_int, [C.c_int, C.c_int, vp, vp, vp]),
            "orc_clear_reference": (None, [C.c_int]),
            "orc_set_abs_output": (None, [vp]),
        }
        for k, (r, a) in sig.items():
            f = getattr(_lib, k)
            f.restype = r
            f.argtypes = a
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def structured_hex8(counts, mins=(0.0, 0.0, 0.0), maxs=(1.0, 1.0, 1.0)):
    """StructuredMesh("hex", ...) (src/meshes/StructuredMesh.jl:85-131): coords (NN,3), conns (NE,8) 1-based."""
    Nx, Ny, Nz = counts
    nn, ne = Nx * Ny * Nz, (Nx - 1) * (Ny - 1) * (Nz - 1)
    coords = np.empty((nn, 3)); conns = np.empty((ne, 8), dtype=np.int64)
    lo, hi = np.array(mins, float), np.array(maxs, float)
    lib().orc_structured_hex8(Nx, Ny, Nz, _p(lo), _p(hi), _p(coords), _p(conns))
    return coords, conns


def structured_quad4(counts, mins=(0.0, 0.0), maxs=(1.0, 1.0)):
    Nx, Ny = counts
    coords = np.empty((Nx * Ny, 2)); conns = np.empty(((Nx - 1) * (Ny - 1), 4), dtype=np.int64)
    lo, hi = np.array(mins, float), np.array(maxs, float)
    lib().orc_structured_quad4(Nx, Ny, _p(lo), _p(hi), _p(coords), _p(conns))
    return coords, conns


HEX8_FACES = ["bottom", "right", "front", "top", "left", "back"]


def hex8_nodeset(counts, face: str) -> np.ndarray:
    Nx, Ny, Nz = counts
    out = np.empty(max(Nx, Ny, Nz) ** 2, dtype=np.int64)
    n = lib().orc_hex8_nodeset(Nx, Ny, Nz, HEX8_FACES.index(face), _p(out))
    return out[:n].copy()


def update_dofs(ndofs: int, dirichlet) -> tuple[np.ndarray, np.ndarray]:
    """DofManager update_dofs! (src/DofManagers.jl:227-298): (unknown_dofs, dof_to_unknown)."""
    d = np.ascontiguousarray(dirichlet, dtype=np.int64)
    u = np.empty(ndofs, dtype=np.int64); dtu = np.empty(ndofs, dtype=np.int64)
    n = lib().orc_update_dofs(ndofs, _p(d), d.size, _p(u), _p(dtu))
    if n < 0:
        raise IndexError("dirichlet dof out of range")
    return u[:n].copy(), dtu


def pattern(blocks, nd: int, dof_to_unknown):
    """_update_dofs!(pattern, ...) (SparsityPatterns.jl:160-231): element-ordered (Is, Js, slots)."""
    types = [ELEM[t] for t, _ in blocks]
    nnpe = np.array([NNPE[t] for t in types], dtype=np.int64)
    ne = np.array([c.shape[0] for _, c in blocks], dtype=np.int64)
    conn = np.ascontiguousarray(np.concatenate([c.ravel() for _, c in blocks]), dtype=np.int64)
    dtu = np.ascontiguousarray(dof_to_unknown, dtype=np.int64)
    n = lib().orc_pattern_count(len(blocks), _p(nnpe), _p(ne), _p(conn), nd, _p(dtu))
    Is = np.empty(n, dtype=np.int64); Js = np.empty(n, dtype=np.int64); slots = np.empty(n, dtype=np.int64)
    lib().orc_pattern_fill(len(blocks), _p(nnpe), _p(ne), _p(conn), nd, _p(dtu), _p(Is), _p(Js), _p(slots))
    return Is, Js, slots


def sparse_csc(m: int, n: int, Is, Js, V):
    """SparseArrays.sparse!(I, J, V, m, n, +) (SparsityPatterns.jl:301-308): 1-based (colptr, rowval, nzval)."""
    L = Is.size
    colptr = np.empty(n + 1, dtype=np.int64); rowval = np.empty(L, dtype=np.int64); nzval = np.empty(L)
    V = np.ascontiguousarray(V, dtype=np.float64)
    Is = np.ascontiguousarray(Is, dtype=np.int64); Js = np.ascontiguousarray(Js, dtype=np.int64)
    nnz = lib().orc_sparse_csc(m, n, L, _p(Is), _p(Js), _p(V), _p(colptr), _p(rowval), _p(nzval))
    return colptr, rowval[:nnz].copy(), nzval[:nnz].copy()


def element(elem: str, phys: str, props, xel, uel, st_old=None, want_state=False):
    """One element's (R_e, K_e, state_new): Assemblers.jl:418-431 for one element.
    K_e is returned as a (NDOF, NDOF) array with K_e[r, c] = dR_r/du_c."""
    et = ELEM[elem]
    nf = 1 if phys == "poisson" else 3
    ndof = nf * NNPE[et]
    nq = NQ[et]
    props = np.ascontiguousarray(props, dtype=np.float64)
    xel = np.ascontiguousarray(xel, dtype=np.float64); uel = np.ascontiguousarray(uel, dtype=np.float64)
    so = np.zeros(7 * nq) if st_old is None else np.ascontiguousarray(st_old, dtype=np.float64)
    sn = np.zeros(7 * nq) if want_state else None
    Re = np.empty(ndof); Ke = np.empty(ndof * ndof)
    rc = lib().orc_element(et, PHYS[phys], _p(props), _p(xel), _p(uel), _p(so), _p(sn), _p(Re), _p(Ke))
    if rc:
        raise RuntimeError(f"orc_element failed ({rc})")
    return Re, Ke.reshape(ndof, ndof, order="F"), sn


def assemble(blocks, coords, phys: str, props, U, st_old=None, st_new=None, *, want_r=True, want_k=True,
             threads: int = 1, abs_out=None):
    """The block loop of assemble_vector!/assemble_matrix! (Assemblers.jl:402-432).
    Returns (R_full, Kstore) with Kstore in the reference's element slot order
    (K_el.data, column-major per element).  abs_out (NF * NN doubles), if given,
    receives per dof the summed magnitudes of the terms its residual entry is
    formed from (sum over elements and points of JxW |grad N_a| |P| for
    mechanics), the scale that bounds the rounding of the entry."""
    types = np.array([ELEM[t] for t, _ in blocks], dtype=np.int32)
    ne = np.array([c.shape[0] for _, c in blocks], dtype=np.int64)
    conn = np.ascontiguousarray(np.concatenate([c.ravel() for _, c in blocks]), dtype=np.int64)
    nf = 1 if phys == "poisson" else 3
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    nn, dim = coords.shape
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.empty(nf * nn) if want_r else None
    nk = int(sum(n * (nf * NNPE[t]) ** 2 for t, n in zip(types, ne)))
    K = np.empty(nk) if want_k else None
    props = np.ascontiguousarray(props, dtype=np.float64)
    if abs_out is not None:
        assert abs_out.dtype == np.float64 and abs_out.size == nf * nn and abs_out.flags.c_contiguous
    lib().orc_set_abs_output(_p(abs_out))
    try:
        rc = lib().orc_assemble(len(blocks), _p(types), _p(ne), _p(conn), dim, _p(coords), PHYS[phys], _p(props),
                                _p(U), _p(st_old), _p(st_new), nn, _p(R), _p(K), threads)
    finally:
        lib().orc_set_abs_output(None)
    if rc:
        raise RuntimeError(f"orc_assemble failed ({rc})")
    return R, K


def assembled_system(blocks, coords, phys, props, U, dof_to_unknown, unknown_dofs, st_old=None, st_new=None,
                     threads: int = 1):
    """residual(asm) and stiffness(asm) the reference way: element loop ->
    COO slot storage -> sparse! over unknowns.  Returns (R_u, colptr, rowval, nzval)."""
    nf = 1 if phys == "poisson" else 3
    R, K = assemble(blocks, coords, phys, props, U, st_old, st_new, threads=threads)
    Is, Js, slots = pattern(blocks, nf, dof_to_unknown)
    n = unknown_dofs.size
    colptr, rowval, nzval = sparse_csc(n, n, Is, Js, K[slots - 1])
    return R[unknown_dofs - 1], colptr, rowval, nzval


def neohookean_PA(F, K, G):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(3, 3)
    P = np.empty(9); A = np.empty(81)
    lib().orc_neohookean_PA(_p(F), K, G, _p(P), _p(A))
    return P, A


def j2_update(gradu, props, st_old):
    g = np.ascontiguousarray(gradu, dtype=np.float64).reshape(3, 3)
    so = np.ascontiguousarray(st_old, dtype=np.float64)
    sn = np.empty(7); P = np.empty(9); A = np.empty(81)
    pr = np.ascontiguousarray(props, dtype=np.float64)
    lib().orc_j2_update(_p(g), _p(pr), _p(so), _p(sn), _p(P), _p(A))
    return P, A, sn


class reference_tables:
    """with reference_tables("HEX8", N, dN, w): the oracle integrates that element
    type with the caller's tables (a ReferenceFE built with another quadrature
    rule, src/FunctionSpaces.jl:104-126) inside the block."""

    def __init__(self, elem: str, N, dN, w):
        self.et = ELEM[elem]
        self.N = np.ascontiguousarray(N, dtype=np.float64)
        self.dN = np.ascontiguousarray(dN, dtype=np.float64)
        self.w = np.ascontiguousarray(w, dtype=np.float64)

    def __enter__(self):
        if lib().orc_set_reference(self.et, int(self.w.size), _p(self.N), _p(self.dN), _p(self.w)):
            raise ValueError("orc_set_reference rejected the tables")
        NQ[self.et] = int(self.w.size)
        return self

    def __exit__(self, *exc):
        lib().orc_clear_reference(self.et)
        NQ[self.et] = {1: 8, 2: 4, 6: 1, 7: 4, 8: 27}[self.et]
        return False


def max_threads() -> int:
    return int(lib().orc_max_threads())
