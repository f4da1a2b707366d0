"""Caller-supplied quadrature and shape-function tables (fec_block_reference_set),
host side: the tables' own identities, the library's built-in tables equal to
the Gauss-Legendre tables of the host mirror bit for bit, the ABI's checks on a
host-only context, and the oracle integrating with caller tables (checked
against a numpy restatement of the element integral on the same tables)."""
import ctypes as C

import numpy as np
import pytest

ELEMS = ["HEX8", "QUAD4", "TETRA4", "TETRA10", "HEX27"]
DIM = {"HEX8": 3, "QUAD4": 2, "TETRA4": 3, "TETRA10": 3, "HEX27": 3}


@pytest.mark.parametrize("rule", ["GaussLegendre", "GaussLobattoLegendre"])
@pytest.mark.parametrize("elem", ["HEX8", "QUAD4", "HEX27"])
def test_tensor_tables_identities(fec, elem, rule):
    from fec_gb300.quadrature import reference_tables
    N, dN, w = reference_tables(elem, rule)
    d = DIM[elem]
    assert np.allclose(N.sum(axis=1), 1.0, atol=1e-15)          # partition of unity
    assert np.allclose(dN.sum(axis=1), 0.0, atol=1e-14)         # gradients of a constant
    assert abs(w.sum() - 2.0 ** d) <= 1e-14                      # reference volume
    if rule == "GaussLobattoLegendre" and elem in ("HEX8", "QUAD4"):
        # the points are the nodes: N is a permutation matrix
        assert np.array_equal(np.sort(N, axis=1)[:, -1], np.ones(N.shape[0]))
        assert sorted(np.argmax(N, axis=1).tolist()) == list(range(N.shape[1]))


def test_one_dimensional_rules(fec):
    from fec_gb300.quadrature import gauss_legendre_1d, gauss_lobatto_1d
    for n in range(2, 7):
        x, w = gauss_legendre_1d(n)
        for k in range(2 * n):                   # exact up to degree 2n-1
            assert abs((w * x ** k).sum() - (2.0 / (k + 1) if k % 2 == 0 else 0.0)) <= 1e-14
        x, w = gauss_lobatto_1d(n)
        assert x[0] == -1.0 and x[-1] == 1.0
        for k in range(2 * n - 2):               # exact up to degree 2n-3
            assert abs((w * x ** k).sum() - (2.0 / (k + 1) if k % 2 == 0 else 0.0)) <= 1e-13
    x, w = gauss_lobatto_1d(2)
    assert abs((w * x ** 2).sum() - 2.0 / 3.0) > 1.0             # not exact at degree 2: a different rule


def _host_ctx(fec, elem, coords, conn):
    lib = fec.load_library()
    from fec_gb300 import _lib
    h = C.c_void_p()
    assert lib.fec_ctx_create(-1, C.byref(h)) == 0
    types = np.array([fec.meshes.ELEMENT_IDS[elem]], dtype=np.int32)
    ne = np.array([conn.shape[0]], dtype=np.int64)
    c = np.ascontiguousarray(conn, dtype=np.int64)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    assert lib.fec_mesh_set(h, X.shape[1], X.shape[0], _lib.ptr(X), 1, _lib.ptr(types), _lib.ptr(ne),
                            _lib.ptr(c)) == 0
    return lib, h


@pytest.mark.parametrize("elem", ELEMS)
def test_builtin_tables_equal_host_gauss_tables_bitwise(fec, elem):
    """Without fec_block_reference_set a block integrates with the library's own
    tables; they are bit for bit the host mirror's Gauss-Legendre tables, so the
    assembler (which always hands its tables over) changes no result."""
    from fec_gb300.quadrature import reference_tables
    from fec_gb300 import _lib
    nnpe = fec.meshes.NNPE[elem]
    d = DIM[elem]
    coords = np.random.default_rng(0).random((nnpe, d))
    conn = np.arange(1, nnpe + 1, dtype=np.int64)[None, :]
    lib, h = _host_ctx(fec, elem, coords, conn)
    try:
        nq = C.c_int()
        assert lib.fec_block_reference_get(h, 1, C.byref(nq), None, None, None) == 0
        N = np.empty((nq.value, nnpe)); dN = np.empty((nq.value, nnpe, d)); w = np.empty(nq.value)
        assert lib.fec_block_reference_get(h, 1, C.byref(nq), _lib.ptr(N), _lib.ptr(dN), _lib.ptr(w)) == 0
        Nh, dNh, wh = reference_tables(elem, "GaussLegendre")
        assert np.array_equal(N, Nh) and np.array_equal(dN, dNh) and np.array_equal(w, wh)
    finally:
        lib.fec_ctx_destroy(h)


def test_reference_set_checks_and_round_trip(fec):
    from fec_gb300.quadrature import reference_tables
    from fec_gb300 import _lib
    coords = np.random.default_rng(1).random((8, 3))
    lib, h = _host_ctx(fec, "HEX8", coords, np.arange(1, 9, dtype=np.int64)[None, :])
    try:
        N, dN, w = (np.ascontiguousarray(a) for a in reference_tables("HEX8", "GaussLobattoLegendre"))
        assert lib.fec_block_reference_set(h, 1, 8, _lib.ptr(N), _lib.ptr(dN), _lib.ptr(w)) == 0
        N2 = np.empty_like(N); dN2 = np.empty_like(dN); w2 = np.empty_like(w)
        nq = C.c_int()
        assert lib.fec_block_reference_get(h, 1, C.byref(nq), _lib.ptr(N2), _lib.ptr(dN2), _lib.ptr(w2)) == 0
        assert nq.value == 8 and np.array_equal(N, N2) and np.array_equal(dN, dN2) and np.array_equal(w, w2)
        # a rule with another point count than the kernels are built for
        N3, dN3, w3 = (np.ascontiguousarray(a) for a in reference_tables("HEX8", "GaussLegendre", 3))
        assert lib.fec_block_reference_set(h, 1, 27, _lib.ptr(N3), _lib.ptr(dN3), _lib.ptr(w3)) == \
            _lib.FEC_ERR_UNSUPPORTED
        assert "8 quadrature points" in _lib.last_error(lib, h)
        assert lib.fec_block_reference_set(h, 2, 8, _lib.ptr(N), _lib.ptr(dN), _lib.ptr(w)) == _lib.FEC_ERR_ARG
        assert lib.fec_block_reference_set(h, 1, 8, None, _lib.ptr(dN), _lib.ptr(w)) == _lib.FEC_ERR_ARG
        bad = w.copy(); bad[3] = np.nan
        assert lib.fec_block_reference_set(h, 1, 8, _lib.ptr(N), _lib.ptr(dN), _lib.ptr(bad)) == _lib.FEC_ERR_ARG
        # the rejected calls left the tables as they were
        assert lib.fec_block_reference_get(h, 1, C.byref(nq), _lib.ptr(N2), _lib.ptr(dN2), _lib.ptr(w2)) == 0
        assert np.array_equal(w, w2)
    finally:
        lib.fec_ctx_destroy(h)


def _numpy_element(N, dN, w, X, u):
    """Poisson element (no source) integrated with the given tables:
    K_ab = sum_q w_q det J_q grad N_a . grad N_b, R = K u."""
    A = N.shape[1]
    K = np.zeros((A, A))
    for q in range(w.size):
        J = X.T @ dN[q]                  # J[d, k] = sum_a X_ad dN_ak
        G = dN[q] @ np.linalg.inv(J)     # spatial gradients
        K += w[q] * np.linalg.det(J) * G @ G.T
    return K @ u, K


@pytest.mark.parametrize("elem,rule", [("HEX8", "GaussLobattoLegendre"), ("HEX8", "GaussLegendre"),
                                       ("HEX27", "GaussLobattoLegendre"), ("QUAD4", "GaussLobattoLegendre")])
def test_oracle_integrates_with_caller_tables(fec, orc, elem, rule):
    from fec_gb300.quadrature import reference_tables
    N, dN, w = reference_tables(elem, rule)
    A, d = N.shape[1], DIM[elem]
    rng = np.random.default_rng(5)
    # a distorted element: reference nodes mapped affinely plus a perturbation
    if elem == "HEX27":
        ref = np.array([[x, y, z] for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1)], float)
    elif elem == "HEX8":
        ref = np.array(fec.quadrature._HEX8_NODES, float)
    else:
        ref = np.array(fec.quadrature._QUAD4_NODES, float)
    X = ref @ (np.eye(d) + 0.1 * rng.standard_normal((d, d))) + 0.05 * rng.standard_normal((A, d))
    u = rng.standard_normal(A)
    R_np, K_np = _numpy_element(N, dN, w, X, u)
    with orc.reference_tables(elem, N, dN, w):
        R_o, K_o, _ = orc.element(elem, "poisson", [0.0], X, u)
    assert np.abs(K_o - K_np).max() <= 1e-13 * np.abs(K_np).max()
    assert np.abs(R_o - R_np).max() <= 1e-13 * np.abs(R_np).max()
    # and the default tables are back afterwards
    R_d, K_d, _ = orc.element(elem, "poisson", [0.0], X, u)
    Ng, dNg, wg = reference_tables(elem, "GaussLegendre")
    _, K_g = _numpy_element(Ng, dNg, wg, X, u)
    assert np.abs(K_d - K_g).max() <= 1e-13 * np.abs(K_g).max()
