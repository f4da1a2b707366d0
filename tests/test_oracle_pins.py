"""The oracle checked against the reference's own golden data and known answers."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

GOLD = Path(__file__).resolve().parent / "golden"


def test_structured_quad4_known_answer(orc):
    """test/TestMesh.jl: StructuredMesh("quad", (0,0), (1,1), (3,3)) coords and connectivity literal."""
    ka = json.loads((GOLD / "known_answers.json").read_text())["structured_quad4_3x3"]
    coords, conns = orc.structured_quad4((3, 3))
    assert np.array_equal(coords.T, np.array(ka["coords"]))
    assert np.array_equal(conns.T, np.array(ka["conns"]))


def test_structured_hex8_nodesets_on_faces(orc):
    """test/TestMesh.jl:77-86: each hex8 nodeset lies on its face."""
    counts = (3, 3, 3)
    coords, _ = orc.structured_hex8(counts)
    expect = dict(bottom=(1, 0.0), right=(0, 1.0), front=(2, 1.0), top=(1, 1.0), left=(0, 0.0), back=(2, 0.0))
    for face, (d, v) in expect.items():
        nodes = orc.hex8_nodeset(counts, face)
        assert nodes.size == 9
        assert np.allclose(coords[nodes - 1, d], v)


def test_update_dofs_matches_reference_rules(orc):
    """src/DofManagers.jl:227-298: unknowns = sorted complement; dof_to_unknown = rank or -1."""
    u, dtu = orc.update_dofs(10, [7, 2, 2, 9])
    assert u.tolist() == [1, 3, 4, 5, 6, 8, 10]
    assert dtu.tolist() == [1, -1, 2, 3, 4, 5, -1, 6, -1, 7]
    with pytest.raises(IndexError):
        orc.update_dofs(10, [11])


def test_sparse_semantics_against_scipy(orc):
    """sparse!(I, J, V, m, n, +): duplicates summed, rows sorted per column."""
    rng = np.random.default_rng(0)
    m = n = 40
    L = 2000
    I = rng.integers(1, m + 1, L); J = rng.integers(1, n + 1, L); V = rng.standard_normal(L)
    colptr, rowval, nzval = orc.sparse_csc(m, n, I, J, V)
    ref = sp.coo_matrix((V, (I - 1, J - 1)), shape=(m, n)).tocsc()
    ref.sum_duplicates(); ref.sort_indices()
    assert np.array_equal(colptr - 1, ref.indptr)
    assert np.array_equal(rowval - 1, ref.indices)
    assert np.allclose(nzval, ref.data, rtol=0, atol=1e-13)
    # summation order: duplicates of one entry are combined in input order
    I2 = np.array([1, 1, 1]); J2 = np.array([1, 1, 1]); V2 = np.array([1e16, 1.0, -1e16])
    _, _, nz = orc.sparse_csc(1, 1, I2, J2, V2)
    assert nz[0] == (1e16 + 1.0) - 1e16


def _poisson_gold_solve(orc, name):
    g = np.load(GOLD / name) if name == "poisson_quad4.npz" else None
    base = np.load(GOLD / "poisson_quad4.npz")
    coords, conn = base["coords"], base["conn"].astype(np.int64)
    bnd = np.unique(np.concatenate([base[f"nset_{i}"] for i in range(1, 5)])).astype(np.int64)
    nn = coords.shape[0]
    unknown, dtu = orc.update_dofs(nn, bnd)
    blocks = [("QUAD4", conn)]
    R, colptr, rowval, nzval = orc.assembled_system(blocks, coords, "poisson", [2 * np.pi ** 2], np.zeros(nn), dtu,
                                                    unknown)
    K = sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(unknown.size, unknown.size))
    u = np.zeros(nn)
    u[unknown - 1] = spl.spsolve(K, -R)
    gold = (g if g is not None else np.load(GOLD / name))["u_gold"]
    return u, gold


@pytest.mark.parametrize("name", ["poisson_quad4.npz", "laplace_quad4.npz"])
def test_oracle_reproduces_gold(orc, name):
    """test/poisson/TestPoisson.jl:54-100 (and the Laplace-with-source twin): one
    linear solve with the oracle's residual and CSC stiffness reproduces the gold."""
    u, gold = _poisson_gold_solve(orc, name)
    assert np.abs(u - gold).max() <= 1e-10 * np.abs(gold).max()


def _nh_energy(F, K, G):
    J = np.linalg.det(F)
    return 0.5 * K * (0.5 * (J - 1) ** 2 - np.log(J)) + 0.5 * G * (J ** (-2 / 3) * np.sum(F * F) - 3)


def test_neohookean_derivatives_by_finite_differences(orc):
    """Analytic P = dpsi/dF and A = d2psi/dF2 (TestMechanicsLargeDeformation.jl:17-27) vs central differences."""
    rng = np.random.default_rng(1)
    F = np.eye(3) + 0.1 * rng.standard_normal((3, 3))
    K, G = 0.8333, 0.3846
    P, A = orc.neohookean_PA(F, K, G)
    h = 1e-6
    for i in range(3):
        for j in range(3):
            dF = np.zeros((3, 3)); dF[i, j] = h
            fd = (_nh_energy(F + dF, K, G) - _nh_energy(F - dF, K, G)) / (2 * h)
            assert abs(fd - P[i + 3 * j]) < 1e-7
            Pp, _ = orc.neohookean_PA(F + dF, K, G)
            Pm, _ = orc.neohookean_PA(F - dF, K, G)
            col = (Pp - Pm) / (2 * h)
            assert np.abs(col - A[9 * (i + 3 * j):9 * (i + 3 * j) + 9]).max() < 1e-7


def test_j2_consistent_tangent_by_finite_differences(orc):
    """Radial-return consistent tangent vs differences of the returned stress (plastic step)."""
    props = [200.0, 0.3, 0.25, 2.0]
    st = np.zeros(7)
    gu = np.zeros((3, 3)); gu[0, 0] = 0.004; gu[1, 1] = -0.0012; gu[0, 1] = 0.0007
    P, A, sn = orc.j2_update(gu, props, st)
    assert sn[6] > 0  # yielded
    h = 1e-8
    for i in range(3):
        for j in range(3):
            d = np.zeros((3, 3)); d[i, j] = h
            Pp, _, _ = orc.j2_update(gu + d, props, st)
            Pm, _, _ = orc.j2_update(gu - d, props, st)
            assert np.abs((Pp - Pm) / (2 * h) - A[9 * (i + 3 * j):9 * (i + 3 * j) + 9]).max() < 1e-4 * np.abs(A).max()


def test_element_tangent_is_residual_jacobian(orc):
    """K_e = dR_e/du_e for the hex8 Neo-Hookean element (the mechanics stiffness of
    TestMechanicsCommon.jl:175-190 is the Jacobian of its residual)."""
    coords, conns = orc.structured_hex8((2, 2, 2))
    rng = np.random.default_rng(2)
    x = coords[conns[0] - 1]
    u = 0.02 * rng.standard_normal(24)
    R, K, _ = orc.element("HEX8", "neohookean", [0.8333, 0.3846], x, u)
    h = 1e-7
    for c in range(0, 24, 5):
        du = np.zeros(24); du[c] = h
        Rp, _, _ = orc.element("HEX8", "neohookean", [0.8333, 0.3846], x, u + du)
        Rm, _, _ = orc.element("HEX8", "neohookean", [0.8333, 0.3846], x, u - du)
        assert np.abs((Rp - Rm) / (2 * h) - K[:, c]).max() < 1e-6 * np.abs(K).max()
