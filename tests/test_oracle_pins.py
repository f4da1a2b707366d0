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


# ---------------------------------------------------------------------------
# Shape functions, gradients and quadrature weights of every element type,
# pinned by identities that hold exactly (to rounding) on an affinely mapped
# element: partition of unity of the gradients (sum_a dN_a = 0), completeness
# (sum_a X_a (x) dN_a = I) and exact volume (sum_q JxW = V).  No reference test
# holds element-level data for these types, so these identities are their pins.
# ---------------------------------------------------------------------------
NEO_HOOKEAN = [0.8333333333333334, 0.38461538461538464]  # bulk, shear of E = 1, nu = 0.3
J2_PROPS = [200.0, 0.3, 0.25, 2.0]


def _affine_element(elem, rng):
    """Node coordinates of the first element of a small generated mesh of the type,
    mapped by a random affine map, and the element's volume (area for quad4)."""
    from fec_gb300 import meshes
    if elem == "HEX8":
        m = meshes.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (2, 2, 2))
    elif elem == "QUAD4":
        m = meshes.StructuredMesh("quad", (0.0, 0.0), (1.0, 1.0), (2, 2))
    elif elem == "TETRA4":
        m = meshes.box_tet4((2, 2, 2))
    elif elem == "TETRA10":
        m = meshes.box_tet10((2, 2, 2))
    else:
        m = meshes.box_hex27((2, 2, 2))
    b = m.element_block_names[0]
    x0 = m.nodal_coords[m.element_conns[b][0] - 1]
    D = x0.shape[1]
    if elem.startswith("TETRA"):  # straight-sided: the corner tet's volume
        c = x0[:4]
        v0 = abs(np.linalg.det((c[1:] - c[0]).T)) / 6.0
    else:  # axis-aligned box cell
        v0 = float(np.prod(x0.max(0) - x0.min(0)))
    A = np.eye(D) + 0.3 * rng.standard_normal((D, D))
    assert np.linalg.det(A) > 0.2
    return x0 @ A.T + rng.standard_normal(D), v0 * np.linalg.det(A)


@pytest.mark.parametrize("elem", ["QUAD4", "HEX8", "TETRA4", "TETRA10", "HEX27"])
def test_element_tables_by_linear_fields(orc, elem):
    """Poisson element (source amplitude 0, so R = K u) under a linear field u = c.X + c0:
    grad u = c at every point, so sum_a R_a = 0 and sum_a R_a X_a = V c; K is symmetric
    with zero row sums."""
    rng = np.random.default_rng(11)
    x, V = _affine_element(elem, rng)
    c = rng.standard_normal(x.shape[1])
    u = x @ c + 0.7
    R, K, _ = orc.element(elem, "poisson", [0.0], x, u)
    scale = np.abs(K).max() * np.abs(u).max()
    assert abs(R.sum()) <= 1e-14 * scale
    assert np.abs(R @ x - V * c).max() <= 1e-13 * V * np.abs(c).max()
    assert np.abs(K.sum(axis=1)).max() <= 1e-14 * np.abs(K).max()
    assert np.array_equal(K, K.T)
    assert np.abs(R - K @ u).max() <= 1e-13 * scale


@pytest.mark.parametrize("elem", ["HEX8", "TETRA4", "TETRA10", "HEX27"])
def test_mechanics_element_identities(orc, elem):
    """Mechanics elements (TestMechanicsCommon.jl:140-190):
    - homogeneous deformation u = H X: sum_a R_a = 0 and sum_a R_a (x) X_a = V P(I + H);
    - at u = 0 the tangent annihilates translations; for rotations W X it gives W R0_a,
      the objectivity of the Neo-Hookean energy of TestMechanicsLargeDeformation.jl:17-27,
      which is not stress-free at F = I (P(I) = -K/2 I from its -ln J term);
    - small-strain J2 at a zero state: the tangent annihilates all six rigid modes."""
    rng = np.random.default_rng(12)
    x, V = _affine_element(elem, rng)
    n = x.shape[0]
    H = 0.05 * rng.standard_normal((3, 3))
    R, _, _ = orc.element(elem, "neohookean", NEO_HOOKEAN, x, (x @ H.T).ravel())
    P, _ = orc.neohookean_PA(np.eye(3) + H, *NEO_HOOKEAN)
    P = P.reshape(3, 3, order="F")  # P[i + 3 J] = P_iJ
    Rn = R.reshape(n, 3)
    assert np.abs(Rn.sum(axis=0)).max() <= 1e-14 * V * np.abs(P).max() * n
    assert np.abs(Rn.T @ x - V * P).max() <= 1e-13 * V * np.abs(P).max()

    P0, _ = orc.neohookean_PA(np.eye(3), *NEO_HOOKEAN)
    assert np.allclose(P0.reshape(3, 3, order="F"), -0.5 * NEO_HOOKEAN[0] * np.eye(3), rtol=0, atol=1e-15)
    R0, K0, _ = orc.element(elem, "neohookean", NEO_HOOKEAN, x, np.zeros(3 * n))
    _, Kj, _ = orc.element(elem, "j2", J2_PROPS, x, np.zeros(3 * n))
    for d in range(3):
        t = np.zeros((n, 3))
        t[:, d] = 1.0
        assert np.abs(K0 @ t.ravel()).max() <= 1e-14 * np.abs(K0).max() * n
        assert np.abs(Kj @ t.ravel()).max() <= 1e-14 * np.abs(Kj).max() * n
    for w in rng.standard_normal((3, 3)):
        W = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
        r = (x @ W.T).ravel()
        scale = np.abs(K0).max() * np.abs(r).max() * n
        assert np.abs((K0 @ r).reshape(n, 3) - R0.reshape(n, 3) @ W.T).max() <= 1e-14 * scale
        assert np.abs(Kj @ r).max() <= 1e-14 * np.abs(Kj).max() * np.abs(r).max() * n


def test_j2_pure_shear_closed_form(orc):
    """J2 radial return (Simo & Hughes 1998, Box 3.2) against the closed form of pure
    shear gamma = du_x/dy from a virgin state: yield at sqrt(3) tau = sigma_y + H eqps with
    eqps = gamma_p / sqrt(3) gives gamma_p = (3 G gamma - sqrt(3) sigma_y) / (3 G + H),
    tau = G (gamma - gamma_p), tangent d tau/d gamma = G H / (3 G + H); the same state in
    three load steps (radial return is exact for monotonic proportional loading with
    linear hardening); elastic unloading with slope G and the state unchanged."""
    E, nu, sy, H = J2_PROPS
    G = E / (2 * (1 + nu))
    gamma = 0.01  # about 5x the shear yield strain
    gu = np.zeros((3, 3)); gu[0, 1] = gamma
    P, A, sn = orc.j2_update(gu, J2_PROPS, np.zeros(7))
    gp = (3 * G * gamma - np.sqrt(3) * sy) / (3 * G + H)
    tau = G * (gamma - gp)
    assert abs(P[3] - tau) <= 1e-14 * tau and abs(P[1] - tau) <= 1e-14 * tau  # sigma_xy = sigma_yx
    assert np.abs(P[[0, 2, 4, 5, 6, 7, 8]]).max() <= 1e-15 * tau
    assert abs(sn[6] - gp / np.sqrt(3)) <= 1e-14 * gp and abs(sn[5] - gp / 2) <= 1e-14 * gp
    assert abs(A[3 + 9 * 3] - G * H / (3 * G + H)) <= 1e-12 * G
    st = np.zeros(7)
    for k in (1, 2, 3):
        gu = np.zeros((3, 3)); gu[0, 1] = gamma * k / 3
        P3, _, st = orc.j2_update(gu, J2_PROPS, st)
    assert abs(P3[3] - P[3]) <= 1e-14 * tau and np.abs(st - sn).max() <= 1e-15
    gu = np.zeros((3, 3)); gu[0, 1] = gamma - 1e-3
    Pu, Au, su = orc.j2_update(gu, J2_PROPS, sn)
    assert abs(Pu[3] - (P[3] - G * 1e-3)) <= 1e-13 * tau
    assert np.array_equal(su, sn) and abs(Au[3 + 9 * 3] - G) <= 1e-13 * G


@pytest.mark.parametrize("elem", ["HEX8", "TETRA4", "TETRA10", "HEX27"])
def test_patch_test_on_assembled_mesh(orc, elem):
    """Patch test of the whole assembly (element loop, connectivity, local node orders of
    the generated meshes): under a linear field (Poisson, no source) and a homogeneous
    deformation (Neo-Hookean) the assembled residual vanishes at every interior node of
    the unit box, however the mesh is distorted by an affine map."""
    from fec_gb300 import meshes
    if elem == "HEX8":
        m = meshes.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (4, 4, 4))
    elif elem == "TETRA4":
        m = meshes.box_tet4((4, 4, 4))
    elif elem == "TETRA10":
        m = meshes.box_tet10((3, 3, 3))
    else:
        m = meshes.box_hex27((3, 3, 3))
    blocks = [(m.element_types[b], m.element_conns[b]) for b in m.element_block_names]
    X0 = m.nodal_coords
    interior = np.all((X0 > 1e-12) & (X0 < 1 - 1e-12), axis=1)
    assert interior.sum() >= 8
    rng = np.random.default_rng(21)
    A = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
    X = X0 @ A.T
    c = rng.standard_normal(3)
    R, _ = orc.assemble(blocks, X, "poisson", [0.0], X @ c + 0.3)
    scale = np.abs(c).max() * np.abs(X).max() ** 2
    assert np.abs(R[interior]).max() <= 1e-13 * scale
    assert np.abs(R[~interior]).max() > 1e-6 * scale  # the boundary carries the flux
    H = 0.05 * rng.standard_normal((3, 3))
    R, _ = orc.assemble(blocks, X, "neohookean", NEO_HOOKEAN, (X @ H.T).ravel())
    Rn = R.reshape(-1, 3)
    assert np.abs(Rn[interior]).max() <= 1e-13 * np.abs(Rn).max()
    assert np.abs(Rn[~interior]).max() > 1e-6
