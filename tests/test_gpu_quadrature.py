"""Assembly with the caller's quadrature rule (fec_block_reference_set): the
same meshes and fields assembled with Gauss-Legendre and with
Gauss-Lobatto-Legendre tables (the reference's default q_type,
src/FunctionSpaces.jl:187), each against the oracle integrating with the same
tables; the two rules give different matrices, so the kernels really use the
tables they are handed."""
import numpy as np
import pytest

from helpers import FLOOR32, blocks_of, rel_err, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
TOL32 = 1e-5
RULES = ["GaussLegendre", "GaussLobattoLegendre"]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _assemble(fec, mesh, var_kind, physics, rule, *, bcs=(), precision="fp64", U=None, state=None, tables=None):
    torch = _torch()
    V = fec.FunctionSpace(mesh, q_type=rule)
    var = fec.ScalarFunction(V, "u") if var_kind == "scalar" else fec.VectorFunction(V, "u")
    asm = fec.SparseMatrixAssembler(var, device=0, precision=precision)
    if tables is not None:
        asm.set_reference_tables(tables)
    p = fec.create_parameters(mesh, asm, physics, dirichlet_bcs=bcs)
    if state is not None:
        p.state_old.copy_(torch.from_numpy(state))
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    return asm, p, R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), K


def _oracle(orc, mesh, asm, phys_name, props, U, tables, st_old=None, st_new=None):
    elems = {t for t in mesh.element_types.values()}
    assert len(elems) == 1
    (elem,) = elems
    N, dN, w = tables
    with orc.reference_tables(elem, N, dN, w):
        return orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, phys_name, props, U,
                                    asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st_old, st_new)


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_neohookean_hex8_both_rules(fec, orc, precision):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (6, 6, 6))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    out = {}
    for rule in RULES:
        asm, p, R, nz, K = _assemble(fec, mesh, "vector", phys, rule, precision=precision, U=U)
        tables = asm.reference_tables(1)
        assert np.array_equal(tables[2], asm.fspace.ref_fes[0][2])
        Ro, colptr, rowval, nzo = _oracle(orc, mesh, asm, "neohookean", phys.create_properties(), U, tables)
        assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
        if precision == "fp64":
            er, ek = rel_err(R, Ro), rel_err(nz, nzo)
            tol = TOL64
        else:
            er, ek = rel_err(R, Ro, FLOOR32), rel_err(nz, nzo, FLOOR32)
            tol = TOL32
        print(rule, precision, "residual", er, "nzval", ek)
        assert max(er) <= tol and max(ek) <= tol
        out[rule] = (R, nz)
    # the rules integrate differently: the tables are what the kernels used
    d = rel_err(out[RULES[0]][1], out[RULES[1]][1])
    assert d[1] > 1e-3, d


def test_poisson_hex8_lobatto_with_dirichlet(fec, orc):
    n = 9
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f) for f in ("left", "bottom")]
    U = np.random.default_rng(0).uniform(-1, 1, n ** 3)
    asm, p, R, nz, K = _assemble(fec, mesh, "scalar", fec.Poisson(1.0), "GaussLobattoLegendre", bcs=bcs, U=U)
    U[asm.dof.dirichlet_dofs - 1] = 0.0
    asm, p, R, nz, K = _assemble(fec, mesh, "scalar", fec.Poisson(1.0), "GaussLobattoLegendre", bcs=bcs, U=U)
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, asm, "poisson", [1.0], U, asm.reference_tables(1))
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64


def test_poisson_quad4_lobatto(fec, orc):
    # square node counts: the reference's structured quad generator (and so its
    # mirror) indexes x-coordinates with the y counter (StructuredMesh.jl:472-483)
    mesh = fec.StructuredMesh("quad", (0.0, 0.0), (1.0, 2.0), (12, 12))
    U = np.random.default_rng(4).uniform(-1, 1, mesh.num_nodes)
    asm, p, R, nz, K = _assemble(fec, mesh, "scalar", fec.Poisson(2.0), "GaussLobattoLegendre", U=U)
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, asm, "poisson", [2.0], U, asm.reference_tables(1))
    assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64


def test_j2_hex8_lobatto_plastic_step(fec, orc):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5))
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    rng = np.random.default_rng(3)
    X = mesh.nodal_coords
    U = np.zeros_like(X)
    U[:, 0] = 0.01 * X[:, 0]
    U[:, 1] = -0.003 * X[:, 1]
    U = (U + 1e-5 * rng.standard_normal(U.shape)).ravel()
    so = rng.uniform(0, 1e-4, 7 * 8 * mesh.num_elements())
    asm, p, R, nz, K = _assemble(fec, mesh, "vector", phys, "GaussLobattoLegendre", U=U, state=so)
    sn = np.zeros_like(so)
    Ro, _, _, nzo = _oracle(orc, mesh, asm, "j2", phys.create_properties(), U, asm.reference_tables(1), so, sn)
    assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64
    assert max(rel_err(p.state_new.cpu().numpy(), sn)) <= TOL64
    assert sn[6::7].max() > 0


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_hex27_lobatto(fec, orc, precision):
    """Hex27 with the 3-point Lobatto rule (nodal points); the FP32-element
    variant runs its contraction on the tensor cores."""
    mesh = fec.meshes.box_hex27((3, 3, 3))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    asm, p, R, nz, K = _assemble(fec, mesh, "vector", phys, "GaussLobattoLegendre", precision=precision, U=U)
    Ro, _, _, nzo = _oracle(orc, mesh, asm, "neohookean", phys.create_properties(), U, asm.reference_tables(1))
    if precision == "fp64":
        assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64
    else:
        assert max(rel_err(R, Ro, FLOOR32)) <= TOL32 and max(rel_err(nz, nzo, FLOOR32)) <= TOL32
        assert fec.load_library().fec_tensor_core_status(1) == 0


def test_tet10_vertex_rule(fec, orc):
    """TETRA10 integrated with a 4-point rule of the caller's (points at the
    vertices, weights 1/24), handed over as raw tables."""
    from fec_gb300.quadrature import tet_tables
    mesh = fec.meshes.box_tet10((3, 3, 3))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(mesh.nodal_coords, seed=6).ravel()
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    tables = tet_tables(10, pts, np.full(4, 1.0 / 24.0))
    asm, p, R, nz, K = _assemble(fec, mesh, "vector", phys, "GaussLegendre", U=U, tables=[tables])
    Ro, _, _, nzo = _oracle(orc, mesh, asm, "neohookean", phys.create_properties(), U, tables)
    assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64
    _, _, R_g, nz_g, _ = _assemble(fec, mesh, "vector", phys, "GaussLegendre", U=U)
    assert rel_err(nz, nz_g)[1] > 1e-3


def test_matrix_free_action_lobatto(fec, orc):
    """The matrix-free action reads the same tables: K v against the oracle's
    Lobatto-integrated matrix."""
    torch = _torch()
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    asm, p, R, nz, K = _assemble(fec, mesh, "vector", phys, "GaussLobattoLegendre", U=U)
    Vu = np.random.default_rng(1).standard_normal(asm.dof.unknown_dofs.size)
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    Kv = fec.assemble_matrix_free_action(asm, fec.stiffness_action, Uu, torch.from_numpy(Vu).cuda(), p)
    torch.cuda.synchronize()
    _, colptr, rowval, nzo = _oracle(orc, mesh, asm, "neohookean", phys.create_properties(), U,
                                     asm.reference_tables(1))
    import scipy.sparse as sp
    n = asm.dof.unknown_dofs.size
    Ko = sp.csc_matrix((nzo, rowval - 1, colptr - 1), shape=(n, n))
    assert max(rel_err(Kv.cpu().numpy(), Ko @ Vu)) <= TOL64
