"""GPU parity: libfec_gb300.so through its C ABI (via the fec_gb300 host mirror)
against the CPU oracle on the same seeded inputs.

Bar: colptr/rowval and DOF numbering bit-exact; FP64 residual and nzval within
1e-12 relative (max-abs over max-abs, and 2-norm); the FP32-element variant
within 1e-5 relative of the FP64 oracle."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from helpers import FLOOR32, blocks_of, entry_err, rel_err, stretch_field

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
TOL64 = 1e-12
TOL32 = 1e-5


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _setup(fec, mesh, var_kind, physics, bcs=(), precision="fp64"):
    V = fec.FunctionSpace(mesh)
    var = fec.ScalarFunction(V, "u") if var_kind == "scalar" else fec.VectorFunction(V, "u")
    asm = fec.SparseMatrixAssembler(var, device=0, precision=precision)
    p = fec.create_parameters(mesh, asm, physics, dirichlet_bcs=bcs)
    return asm, p


def _run(fec, asm, p, Ufull, precision=None):
    torch = _torch()
    Uu = torch.from_numpy(Ufull[asm.dof.unknown_dofs - 1].copy()).cuda()
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=precision)
    torch.cuda.synchronize()
    return R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), K


def _oracle(orc, mesh, phys_name, props, Ufull, asm, st_old=None, st_new=None):
    return orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, phys_name, props, Ufull,
                                asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st_old, st_new)


def test_poisson_hex8_32cubed_all_faces_dirichlet(fec, orc):
    """Plain Poisson workload: unit cube, 32^3 hex8, u = 0 on all faces, u ~ U[-1,1] (seed 0),
    f = sin(pi x) sin(pi y) sin(pi z)."""
    n = 33
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f) for f in orc.HEX8_FACES]
    asm, p = _setup(fec, mesh, "scalar", fec.Poisson(1.0), bcs)
    assert asm.dof.unknown_dofs.size == 29791
    rng = np.random.default_rng(0)
    U = rng.uniform(-1.0, 1.0, n ** 3)
    U[asm.dof.dirichlet_dofs - 1] = 0.0
    R, nz, K = _run(fec, asm, p, U)
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, "poisson", [1.0], U, asm)
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert K.nnz == 753571
    print("Poisson 32^3: residual", rel_err(R, Ro), "nzval", rel_err(nz, nzo),
          "entry-wise with floor 1e-14 (residue entries included):", entry_err(nz, nzo, 1e-14))
    assert max(rel_err(R, Ro)) <= TOL64
    assert max(rel_err(nz, nzo)) <= TOL64
    # determinism: bitwise-identical on a second call
    R2, nz2, _ = _run(fec, asm, p, U)
    assert np.array_equal(R, R2) and np.array_equal(nz, nz2)


def test_poisson_vector_and_matrix_entry_points_agree(fec, orc):
    """assemble_vector / assemble_stiffness separately equal the fused pass."""
    torch = _torch()
    n = 9
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name="left")]
    asm, p = _setup(fec, mesh, "scalar", fec.Poisson(2.0), bcs)
    U = np.random.default_rng(3).uniform(-1, 1, n ** 3)
    R, nz, _ = _run(fec, asm, p, U)
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    fec.assemble_vector(asm, fec.residual, Uu, p)
    fec.assemble_stiffness(asm, fec.stiffness, Uu, p)
    torch.cuda.synchronize()
    assert np.array_equal(fec.residual(asm).cpu().numpy(), R)
    assert np.array_equal(fec.stiffness(asm).nzval.cpu().numpy(), nz)
    # host input (end-to-end path) gives the same bits
    fec.assemble_vector(asm, fec.residual, U[asm.dof.unknown_dofs - 1].copy(), p)
    torch.cuda.synchronize()
    assert np.array_equal(fec.residual(asm).cpu().numpy(), R)


def test_fused_pass_into_caller_buffers(fec):
    """assemble_residual_and_stiffness(..., out=(R, nzval)) writes the caller's
    device arrays, bitwise what the assembler's own arrays receive; wrong
    shapes are refused."""
    torch = _torch()
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (6, 6, 6))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, "vector", phys)
    U = stretch_field(mesh.nodal_coords, seed=3).ravel()
    R, nz, _ = _run(fec, asm, p, U)
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    out = (torch.full((asm.dof.unknown_dofs.size,), np.nan, dtype=torch.float64, device="cuda"),
           torch.full((asm.nnz,), np.nan, dtype=torch.float64, device="cuda"))
    R2, K2 = fec.assemble_residual_and_stiffness(asm, Uu, p, out=out)
    torch.cuda.synchronize()
    assert R2.data_ptr() == out[0].data_ptr() and K2.nzval.data_ptr() == out[1].data_ptr()
    assert np.array_equal(out[0].cpu().numpy(), R) and np.array_equal(out[1].cpu().numpy(), nz)
    with pytest.raises(ValueError):
        fec.assemble_residual_and_stiffness(asm, Uu, p, out=(out[0][:-1], out[1]))


def test_poisson_quad4_gold_through_gpu(fec):
    """test/poisson/TestPoisson.jl:54-100: GPU-assembled residual and CSC stiffness
    on poisson.g, one linear solve, compared with poisson.gold."""
    g = np.load(GOLD / "poisson_quad4.npz")
    mesh = fec.UnstructuredMesh(g["coords"], {"block_1": ("QUAD4", g["conn"])},
                                nodesets={f"nset_{i}": g[f"nset_{i}"] for i in range(1, 5)})
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f"nset_{i}") for i in range(1, 5)]
    asm, p = _setup(fec, mesh, "scalar", fec.Poisson(2 * np.pi ** 2), bcs)
    R, nz, K = _run(fec, asm, p, np.zeros(mesh.num_nodes))
    Ks = K.to_scipy()
    u = np.zeros(mesh.num_nodes)
    u[asm.dof.unknown_dofs - 1] = spl.spsolve(Ks.tocsc(), -R)
    assert np.abs(u - g["u_gold"]).max() <= 1e-10 * np.abs(g["u_gold"]).max()


@pytest.mark.parametrize("n", [5, 9])
def test_neohookean_hex8_fp64(fec, orc, n):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, "vector", phys)
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    R, nz, K = _run(fec, asm, p, U)
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, "neohookean", phys.create_properties(), U, asm)
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    print(f"Neo-Hookean {n - 1}^3: residual", rel_err(R, Ro), "nzval", rel_err(nz, nzo),
          "entry-wise with floor 1e-14:", entry_err(nz, nzo, 1e-14))
    assert max(rel_err(R, Ro)) <= TOL64, rel_err(R, Ro)
    assert max(rel_err(nz, nzo)) <= TOL64, rel_err(nz, nzo)


def test_neohookean_hex8_fp32_element(fec, orc):
    n = 9
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, "vector", phys, precision="fp32_element")
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    R, nz, _ = _run(fec, asm, p, U)
    Ro, _, _, nzo = _oracle(orc, mesh, "neohookean", phys.create_properties(), U, asm)
    er, ek = rel_err(R, Ro, FLOOR32), rel_err(nz, nzo, FLOOR32)
    print(f"fp32-element error vs FP64 oracle: residual {er}, stiffness {ek}")
    assert max(ek) <= TOL32 and er[1] <= TOL32


def test_neohookean_with_dirichlet_and_two_blocks(fec, orc):
    """Two element blocks with different properties and partial Dirichlet elimination."""
    a = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5))
    b = fec.StructuredMesh("hex", (1.5, 0.0, 0.0), (2.5, 1.0, 1.2), (4, 4, 4))
    mesh = fec.meshes.merge_meshes([a, b])
    mesh.nodeset_nodes["fix"] = np.arange(1, 30, dtype=np.int64)
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0)
    p1, p2 = fec.NeoHookean(0.8, 0.4), fec.NeoHookean(2.0, 0.1)
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="fix"),
           fec.DirichletBC("u_z", lambda X, t: 0.0, nodeset_name="fix")]
    p = fec.create_parameters(mesh, asm, {"block_1": p1, "block_2": p2}, dirichlet_bcs=bcs)
    U = stretch_field(mesh.nodal_coords, seed=5).ravel()
    U[asm.dof.dirichlet_dofs - 1] = 0.0
    R, nz, K = _run(fec, asm, p, U)
    # oracle per block, merged the reference way (single COO over both blocks)
    Rf = np.zeros(U.size)
    Ks = []
    for name, ph in (("block_1", p1), ("block_2", p2)):
        r, k = orc.assemble([("HEX8", mesh.element_conns[name])], mesh.nodal_coords, "neohookean",
                            ph.create_properties(), U)
        Rf += r
        Ks.append(k)
    Is, Js, slots = orc.pattern(blocks_of(mesh), 3, asm.dof.dof_to_unknown)
    n_u = asm.dof.unknown_dofs.size
    colptr, rowval, nzo = orc.sparse_csc(n_u, n_u, Is, Js, np.concatenate(Ks)[slots - 1])
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert max(rel_err(nz, nzo)) <= TOL64
    assert max(rel_err(R, Rf[asm.dof.unknown_dofs - 1])) <= 1e-11


@pytest.mark.parametrize("kind", ["tet4", "tet10", "hex27"])
def test_higher_order_and_simplex_elements(fec, orc, kind):
    gen = {"tet4": fec.meshes.box_tet4, "tet10": fec.meshes.box_tet10, "hex27": fec.meshes.box_hex27}[kind]
    mesh = gen((4, 4, 4))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, "vector", phys)
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    R, nz, K = _run(fec, asm, p, U)
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, "neohookean", phys.create_properties(), U, asm)
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert max(rel_err(R, Ro)) <= TOL64
    assert max(rel_err(nz, nzo)) <= TOL64


def test_hex27_j2_fp64(fec, orc):
    """FP64 hex27 J2 (the symmetric double-float hex27 kernel) against the oracle,
    from a plastic first step."""
    mesh = fec.meshes.box_hex27((3, 3, 3))
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    asm, p = _setup(fec, mesh, "vector", phys)
    R, nz, K = _run(fec, asm, p, U)
    st = np.zeros(7 * 27 * mesh.num_elements())
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, "j2", phys.create_properties(), U, asm, st, np.zeros_like(st))
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert max(rel_err(R, Ro)) <= TOL64
    assert max(rel_err(nz, nzo)) <= TOL64


@pytest.mark.parametrize("classes", [True, False], ids=["class_gradients", "per_element_map"])
@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_hex27_fp64_pair_workspace_matches_whole_matrices(fec, phys_name, classes):
    """The FP64 hex27 double-float kernel writes the symmetric half of each
    element matrix (378 node pairs x 9 entries); with FEC_HEX27_PAIRS=0 it writes
    them whole.  Both hold the same values, so R, nzval and the state agree
    bitwise, with and without the class gradients (FEC_CLASS_TC=0) and with a
    Dirichlet face."""
    import os
    torch = _torch()
    mesh = fec.meshes.box_hex27((3, 3, 3))
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=6).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    mesh.nodeset_nodes["fix"] = np.flatnonzero(mesh.nodal_coords[:, 0] < 1e-12).astype(np.int64) + 1

    def run():
        bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="fix")]
        asm, p = _setup(fec, mesh, "vector", phys, bcs)
        R, nz, _ = _run(fec, asm, p, U)
        st = p.state_new.cpu().numpy().copy() if phys_name == "j2" else None
        return R, nz, st

    if not classes:
        os.environ["FEC_CLASS_TC"] = "0"
    try:
        R, nz, st = run()
        os.environ["FEC_HEX27_PAIRS"] = "0"
        R0, nz0, st0 = run()
    finally:
        os.environ.pop("FEC_HEX27_PAIRS", None)
        os.environ.pop("FEC_CLASS_TC", None)
    assert np.array_equal(R, R0) and np.array_equal(nz, nz0)
    if st is not None:
        assert np.array_equal(st, st0)


@pytest.mark.parametrize("kind", ["tet4", "tet10", "hex27"])
@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_higher_order_fp32_element(fec, orc, kind, phys_name):
    """FP32-element tet4/tet10/hex27 against the FP64 oracle.  These box meshes
    are blocks of translation classes, so tet10 and hex27 run the class
    tensor-core kernel; with it switched off (FEC_CLASS_TC=0) hex27 runs the
    per-element tensor-core kernel (tcgen05 kind::tf32 with a two-term split),
    which is also checked against the CUDA-core kernel."""
    import os
    gen = {"tet4": fec.meshes.box_tet4, "tet10": fec.meshes.box_tet10, "hex27": fec.meshes.box_hex27}[kind]
    mesh = gen((4, 4, 4))
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    asm, p = _setup(fec, mesh, "vector", phys, precision="fp32_element")
    R, nz, K = _run(fec, asm, p, U)
    nq = {"tet4": 1, "tet10": 4, "hex27": 27}[kind]
    ne = mesh.num_elements()
    st = np.zeros(7 * nq * ne) if phys_name == "j2" else None
    Ro, colptr, rowval, nzo = _oracle(orc, mesh, phys_name, phys.create_properties(), U, asm, st,
                                      None if st is None else np.zeros_like(st))
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    e_r, e_k = rel_err(R, Ro, FLOOR32), rel_err(nz, nzo, FLOOR32)
    print(kind, phys_name, "fp32-element vs FP64 oracle: residual", e_r, "nzval", e_k)
    assert max(e_r) <= TOL32 and max(e_k) <= TOL32
    if kind == "hex27":
        assert fec.load_library().fec_tensor_core_status(1) == 0
        out = {}
        for flags in (("FEC_CLASS_TC",), ("FEC_CLASS_TC", "FEC_HEX27_ON_CUDA_CORES")):
            for f in flags:
                os.environ[f] = "0" if f == "FEC_CLASS_TC" else "1"
            try:
                asm2, p2 = _setup(fec, mesh, "vector", phys, precision="fp32_element")
                out[len(flags)] = _run(fec, asm2, p2, U)[:2]
            finally:
                for f in flags:
                    del os.environ[f]
        (R1, nz1), (R2, nz2) = out[1], out[2]
        print("hex27 per-element tensor cores vs CUDA cores: residual", rel_err(R1, R2), "nzval",
              rel_err(nz1, nz2, FLOOR32))
        assert np.array_equal(R1, R2)  # the per-element kernels form the residual alike
        assert max(rel_err(nz1, nz2, FLOOR32)) <= 5e-6   # two FP32-element paths, entry-wise
        assert max(rel_err(nz, nz1, FLOOR32)) <= TOL32 and max(rel_err(R, R1, FLOOR32)) <= TOL32


def test_j2_one_load_step_with_state(fec, orc):
    torch = _torch()
    n = 6
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    asm, p = _setup(fec, mesh, "vector", phys)
    rng = np.random.default_rng(3)
    X = mesh.nodal_coords
    U = np.zeros_like(X)
    U[:, 0] = 0.01 * X[:, 0]
    U[:, 1] = -0.003 * X[:, 1]
    U = (U + 1e-5 * rng.standard_normal(U.shape)).ravel()
    so = rng.uniform(0, 1e-4, p.state_old.numel())
    p.state_old.copy_(torch.from_numpy(so))
    R, nz, _ = _run(fec, asm, p, U)
    sn = np.zeros_like(so)
    Ro, _, _, nzo = _oracle(orc, mesh, "j2", phys.create_properties(), U, asm, so, sn)
    assert max(rel_err(R, Ro)) <= TOL64
    assert max(rel_err(nz, nzo)) <= TOL64
    assert max(rel_err(p.state_new.cpu().numpy(), sn)) <= TOL64
    assert sn[6::7].max() > 0  # some points yielded


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_j2_load_path_with_state(fec, orc, precision):
    """J2 plasticity over a 6-step uniaxial load path: state carried step to step
    (state_new of step s becomes state_old of step s+1), compared with the oracle
    doing the same at every step."""
    torch = _torch()
    from fec_gb300.workloads import uniaxial_path
    n = 6
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    asm, p = _setup(fec, mesh, "vector", phys)
    so = np.zeros(p.state_old.numel())
    tol = TOL64 if precision == "fp64" else TOL32
    floor = 1e-2 if precision == "fp64" else FLOOR32
    yielded = 0
    for step in range(1, 7):
        U = uniaxial_path(mesh.nodal_coords, step, nsteps=6, final_strain=0.01).ravel()
        R, nz, _ = _run(fec, asm, p, U, precision=precision)
        sn = np.zeros_like(so)
        Ro, _, _, nzo = _oracle(orc, mesh, "j2", phys.create_properties(), U, asm, so, sn)
        assert max(rel_err(R, Ro, floor)) <= tol, (step, rel_err(R, Ro, floor))
        assert max(rel_err(nz, nzo, floor)) <= tol, (step, rel_err(nz, nzo, floor))
        assert max(rel_err(p.state_new.cpu().numpy(), sn, floor)) <= (1e-12 if precision == "fp64" else 1e-4)
        yielded = max(yielded, int((sn[6::7] > 0).sum()))
        p.swap_states()
        so = sn
        # the library reads state_old from the parameters; keep it equal to the oracle's
        p.state_old.copy_(torch.from_numpy(so))
    assert yielded > 0


def test_nonfinite_outputs_are_reported(fec):
    """The boundary's NaN/Inf check: a NaN in the unknowns reaches the residual and
    nzval, and fec_check_finite reports FEC_ERR_NONFINITE naming the array."""
    torch = _torch()
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (4, 4, 4))
    asm, p = _setup(fec, mesh, "vector", fec.NeoHookean.from_youngs(1.0, 0.3))
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    fec.assemble_residual_and_stiffness(asm, Uu, p, check_finite=True)   # finite: no error
    Uu[7] = float("nan")
    with pytest.raises(fec.FECError) as info:
        fec.assemble_residual_and_stiffness(asm, Uu, p, check_finite=True)
    assert info.value.status == -5 and "residual" in str(info.value)


@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
@pytest.mark.parametrize("n", [3, 17, 40])
def test_fp64_hex8_warp_specialised_kernel_matches_tile_kernel(fec, n, phys_name):
    """The persistent warp-specialised FP64 hex8 kernel (default) against the
    one-tile-per-CTA kernel (FEC_HEX8_DF64=tile): bitwise the same residual,
    stiffness and new state, for a single partial tile (27 elements), a few
    tiles per CTA (4,913) and many (64,000); fused and separate R / K calls.
    These structured meshes would take the affine tensor-core path: both runs
    keep the per-element kernels (FEC_HEX8_AFFINE=0)."""
    import os
    torch = _torch()
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    asm, p = _setup(fec, mesh, "vector", phys)
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    out = {}
    for kernel in ("ws", "tile"):
        os.environ["FEC_HEX8_AFFINE"] = "0"
        if kernel == "tile":
            os.environ["FEC_HEX8_DF64"] = "tile"
        try:
            R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
            torch.cuda.synchronize()
            res = [R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), p.state_new.cpu().numpy().copy()]
            fec.assemble_vector(asm, fec.residual, Uu, p)
            fec.assemble_stiffness(asm, fec.stiffness, Uu, p)
            torch.cuda.synchronize()
            res += [fec.residual(asm).cpu().numpy().copy(), fec.stiffness(asm).nzval.cpu().numpy().copy()]
            out[kernel] = res
        finally:
            os.environ.pop("FEC_HEX8_DF64", None)
            os.environ.pop("FEC_HEX8_AFFINE", None)
    for a, b in zip(out["ws"], out["tile"]):
        assert np.array_equal(a, b)
    assert np.array_equal(out["ws"][0], out["ws"][3]) and np.array_equal(out["ws"][1], out["ws"][4])


@pytest.mark.parametrize("case", ["neohookean", "neohookean_dirichlet", "j2_fp32", "batch"])
def test_pipelined_gather_matches_node_gather(fec, case):
    """The software-pipelined hex8 node gather (default for one hex8 block)
    against the one-warp-per-node gather (FEC_GATHER_PIPE=0): bitwise the same
    residual and stiffness, with every node in the staged fast path, with
    Dirichlet neighbourhoods (nodes gathered in place), J2 in FP32-element
    arithmetic, and a batch of uneven meshes (nodes with 1 to 8 elements)."""
    import os
    torch = _torch()
    from fec_gb300 import batching
    precision = "fp64"
    bcs = ()
    if case == "batch":
        mesh = batching.box_batch([3, 1, 5, 2, 7]).mesh
    else:
        # a cube: the reference's structured hex generator (and so its mirror) is only
        # consistent for equal counts (StructuredMesh.jl:433-449)
        mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 2.0, 1.5), (11, 11, 11))
    if case.startswith("j2"):
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
        precision = "fp32_element"
    else:
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    if case == "neohookean_dirichlet":
        bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
               fec.DirichletBC("u_z", lambda X, t: 0.0, nodeset_name="top")]
    asm, p = _setup(fec, mesh, "vector", phys, bcs, precision=precision)
    U[asm.dof.dof_to_unknown < 0] = 0.0
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    out = {}
    for pipe in ("1", "0"):
        os.environ["FEC_GATHER_PIPE"] = pipe
        try:
            R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
            torch.cuda.synchronize()
            out[pipe] = (R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy())
        finally:
            del os.environ["FEC_GATHER_PIPE"]
    assert np.array_equal(out["1"][0], out["0"][0]) and np.array_equal(out["1"][1], out["0"][1])


def test_bounded_waits_report_and_drain(fec):
    """The element kernels' bounded waits, made to give up on operations that
    complete anyway (a budget of one SM clock, fec_set_wait_budget: a wait that
    starts right after its copy or MMAs were issued gives up): the hex8
    kernel's wait on its bulk table copy reports through the device flag, waits
    again and falls back to plain loads (the results stay bitwise exact); the
    affine hex8 tensor-core kernel reports, waits its MMAs out and carries on
    (bitwise exact); the hex27 tensor-core kernel reports, drains its MMAs and frees its tensor
    memory (its results are invalid, but the context stays usable: the next
    call is exact and the flag stays clear)."""
    import os
    torch = _torch()
    lib = fec.load_library()
    from fec_gb300 import _lib
    assert lib.fec_tensor_core_status(1) == 0
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (7, 7, 7))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, "vector", phys)
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    os.environ["FEC_HEX8_DF64"] = "tile"   # the hex8 kernel that stages by bulk copy
    os.environ["FEC_HEX8_AFFINE"] = "0"    # (not the affine path this structured mesh would take)
    try:
        R0, nz0, _ = _run(fec, asm, p, U)
        assert lib.fec_tensor_core_status(0) == 0
        assert lib.fec_set_wait_budget(1) == 0
        R1, nz1, _ = _run(fec, asm, p, U)
    finally:
        lib.fec_set_wait_budget(0)
        del os.environ["FEC_HEX8_DF64"]
        del os.environ["FEC_HEX8_AFFINE"]
    assert lib.fec_tensor_core_status(1) == _lib.FEC_ERR_DEVICE    # the waits gave up, and said so
    assert np.array_equal(R0, R1) and np.array_equal(nz0, nz1)      # ... and the plain loads took over
    # the affine tensor-core kernel (this structured mesh, FP64): its epilogue's
    # waits give up, report, wait the MMAs out and carry on, so the results stay exact
    R2, nz2, _ = _run(fec, asm, p, U)
    assert lib.fec_tensor_core_status(0) == 0
    assert lib.fec_set_wait_budget(1) == 0
    try:
        R3, nz3, _ = _run(fec, asm, p, U)
    finally:
        lib.fec_set_wait_budget(0)
    assert lib.fec_tensor_core_status(1) == _lib.FEC_ERR_DEVICE
    assert np.array_equal(R2, R3) and np.array_equal(nz2, nz3)
    assert not np.array_equal(nz0, nz2)  # (the affine path, not the per-element kernel, ran)
    # hex27 FP32-element on the tensor cores
    mesh27 = fec.meshes.box_hex27((3, 3, 3))
    asm27, p27 = _setup(fec, mesh27, "vector", phys, precision="fp32_element")
    U27 = stretch_field(mesh27.nodal_coords, seed=2).ravel()
    Ra, nza, _ = _run(fec, asm27, p27, U27)
    assert lib.fec_tensor_core_status(0) == 0
    assert lib.fec_set_wait_budget(1) == 0
    try:
        _run(fec, asm27, p27, U27)
    finally:
        lib.fec_set_wait_budget(0)
    assert lib.fec_tensor_core_status(1) == _lib.FEC_ERR_DEVICE
    with pytest.raises(fec.FECError) as info:   # the boundary's output check reports it too
        lib2 = fec.load_library()
        lib2.fec_set_wait_budget(1)
        try:
            fec.assemble_residual_and_stiffness(asm27, torch.from_numpy(U27[asm27.dof.unknown_dofs - 1].copy()).cuda(),
                                                p27, check_finite=True)
        finally:
            lib2.fec_set_wait_budget(0)
    assert info.value.status == _lib.FEC_ERR_DEVICE
    assert lib.fec_tensor_core_status(1) == _lib.FEC_ERR_DEVICE
    Rb, nzb, _ = _run(fec, asm27, p27, U27)
    assert lib.fec_tensor_core_status(0) == 0
    assert np.array_equal(Ra, Rb) and np.array_equal(nza, nzb)
