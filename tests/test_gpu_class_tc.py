"""FP32-element tet10 / hex27 blocks made of translation classes (element e a
translate of element e mod P: one class for a hex27 box, the six Kuhn tets of
a cube for a tet10 box): the element stiffness on the tensor cores against
each class's constant gradient products (class_tc_kernel).  Checked against
the FP64 oracle at the FP32-element bar, against the per-element kernels
(FEC_CLASS_TC=0) entry by entry, with state carried over load steps, with
tiles that are not full, and on a mesh that is not made of classes (the
per-element kernels stay in charge: bitwise their results)."""
import os

import numpy as np
import pytest

from helpers import FLOOR32, FLOOR64, blocks_of, rel_err, stretch_field

pytestmark = pytest.mark.gpu
TOL32 = 1e-5


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _setup(fec, mesh, physics):
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0, precision="fp32_element")
    return asm, fec.create_parameters(mesh, asm, physics)


def _run(fec, asm, p, U, class_tc=True):
    torch = _torch()
    if not class_tc:
        os.environ["FEC_CLASS_TC"] = "0"
    try:
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
    finally:
        os.environ.pop("FEC_CLASS_TC", None)
    sn = p.state_new.cpu().numpy().copy() if any(ph.NS for ph in p.physics) else None
    return R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), sn, K


def _mesh(fec, kind, n=4):
    # 3^3 cubes: 27 hex27 elements (tiles of 12, 12, 3), 162 tets (27 per class: 12, 12, 3)
    return {"tet10": fec.meshes.box_tet10, "hex27": fec.meshes.box_hex27}[kind]((n, n, n))


@pytest.mark.parametrize("kind", ["tet10", "hex27"])
def test_class_tensor_cores_neohookean(fec, orc, kind):
    mesh = _mesh(fec, kind)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, phys)
    U = stretch_field(mesh.nodal_coords, seed=3).ravel()
    R, nz, _, K = _run(fec, asm, p, U)
    R0, nz0, _, _ = _run(fec, asm, p, U, class_tc=False)
    Ro, colptr, rowval, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean",
                                                   phys.create_properties(), U, asm.dof.dof_to_unknown,
                                                   asm.dof.unknown_dofs)
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    e_r, e_k = rel_err(R, Ro, FLOOR32), rel_err(nz, nzo, FLOOR32)
    e_r0, e_k0 = rel_err(R, R0, FLOOR32), rel_err(nz, nz0, FLOOR32)
    print(kind, "class tensor cores vs FP64 oracle: residual", e_r, "nzval", e_k,
          "| vs per-element kernels: residual", e_r0, "nzval", e_k0)
    assert max(e_r) <= TOL32 and max(e_k) <= TOL32
    assert max(e_r0) <= 5e-6 and max(e_k0) <= 5e-6
    assert not np.array_equal(nz, nz0)   # (the class kernel, not the per-element one, ran)
    assert fec.load_library().fec_tensor_core_status(1) == 0


@pytest.mark.parametrize("kind", ["tet10", "hex27"])
def test_class_tensor_cores_j2_with_state(fec, orc, kind):
    """J2 over three load steps with the state carried by each path: residual,
    tangent and state against the per-element kernels each step, and the first
    step against the FP64 oracle."""
    from fec_gb300.workloads import uniaxial_path
    mesh = _mesh(fec, kind)
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    asm, p = _setup(fec, mesh, phys)
    asm0, p0 = _setup(fec, mesh, phys)
    nq = {"tet10": 4, "hex27": 27}[kind]
    plastic = 0
    for step in (2, 4, 6):
        U = uniaxial_path(mesh.nodal_coords, step, nsteps=6, final_strain=0.01).ravel()
        R, nz, sn, _ = _run(fec, asm, p, U)
        R0, nz0, sn0, _ = _run(fec, asm0, p0, U, class_tc=False)
        e = (rel_err(R, R0, FLOOR32), rel_err(nz, nz0, FLOOR32), rel_err(sn, sn0, FLOOR32))
        print(kind, "step", step, "class vs per-element: residual", e[0], "nzval", e[1], "state", e[2])
        assert max(e[0]) <= 1e-4 and max(e[1]) <= 1e-4 and max(e[2]) <= 1e-4
        if step == 2:
            st = np.zeros(7 * nq * mesh.num_elements())
            Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "j2", phys.create_properties(),
                                                 U, asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st,
                                                 np.zeros_like(st))
            assert max(rel_err(R, Ro, FLOOR32)) <= TOL32 and max(rel_err(nz, nzo, FLOOR32)) <= TOL32
        plastic = max(plastic, int((sn[6::7] > 0).sum()))
        p.swap_states()
        p0.swap_states()
    assert plastic > 0


def test_mesh_without_classes_keeps_per_element_kernels(fec):
    """One interior node moved: no element period exists, and the per-element
    kernels assemble the block (bitwise their results with the class kernel
    switched off)."""
    mesh = _mesh(fec, "tet10")
    X = mesh.nodal_coords
    inner = np.nonzero(np.all((X > 0.1) & (X < 0.9), axis=1))[0][0]
    X[inner] += np.array([0.01, -0.005, 0.007])
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, phys)
    U = stretch_field(X, seed=4).ravel()
    R, nz, _, _ = _run(fec, asm, p, U)
    R0, nz0, _, _ = _run(fec, asm, p, U, class_tc=False)
    assert np.array_equal(R, R0) and np.array_equal(nz, nz0)


def test_mixed_mesh_fp32_against_oracle(fec, orc):
    """The tet4 + tet10 + hex27 mesh of the batched workload (three blocks)."""
    from fec_gb300 import batching
    mesh = batching.mixed_mesh(2, 2, 3)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    asm, p = _setup(fec, mesh, phys)
    U = stretch_field(mesh.nodal_coords, seed=6).ravel()
    R, nz, _, _ = _run(fec, asm, p, U)
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean", phys.create_properties(),
                                         U, asm.dof.dof_to_unknown, asm.dof.unknown_dofs)
    assert max(rel_err(R, Ro, FLOOR32)) <= TOL32 and max(rel_err(nz, nzo, FLOOR32)) <= TOL32


def _hex_tet_mesh(fec, n=4):
    """A hex8 box whose last layer of cubes is split into Kuhn tets: a hex8 block
    and a tet4 block sharing the interface nodes."""
    from fec_gb300.meshes import _KUHN, _orient_tets
    box = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1, n + 1, n + 1))
    X = box.nodal_coords
    hexes = box.element_conns["block_1"]
    last = X[hexes - 1][:, :, 0].max(axis=1) > 1.0 - 1e-12   # cubes touching x = 1
    tets = _orient_tets(X, hexes[last][:, _KUHN].reshape(-1, 4))
    return fec.UnstructuredMesh(X, {"hexes": ("HEX8", hexes[~last]), "tets": ("TETRA4", tets)})


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
@pytest.mark.parametrize("kind", ["mixed", "hex_tet"])
def test_mixed_mesh_gather_groups(fec, orc, precision, kind):
    """Meshes of mixed element sizes gather their nodes in groups of one element size
    (several elements' loads in flight), nodes shared between sizes on the generic
    routine; FEC_GATHER_RUNS=generic gathers every node on the generic routine in one
    launch: bitwise the same residual and nzval, and the FP64 oracle agrees."""
    torch = _torch()
    from fec_gb300 import batching
    mesh = batching.mixed_mesh(2, 2, 3) if kind == "mixed" else _hex_tet_mesh(fec)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0, precision=precision)
    p = fec.create_parameters(mesh, asm, phys)
    U = stretch_field(mesh.nodal_coords, seed=8).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    out = []
    for runs in (None, "generic"):
        if runs:
            os.environ["FEC_GATHER_RUNS"] = runs
        try:
            R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
            torch.cuda.synchronize()
            out.append((R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy()))
        finally:
            os.environ.pop("FEC_GATHER_RUNS", None)
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean", phys.create_properties(),
                                         U, asm.dof.dof_to_unknown, asm.dof.unknown_dofs)
    tol, floor = (1e-12, FLOOR64) if precision == "fp64" else (TOL32, FLOOR32)
    e_r, e_k = rel_err(out[0][0], Ro, floor), rel_err(out[0][1], nzo, floor)
    print(kind, precision, "vs oracle: residual", e_r, "nzval", e_k)
    assert max(e_r[:2]) <= tol and max(e_k) <= tol   # residual normwise (it cancels), nzval entry by entry


@pytest.mark.parametrize("kind", ["tet10", "hex27"])
@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_class_fp64(fec, orc, phys_name, kind):
    """FP64 blocks of translation classes: tet10 with the tangent on the tensor cores
    in exact BF16 digit slices, hex27 with the double-float kernel reading each class's
    gradients instead of mapping every element. Within the FP64 bar (1e-12) of the
    oracle entry by entry (nzval) and normwise (the residual), and of the per-element
    double-float kernel (FEC_CLASS_TC=0)."""
    torch = _torch()
    mesh = _mesh(fec, kind)
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=3).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0, precision="fp64")
    p = fec.create_parameters(mesh, asm, phys)
    R, nz, sn, _ = _run(fec, asm, p, U)
    R0, nz0, sn0, _ = _run(fec, asm, p, U, class_tc=False)
    ne = mesh.num_elements()
    nq = 4 if kind == "tet10" else 27
    st = np.zeros(7 * nq * ne) if phys_name == "j2" else None
    st_new = None if st is None else np.zeros_like(st)
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, phys_name, phys.create_properties(), U,
                                         asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st, st_new)
    e_r, e_k = rel_err(R, Ro), rel_err(nz, nzo)
    e_r0, e_k0 = rel_err(R, R0), rel_err(nz, nz0)
    print("fp64", kind, phys_name, "class vs oracle: residual", e_r, "nzval", e_k, "| vs per-element: residual", e_r0,
          "nzval", e_k0)
    assert max(e_r[:2]) <= 1e-12 and max(e_k) <= 1e-12
    assert max(e_r0[:2]) <= 1e-12 and max(e_k0) <= 1e-12
    assert not np.array_equal(nz, nz0)   # (the class kernel ran)
    if phys_name == "j2":
        assert max(rel_err(sn, st_new)[:2]) <= 1e-12 and int((sn[6::7] > 0).sum()) > 0
    assert fec.load_library().fec_tensor_core_status(1) == 0


@pytest.mark.parametrize("case", ["tet10-fp64", "tet10-fp32_element", "hex27-fp32_element"])
def test_class_separate_calls_equal_fused(fec, case):
    """Residual-only and stiffness-only calls on class blocks run the class kernel's
    point phase and arithmetic too: bitwise the fused call's residual and tangent."""
    torch = _torch()
    kind, precision = case.split("-")
    mesh = _mesh(fec, kind)
    V = fec.FunctionSpace(mesh)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(V, "u"), device=0, precision=precision)
    p = fec.create_parameters(mesh, asm, fec.NeoHookean.from_youngs(1.0, 0.3))
    U = stretch_field(mesh.nodal_coords, seed=9).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    R_f, nz_f = R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy()
    fec.assemble_vector(asm, fec.residual, Uu, p)
    R_s = fec.residual(asm).cpu().numpy().copy()
    fec.assemble_stiffness(asm, fec.stiffness, Uu, p)
    nz_s = fec.stiffness(asm).nzval.cpu().numpy().copy()
    assert np.array_equal(R_s, R_f) and np.array_equal(nz_s, nz_f)
