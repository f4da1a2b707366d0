"""Matrix-free tangent action (assemble_matrix_free_action! + hvp) against the
oracle's assembled CSC stiffness times the direction, as the reference's
test/TestAssemblers.jl:279-339 compares the matrix-free and assembled products:
Poisson (all faces Dirichlet), Neo-Hookean on hex8/tet4/tet10/hex27 with
Dirichlet dofs, J2 with a plastic state; FP64 within 1e-12, FP32-element within
1e-5; repeated calls bitwise identical."""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import FLOOR32, FLOOR64, blocks_of, rel_err, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
TOL32 = 1e-5


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _oracle_matrix(orc, mesh, phys_name, props, U, asm, st_old=None):
    st_new = None if st_old is None else np.zeros_like(st_old)
    _, colptr, rowval, nzval = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, phys_name, props, U,
                                                    asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st_old, st_new)
    n = asm.dof.unknown_dofs.size
    return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(n, n))


def _action(fec, asm, p, U, Vu):
    torch = _torch()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    Kv = fec.assemble_matrix_free_action(asm, fec.stiffness_action, Uu, torch.from_numpy(Vu).cuda(), p)
    torch.cuda.synchronize()
    return Kv.cpu().numpy().copy()


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_poisson_action(fec, orc, precision):
    n = 12
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    asm = fec.SparseMatrixAssembler(fec.ScalarFunction(fec.FunctionSpace(mesh), "u"), device=0, precision=precision)
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f)
           for f in ("bottom", "right", "front", "top", "left", "back")]
    p = fec.create_parameters(mesh, asm, fec.Poisson(1.0), dirichlet_bcs=bcs)
    rng = np.random.default_rng(0)
    U = rng.uniform(-1, 1, mesh.num_nodes)
    Vu = rng.standard_normal(asm.dof.unknown_dofs.size)
    Kv = _action(fec, asm, p, U, Vu)
    K = _oracle_matrix(orc, mesh, "poisson", fec.Poisson(1.0).create_properties(), U, asm)
    e = rel_err(Kv, K @ Vu, FLOOR64 if precision == "fp64" else FLOOR32)
    print(precision, "Poisson K v vs assembled:", e)
    assert max(e) <= (TOL64 if precision == "fp64" else TOL32)
    # the reference's direction: all ones
    ones = np.ones_like(Vu)
    Kv1 = _action(fec, asm, p, U, ones)
    ref1 = K @ ones
    assert np.abs(Kv1 - ref1).max() <= (1e-12 if precision == "fp64" else 1e-5) * np.abs(K).max()


@pytest.mark.parametrize("kind", ["hex8", "tet4", "tet10", "hex27"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_neohookean_action(fec, orc, kind, precision):
    if kind == "hex8":
        mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (7, 7, 7))
    else:
        mesh = {"tet4": fec.meshes.box_tet4, "tet10": fec.meshes.box_tet10, "hex27": fec.meshes.box_hex27}[kind](
            (4, 4, 4))
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0, precision=precision)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom")] if kind == "hex8" else []
    p = fec.create_parameters(mesh, asm, phys, dirichlet_bcs=bcs)
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    if bcs:
        U[asm.dof.dof_to_unknown < 0] = 0.0   # the Dirichlet values the field update writes
    Vu = np.random.default_rng(1).standard_normal(asm.dof.unknown_dofs.size)
    Kv = _action(fec, asm, p, U, Vu)
    K = _oracle_matrix(orc, mesh, "neohookean", phys.create_properties(), U, asm)
    e = rel_err(Kv, K @ Vu, FLOOR64 if precision == "fp64" else FLOOR32)
    print(kind, precision, "Neo-Hookean K v vs assembled:", e)
    assert max(e) <= (TOL64 if precision == "fp64" else TOL32)
    assert np.array_equal(Kv, _action(fec, asm, p, U, Vu))   # deterministic


def test_j2_action_with_plastic_state(fec, orc):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (6, 6, 6))
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    p = fec.create_parameters(mesh, asm, phys)
    torch = _torch()
    rng = np.random.default_rng(3)
    st = np.concatenate([rng.normal(0, 5e-4, (8 * mesh.num_elements(), 6)),
                         rng.uniform(0, 1e-3, (8 * mesh.num_elements(), 1))], 1).ravel()
    p.state_old.copy_(torch.from_numpy(st))
    U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    Vu = rng.standard_normal(asm.dof.unknown_dofs.size)
    Kv = _action(fec, asm, p, U, Vu)
    K = _oracle_matrix(orc, mesh, "j2", phys.create_properties(), U, asm, st)
    e = rel_err(Kv, K @ Vu)
    print("J2 K v vs assembled:", e)
    assert max(e) <= TOL64


@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_affine_action_matches_per_element_map(fec, phys_name):
    """FP64 blocks of translated hex8 elements read the block's constant spatial
    gradients and JxW instead of mapping every element: within 1e-12 of the
    per-element map (FEC_HEX8_AFFINE=0), and a different rounding of it (the
    path ran)."""
    import os
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (9, 9, 9))
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=4).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    p = fec.create_parameters(mesh, asm, phys)
    Vu = np.random.default_rng(5).standard_normal(asm.dof.unknown_dofs.size)
    Kv = _action(fec, asm, p, U, Vu)
    os.environ["FEC_HEX8_AFFINE"] = "0"
    try:
        Kv_pe = _action(fec, asm, p, U, Vu)
    finally:
        os.environ.pop("FEC_HEX8_AFFINE", None)
    e = rel_err(Kv, Kv_pe)
    print(phys_name, "affine action vs per-element map:", e)
    assert max(e) <= TOL64
    assert not np.array_equal(Kv, Kv_pe)
