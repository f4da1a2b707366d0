"""Hex8 blocks whose elements are translates of one another (structured meshes)
take the affine path: the FP64 Neo-Hookean / J2 tangent contraction runs on the
tensor cores in exact 8-bit digit slices against one constant gradient-product
operand per block (csrc/fec_hex8_affine_tc.cu).  It is held to the oracle at
the FP64 bar (entry-wise), for partial, single and many tiles per CTA; its
residual-only and tangent-only calls agree bitwise with the fused call; and a
block that is not congruent keeps the per-element kernels."""
import os

import numpy as np
import pytest

from helpers import blocks_of, rel_err, residual_err, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


class per_element_kernels:
    """with per_element_kernels(): FEC_HEX8_AFFINE=0 for the block."""

    def __enter__(self):
        os.environ["FEC_HEX8_AFFINE"] = "0"

    def __exit__(self, *exc):
        os.environ.pop("FEC_HEX8_AFFINE", None)


def _assemble(fec, mesh, phys, U, state=None):
    torch = _torch()
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    p = fec.create_parameters(mesh, asm, phys)
    if state is not None:
        p.state_old.copy_(torch.from_numpy(state))
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    st = p.state_new.cpu().numpy().copy() if state is not None else None
    return asm, p, Uu, R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), st


def _oracle(orc, mesh, asm, phys_name, props, U, st_old=None, st_new=None):
    ab = np.zeros(U.size)  # per dof the summed magnitudes of its residual's terms
    if st_old is None:
        orc.assemble(blocks_of(mesh), mesh.nodal_coords, phys_name, props, U, want_k=False, abs_out=ab)
    Ro, colptr, rowval, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, phys_name, props, U,
                                                   asm.dof.dof_to_unknown, asm.dof.unknown_dofs, st_old, st_new)
    return Ro, nzo, ab[asm.dof.unknown_dofs - 1]


@pytest.mark.parametrize("n", [2, 4, 15, 24])
def test_neohookean_affine_matches_oracle(fec, orc, n):
    """n^3 elements: 8 (less than one 14-element tile), 64 (five tiles, the last
    partial), 3,375 and 13,824 (several tiles per CTA)."""
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    asm, p, _, R, nz, _ = _assemble(fec, mesh, phys, U)
    Ro, nzo, ab = _oracle(orc, mesh, asm, "neohookean", phys.create_properties(), U)
    er, ek = residual_err(R, Ro, ab), rel_err(nz, nzo)
    with per_element_kernels():
        _, _, _, R_pe, nz_pe, _ = _assemble(fec, mesh, phys, U)
    print(f"affine {n}^3: residual {er}, nzval {ek}; per-element kernels: residual {residual_err(R_pe, Ro, ab)}, "
          f"nzval {rel_err(nz_pe, nzo)}")
    assert max(er) <= TOL64 and max(ek) <= TOL64
    if n >= 4:
        assert not np.array_equal(nz, nz_pe)  # the affine path is the one that ran


def test_j2_affine_plastic_step_matches_oracle(fec, orc):
    """A plastic J2 step from a stored state: residual, tangent and new state."""
    n = 10
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
    rng = np.random.default_rng(3)
    X = mesh.nodal_coords
    U = np.zeros_like(X)
    U[:, 0] = 0.01 * X[:, 0]
    U[:, 1] = -0.003 * X[:, 1]
    U = (U + 1e-5 * rng.standard_normal(U.shape)).ravel()
    so = rng.uniform(0, 1e-4, 7 * 8 * mesh.num_elements())
    asm, p, _, R, nz, sn = _assemble(fec, mesh, phys, U, state=so)
    sno = np.zeros_like(so)
    Ro, nzo, _ = _oracle(orc, mesh, asm, "j2", phys.create_properties(), U, so, sno)
    print("affine J2: residual", rel_err(R, Ro), "nzval", rel_err(nz, nzo), "state", rel_err(sn, sno))
    assert max(rel_err(R, Ro)) <= TOL64 and max(rel_err(nz, nzo)) <= TOL64
    assert max(rel_err(sn, sno)) <= TOL64
    assert sno[6::7].max() > 0  # points yielded


@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_affine_fused_and_separate_calls_agree_bitwise(fec, phys_name):
    """Residual-only (its own kernel), tangent-only and fused calls of the
    affine path give bitwise the same R, nzval and new state."""
    torch = _torch()
    n = 9
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=1).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    asm, p, Uu, R, nz, _ = _assemble(fec, mesh, phys, U)
    st = p.state_new.cpu().numpy().copy()
    fec.assemble_vector(asm, fec.residual, Uu, p)
    torch.cuda.synchronize()
    assert np.array_equal(fec.residual(asm).cpu().numpy(), R)
    assert np.array_equal(p.state_new.cpu().numpy(), st)
    fec.assemble_stiffness(asm, fec.stiffness, Uu, p)
    torch.cuda.synchronize()
    assert np.array_equal(fec.stiffness(asm).nzval.cpu().numpy(), nz)


def test_noncongruent_block_keeps_per_element_kernels(fec, orc):
    """One interior node moved by 1e-3 of the element size: the block is not
    congruent, so the results are bitwise those of the per-element kernels."""
    n = 6
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    X = mesh.nodal_coords.copy()
    X[(n + 1) ** 2 * 3 + (n + 1) * 3 + 3] += 1e-3 / n
    mesh = fec.meshes.UnstructuredMesh(X, {b: (mesh.element_types[b], mesh.element_conns[b])
                                            for b in mesh.element_block_names})
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    U = stretch_field(X, seed=1).ravel()
    _, _, _, R, nz, _ = _assemble(fec, mesh, phys, U)
    with per_element_kernels():
        _, _, _, R_pe, nz_pe, _ = _assemble(fec, mesh, phys, U)
    assert np.array_equal(R, R_pe) and np.array_equal(nz, nz_pe)


class node_row_workspace:
    """with node_row_workspace(): FEC_HEX8_PAIRS=0, the tensor-core kernel writes
    node rows of the whole K_e instead of the symmetric half."""

    def __enter__(self):
        os.environ["FEC_HEX8_PAIRS"] = "0"

    def __exit__(self, *exc):
        os.environ.pop("FEC_HEX8_PAIRS", None)


@pytest.mark.parametrize("phys_name", ["neohookean", "j2"])
def test_pair_workspace_matches_node_rows_bitwise(fec, orc, phys_name):
    """The symmetric-half workspace (36 node pairs x 9 entries per element) and
    the node rows of the whole K_e hold the same values, so the pipelined gather
    over either gives bitwise the same R, nzval and state -- with Dirichlet dofs,
    whose neighbourhoods the gather assembles in place -- and the pair path is
    held to the oracle at the FP64 bar."""
    torch = _torch()
    n = 9
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    if phys_name == "neohookean":
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        U = stretch_field(mesh.nodal_coords, seed=5).ravel()
    else:
        phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
        U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom")]

    def run():
        asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
        p = fec.create_parameters(mesh, asm, phys, dirichlet_bcs=bcs)
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        st = p.state_new.cpu().numpy().copy() if phys_name == "j2" else None
        return asm, R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), st

    asm, R, nz, st = run()
    with node_row_workspace():
        _, R_nr, nz_nr, st_nr = run()
    assert np.array_equal(R, R_nr) and np.array_equal(nz, nz_nr)
    if st is not None:
        assert np.array_equal(st, st_nr)
    ne = mesh.num_elements()
    st_old = np.zeros(7 * 8 * ne) if phys_name == "j2" else None
    st_new = None if st_old is None else np.zeros_like(st_old)
    Uo = np.zeros_like(U)   # the field the assembly saw: the Dirichlet dofs at their value 0
    Uo[asm.dof.unknown_dofs - 1] = U[asm.dof.unknown_dofs - 1]
    Ro, nzo, ab = _oracle(orc, mesh, asm, phys_name, phys.create_properties(), Uo, st_old, st_new)
    er = residual_err(R, Ro, ab) if st_old is None else rel_err(R, Ro)[:2]
    print("pair workspace", phys_name, "residual", er, "nzval", rel_err(nz, nzo))
    assert max(rel_err(nz, nzo)) <= TOL64 and max(er) <= TOL64
    if st is not None:
        assert max(rel_err(st, st_new)) <= TOL64


def test_poisson_block_gradients_match_per_element_map(fec, orc):
    """FP64 Poisson on a block of translated hex8 elements reads the block's
    spatial gradients and JxW (forming only the quadrature points' coordinates
    for the source term): residual and nzval within 1e-12 of the per-element map
    (FEC_HEX8_AFFINE=0) and of the oracle, and a different rounding of the
    per-element map (the path ran)."""
    torch = _torch()
    n = 12
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f) for f in ("left", "right", "bottom", "top")]

    def run():
        asm = fec.SparseMatrixAssembler(fec.ScalarFunction(fec.FunctionSpace(mesh), "u"), device=0)
        p = fec.create_parameters(mesh, asm, fec.Poisson(2.0), dirichlet_bcs=bcs)
        U = np.random.default_rng(7).uniform(-1.0, 1.0, mesh.num_nodes)
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        return asm, U, R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy()

    asm, U, R, nz = run()
    with per_element_kernels():
        _, _, R_pe, nz_pe = run()
    print("Poisson block gradients vs per-element map: residual", rel_err(R, R_pe), "nzval", rel_err(nz, nz_pe))
    assert max(rel_err(R, R_pe)) <= TOL64 and max(rel_err(nz, nz_pe)) <= TOL64
    assert not (np.array_equal(R, R_pe) and np.array_equal(nz, nz_pe))
    Uo = np.zeros_like(U)
    Uo[asm.dof.unknown_dofs - 1] = U[asm.dof.unknown_dofs - 1]
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "poisson", [2.0], Uo,
                                         asm.dof.dof_to_unknown, asm.dof.unknown_dofs)
    assert max(rel_err(nz, nzo)) <= TOL64 and max(rel_err(R, Ro)[:2]) <= TOL64
