"""Batched uneven meshes in one launch, the mixed tet4/tet10/hex27 mesh, and the
CUDA-graph Newton loop (GPU, against the oracle and against eager execution)."""
import numpy as np
import pytest

from helpers import blocks_of, rel_err, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _system(fec, mesh, precision="fp64"):
    torch = _torch()
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0, precision=precision)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    p = fec.create_parameters(mesh, asm, phys)
    U = stretch_field(mesh.nodal_coords, seed=2).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    return asm, p, U, Uu, phys


def test_batch_of_uneven_meshes_matches_per_mesh_oracle(fec, orc):
    torch = _torch()
    from fec_gb300 import batching
    sides = [2, 5, 1, 3, 4]
    batch = batching.box_batch(sides)
    assert batch.mesh.element_block_names == ["block_1"]           # one block -> one launch per kernel
    asm, p, U, Uu, phys = _system(fec, batch.mesh)
    fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    assert asm.last_launch_count() == 2                             # element kernel + gather for all meshes
    for i, n in enumerate(sides):
        m = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
        n0, n1 = batch.node_offsets[i], batch.node_offsets[i + 1]
        Ui = U.reshape(-1, 3)[n0:n1].ravel()
        unknown, dtu = orc.update_dofs(3 * m.num_nodes, [])
        Ro, colptr, rowval, nzo = orc.assembled_system(blocks_of(m), m.nodal_coords, "neohookean",
                                                       phys.create_properties(), Ui, dtu, unknown)
        Ri, Ki = batching.mesh_system(asm, batch, i)
        assert np.array_equal(Ki.colptr, colptr) and np.array_equal(Ki.rowval, rowval)
        assert max(rel_err(Ri.cpu().numpy(), Ro)) <= TOL64
        assert max(rel_err(Ki.nzval.cpu().numpy(), nzo)) <= TOL64


def test_mixed_tet4_tet10_hex27_mesh(fec, orc):
    from fec_gb300 import batching
    mesh = batching.mixed_mesh(2, 2, 2)
    asm, p, U, Uu, phys = _system(fec, mesh)
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    Ro, colptr, rowval, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean",
                                                   phys.create_properties(), U, asm.dof.dof_to_unknown,
                                                   asm.dof.unknown_dofs)
    assert np.array_equal(K.colptr, colptr) and np.array_equal(K.rowval, rowval)
    assert max(rel_err(R.cpu().numpy(), Ro)) <= TOL64
    assert max(rel_err(K.nzval.cpu().numpy(), nzo)) <= TOL64


@pytest.mark.parametrize("precision", ["fp64", "fp32_element"])
def test_newton_loop_graph_replays_eager_bits(fec, precision):
    torch = _torch()
    from fec_gb300 import batching
    s1 = _system(fec, batching.box_batch([3, 6, 2]).mesh, precision)
    s2 = _system(fec, batching.mixed_mesh(2, 1, 1), precision)
    systems = [(s1[0], s1[1], s1[3]), (s2[0], s2[1], s2[3])]
    eager = batching.NewtonLoop(systems, iterations=5)
    eager.run_eager()
    torch.cuda.synchronize()
    graph = batching.NewtonLoop(systems, iterations=5).capture()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(eager.norms, graph.norms)
    for s in range(2):
        assert torch.equal(eager.unknowns(s), graph.unknowns(s))
    assert bool(torch.isfinite(graph.norms).all())
    # replaying again restarts from the captured inputs' current values: the loop advances
    graph.replay()
    torch.cuda.synchronize()
    assert not torch.equal(eager.unknowns(0), graph.unknowns(0))


def test_autotuned_generic_kernels_are_bitwise_identical(fec):
    """Every launch configuration the autotuner may pick for the tet4/tet10
    kernels (elements per CTA) gives bitwise the same residual and nzval, in FP64
    and FP32-element arithmetic; the tuned run reports its choices.  The tet10
    box is a block of translation classes, whose tensor-core kernel FEC_CLASS_TC=0
    switches off here so that the generic kernels run.  (Hex27 has its own
    kernels in both arithmetics: double-float in FP64, tensor cores in
    FP32-element; its generic configurations stay tunable behind
    FEC_HEX27_ON_CUDA_CORES=1 and FEC_FP64_CONTRACTION=native.)"""
    import os
    torch = _torch()
    from fec_gb300 import batching
    from helpers import stretch_field
    mesh = batching.mixed_mesh(3, 3, 2)
    results = {}
    os.environ["FEC_CLASS_TC"] = "0"
    try:
        _autotune_candidates(fec, torch, mesh, stretch_field, results)
    finally:
        os.environ.pop("FEC_CLASS_TC", None)
    report = fec.autotune_report()
    print("\n".join(report))
    assert any("tet4" in line for line in report) and any("tet10" in line for line in report)


def _autotune_candidates(fec, torch, mesh, stretch_field, results):
    import os
    for precision in ("fp64", "fp32_element"):
        for cand in ("0", "1", "2", None):
            if cand is None:
                os.environ.pop("FEC_AUTOTUNE_CANDIDATE", None)
            else:
                os.environ["FEC_AUTOTUNE_CANDIDATE"] = cand
            try:
                asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0,
                                                precision=precision)
                p = fec.create_parameters(mesh, asm, fec.NeoHookean.from_youngs(1.0, 0.3))
                U = stretch_field(mesh.nodal_coords, seed=2).ravel()
                Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
                R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
                torch.cuda.synchronize()
                results[(precision, cand)] = (R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy())
            finally:
                os.environ.pop("FEC_AUTOTUNE_CANDIDATE", None)
        ref = results[(precision, "0")]
        for cand in ("1", "2", None):
            assert np.array_equal(results[(precision, cand)][0], ref[0])
            assert np.array_equal(results[(precision, cand)][1], ref[1])


@pytest.mark.parametrize("physics", ["neohookean", "j2"])
def test_single_launch_matches_per_block_launches(fec, physics):
    """hex8 + tet4 + tet10 + hex27 blocks in ONE persistent element launch give
    bitwise the residual, nzval and state of one launch per block.  The single
    launch runs the per-element kernels, so the per-block launches do too
    (FEC_HEX8_AFFINE=0 and FEC_CLASS_TC=0: the structured hex8 block and the tet10
    box of translation classes would take their tensor-core kernels)."""
    import os
    torch = _torch()
    from fec_gb300 import batching
    from helpers import stretch_field
    mesh = fec.meshes.merge_meshes(
        [fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5)), fec.meshes.box_tet4((3, 3, 3)),
         fec.meshes.box_tet10((3, 3, 3)), fec.meshes.box_hex27((3, 3, 3))],
        names=["hex8", "tet4", "tet10", "hex27"])
    out = []
    os.environ["FEC_HEX8_AFFINE"] = "0"
    os.environ["FEC_CLASS_TC"] = "0"
    try:
        _single_vs_per_block(fec, torch, mesh, physics, stretch_field, out)
    finally:
        os.environ.pop("FEC_HEX8_AFFINE", None)
        os.environ.pop("FEC_CLASS_TC", None)
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    if physics == "j2":
        assert torch.equal(out[0][3], out[1][3])
    # element launches + the gather: one launch per group of nodes of one element size (four sizes here)
    assert out[0][2] == 4 + 4 and out[1][2] == 1 + 4


@pytest.mark.parametrize("physics", ["neohookean", "j2"])
def test_single_launch_with_class_tables_present(fec, physics):
    """With the tables of the structured hex8 block and the tet10 / hex27 boxes of
    translation classes present (the defaults), the single launch still runs the
    per-element kernels and its workspace is sized and laid out for whole element
    matrices: its results are bitwise those with the tables switched off, and within
    1e-12 of the per-block launches, which take the tensor-core and class kernels
    (symmetric-half workspaces)."""
    import os
    torch = _torch()
    mesh = fec.meshes.merge_meshes(
        [fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5)), fec.meshes.box_tet4((3, 3, 3)),
         fec.meshes.box_tet10((3, 3, 3)), fec.meshes.box_hex27((3, 3, 3))],
        names=["hex8", "tet4", "tet10", "hex27"])
    tables = []
    _single_vs_per_block(fec, torch, mesh, physics, stretch_field, tables)
    off = []
    os.environ["FEC_HEX8_AFFINE"] = "0"
    os.environ["FEC_CLASS_TC"] = "0"
    try:
        _single_vs_per_block(fec, torch, mesh, physics, stretch_field, off)
    finally:
        os.environ.pop("FEC_HEX8_AFFINE", None)
        os.environ.pop("FEC_CLASS_TC", None)
    (R_pb, nz_pb, _, st_pb), (R_1, nz_1, _, st_1) = tables
    assert torch.equal(R_1, off[1][0]) and torch.equal(nz_1, off[1][1])
    assert not torch.equal(nz_pb, off[0][1])   # (the per-block launches took the tensor-core kernels)
    e_r, e_k = rel_err(R_pb.cpu().numpy(), R_1.cpu().numpy()), rel_err(nz_pb.cpu().numpy(), nz_1.cpu().numpy())
    print(physics, "per-block (tables) vs single launch: residual", e_r, "nzval", e_k)
    assert max(e_r[:2]) <= TOL64 and max(e_k) <= TOL64
    if physics == "j2":
        assert torch.equal(st_1, off[1][3])
        assert max(rel_err(st_pb.cpu().numpy(), st_1.cpu().numpy())[:2]) <= TOL64


def _single_vs_per_block(fec, torch, mesh, physics, stretch_field, out):
    for single in (False, True):
        asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
        asm.set_single_launch(single)
        if physics == "neohookean":
            phys = fec.NeoHookean.from_youngs(1.0, 0.3)
            U = stretch_field(mesh.nodal_coords, seed=2).ravel()
        else:
            phys = fec.J2Plasticity(200.0, 0.3, 0.25, 2.0)
            U = 3.0 * stretch_field(mesh.nodal_coords, seed=2, noise=1e-4, diag=(1.004, 0.999, 0.999)).ravel()
        p = fec.create_parameters(mesh, asm, phys)
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        st = p.state_new.clone() if physics == "j2" else None
        out.append((R.clone(), K.nzval.clone(), asm.last_launch_count(), st))


def test_newton_loop_graph_with_single_launch(fec):
    """The CUDA-graph Newton loop over the tet4/tet10/hex27 system with all its
    element blocks in one persistent launch replays the eager loop bitwise, and
    both equal the loop with one launch per block (its per-element kernels:
    FEC_CLASS_TC=0 keeps the tet10 box off its tensor-core kernel)."""
    import os
    torch = _torch()
    os.environ["FEC_CLASS_TC"] = "0"
    try:
        _newton_single_vs_per_block(fec, torch)
    finally:
        os.environ.pop("FEC_CLASS_TC", None)


def _newton_single_vs_per_block(fec, torch):
    from fec_gb300 import batching
    runs = []
    for single in (False, True):
        asm, p, _, Uu, _ = _system(fec, batching.mixed_mesh(2, 1, 1))
        asm.set_single_launch(single)
        systems = [(asm, p, Uu)]
        eager = batching.NewtonLoop(systems, iterations=5)
        eager.run_eager()
        torch.cuda.synchronize()
        runs.append((eager.norms.clone(), eager.unknowns(0).clone(), asm.last_launch_count()))
        if single:
            graph = batching.NewtonLoop(systems, iterations=5).capture()
            graph.replay()
            torch.cuda.synchronize()
            assert torch.equal(eager.norms, graph.norms)
            assert torch.equal(eager.unknowns(0), graph.unknowns(0))
    assert torch.equal(runs[0][0], runs[1][0]) and torch.equal(runs[0][1], runs[1][1])
    assert bool(torch.isfinite(runs[1][0]).all())
    # element launches + the gather: one launch per group of nodes of one element size (three sizes here)
    assert runs[0][2] == 3 + 3 and runs[1][2] == 1 + 3
