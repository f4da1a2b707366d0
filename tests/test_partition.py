"""Partitioned assembly: the part/ghost bookkeeping on the host, the multi-rank
exchange with 2 gloo ranks (on CPU with the oracle's part values, the exchange
logic alone; and with each rank assembling its part through the library on the
GPU), and the one-GPU partitioned assembler against the single-part assembly."""
import os
import socket

import numpy as np
import pytest

from helpers import blocks_of, rel_err, stretch_field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _problem(fec, orc, nparts):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 5, 5))
    nn = mesh.num_nodes
    dd = 3 * (mesh.nodeset_nodes["left"] - 1) + 1          # u_x fixed on x = 0
    unknown, dtu = orc.update_dofs(3 * nn, dd)
    host = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=-1)
    fec.update_dofs(host.dof, dd)
    host._push_dofs()
    colptr, rowval = host.pattern()
    from fec_gb300 import partition
    parts = partition.build_parts(mesh, 3, dtu, nparts)
    for part in parts:
        partition.part_pattern(part, colptr, rowval)
    U = stretch_field(mesh.nodal_coords, seed=4).ravel()
    U[dd - 1] = 0.0
    return mesh, unknown, dtu, colptr, rowval, parts, U


def _local_values(orc, part, U, props):
    gdofs = (3 * (part.nodes[:, None] - 1) + np.arange(3)[None, :]).ravel()
    lunknown = np.nonzero(part.dof_to_unknown > 0)[0] + 1
    R, _, _, nz = orc.assembled_system(blocks_of(part.mesh), part.mesh.nodal_coords, "neohookean", props,
                                       U[gdofs], part.dof_to_unknown, lunknown)
    return R, nz


def test_parts_cover_elements_and_own_each_column_once(fec, orc):
    mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, 3)
    assert sum(p.elems[1] - p.elems[0] for p in parts) == mesh.num_elements()
    owned = np.concatenate([p.unknown_l2g[p.owned_cols] for p in parts])
    assert np.array_equal(np.sort(owned), np.arange(unknown.size))


def test_in_order_combination_matches_single_part(fec, orc):
    mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, 3)
    props = fec.NeoHookean.from_youngs(1.0, 0.3).create_properties()
    R = np.zeros(unknown.size)
    nz = np.zeros(rowval.size)
    for part in parts:
        Rl, nzl = _local_values(orc, part, U, props)
        R[part.unknown_l2g] += Rl
        nz[part.kmap] += nzl
    Ro, cp, rv, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean", props, U, dtu, unknown)
    assert np.array_equal(cp, colptr) and np.array_equal(rv, rowval)
    assert max(rel_err(R, Ro)) <= 1e-12 and max(rel_err(nz, nzo)) <= 1e-12


def _worker(rank, world, port, out_path):
    import sys
    sys.path[:0] = [os.path.join(ROOT, "finiteelementcontainers.jl_gb300"), ROOT, os.path.join(ROOT, "tests")]
    import torch.distributed as dist
    import fec_gb300 as fec
    from fec_gb300 import partition
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, world)
        props = fec.NeoHookean.from_youngs(1.0, 0.3).create_properties()
        part = parts[rank]
        Rl, nzl = _local_values(orc, part, U, props)
        cols, Rown, pos, nzown = partition.exchange_to_owners(part, Rl, nzl, rank, world, colptr)
        # collect everything on rank 0
        import torch
        R = torch.zeros(unknown.size, dtype=torch.float64)
        nz = torch.zeros(rowval.size, dtype=torch.float64)
        R[torch.from_numpy(cols)] = torch.from_numpy(Rown)
        nz[torch.from_numpy(pos)] = torch.from_numpy(nzown)
        dist.reduce(R, 0)
        dist.reduce(nz, 0)
        if rank == 0:
            np.savez(out_path, R=R.numpy(), nz=nz.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_exchange_gloo(fec, orc, tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, 2)
    props = fec.NeoHookean.from_youngs(1.0, 0.3).create_properties()
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean", props, U, dtu, unknown)
    assert max(rel_err(got["R"], Ro)) <= 1e-12 and max(rel_err(got["nz"], nzo)) <= 1e-12
    # identical to the one-process, in-order combination of the same parts
    R = np.zeros(unknown.size)
    nz = np.zeros(rowval.size)
    for part in parts:
        Rl, nzl = _local_values(orc, part, U, props)
        R[part.unknown_l2g] += Rl
        nz[part.kmap] += nzl
    assert np.array_equal(got["R"], R) and np.array_equal(got["nz"], nz)


@pytest.mark.gpu
@pytest.mark.parametrize("nparts", [2, 4])
def test_partitioned_assembler_on_one_gpu(fec, orc, nparts):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fec_gb300 import partition
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (9, 9, 9))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom")]
    pa = partition.PartitionedAssembler(mesh, phys, nparts, dirichlet_bcs=bcs)
    single = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    p = fec.create_parameters(mesh, single, phys, dirichlet_bcs=bcs)
    assert np.array_equal(single.dof.dof_to_unknown, pa.dof.dof_to_unknown)
    U = stretch_field(mesh.nodal_coords, seed=6).ravel()
    Uu = torch.from_numpy(U[single.dof.unknown_dofs - 1].copy()).cuda()
    R1, K1 = fec.assemble_residual_and_stiffness(single, Uu, p)
    R2, nz2 = pa.assemble(Uu)
    torch.cuda.synchronize()
    assert np.array_equal(K1.colptr, pa.colptr) and np.array_equal(K1.rowval, pa.rowval)
    assert max(rel_err(R2.cpu().numpy(), R1.cpu().numpy())) <= 1e-12
    assert max(rel_err(nz2.cpu().numpy(), K1.nzval.cpu().numpy())) <= 1e-12


def _gpu_worker(rank, world, port, out_path):
    """One rank: its part assembled through the product path on the GPU (each
    rank its own process and context on device 0, no kernel waits on another
    rank), then the host exchange to the owners over gloo."""
    import sys
    sys.path[:0] = [os.path.join(ROOT, "finiteelementcontainers.jl_gb300"), ROOT, os.path.join(ROOT, "tests")]
    import torch
    import torch.distributed as dist
    import fec_gb300 as fec
    from fec_gb300 import partition
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, world)
        part = parts[rank]
        asm, p = partition.local_assembler(part, fec.NeoHookean.from_youngs(1.0, 0.3), np.zeros(U.size), colptr,
                                           rowval, device=0)
        Uu = torch.from_numpy(U[unknown - 1][part.unknown_l2g].copy()).cuda()
        R_l, K_l = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        cols, Rown, pos, nzown = partition.exchange_to_owners(part, R_l.cpu().numpy(), K_l.nzval.cpu().numpy(),
                                                              rank, world, colptr)
        R = torch.zeros(unknown.size, dtype=torch.float64)
        nz = torch.zeros(rowval.size, dtype=torch.float64)
        R[torch.from_numpy(cols)] = torch.from_numpy(Rown)
        nz[torch.from_numpy(pos)] = torch.from_numpy(nzown)
        dist.reduce(R, 0)
        dist.reduce(nz, 0)
        if rank == 0:
            np.savez(out_path, R=R.numpy(), nz=nz.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_two_rank_exchange_of_gpu_assembled_parts(fec, orc, tmp_path):
    """2 gloo ranks, each assembling its part with the library on the GPU: the
    exchanged global residual and CSC values against the oracle's single-part
    assembly (<= 1e-12), and bitwise the one-GPU partitioned assembler's."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import torch.multiprocessing as mp
    from fec_gb300 import partition
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_gpu_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    mesh, unknown, dtu, colptr, rowval, parts, U = _problem(fec, orc, 2)
    props = fec.NeoHookean.from_youngs(1.0, 0.3).create_properties()
    Ro, _, _, nzo = orc.assembled_system(blocks_of(mesh), mesh.nodal_coords, "neohookean", props, U, dtu, unknown)
    assert max(rel_err(got["R"], Ro)) <= 1e-12 and max(rel_err(got["nz"], nzo)) <= 1e-12
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left")]
    pa = partition.PartitionedAssembler(mesh, fec.NeoHookean.from_youngs(1.0, 0.3), 2, dirichlet_bcs=bcs)
    assert np.array_equal(pa.dof.dof_to_unknown, dtu)
    R2, nz2 = pa.assemble(torch.from_numpy(U[unknown - 1].copy()).cuda())
    assert np.array_equal(got["R"], R2.cpu().numpy()) and np.array_equal(got["nz"], nz2.cpu().numpy())
