"""Parity at the configured sizes of the two remaining workloads:

  * J2 plasticity on the 96^3 hex8 box (884,736 elements) along the whole
    20-step uniaxial load path to 1% strain.  The oracle carries its state
    along the path.  At every step the library assembles from the oracle's old
    state (the same inputs), and the full residual over the unknowns, every
    quadrature point's new state and sampled CSC columns are compared entry by
    entry; and the library also runs the path carrying its own state, compared
    normwise (two FP64 state paths drift apart at the rounding level of the
    return map, amplified by E / sigma_y, so their residuals agree to ~1e-14 of
    the element forces rather than of each entry);
  * the batched workload: the 64 hex8 Neo-Hookean meshes of 8^3 to 48^3
    elements (seed 2) in one block, and the tet4 + tet10 + hex27 mesh of
    196,608 + 196,608 + 97,336 elements: per mesh (and per block) the full
    residual entry by entry, sampled columns of every mesh, and each mesh's
    entry count against the closed form of its 27-point coupling.

Bars: FP64 within 1e-12 entry-wise and normwise (tests/helpers.py: matrix
entries with an absolute floor of 1e-14 of the largest entry, residual entries
with a floor of 1e-14 of the element forces each one sums)."""
import numpy as np
import pytest

from helpers import blocks_of, compare_sampled_columns, rel_err, residual_err, sampled_columns, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
J2_PROPS = [200.0, 0.3, 0.25, 2.0]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_j2_96cubed_full_load_path(fec, orc):
    torch = _torch()
    from fec_gb300.workloads import uniaxial_bcs, uniaxial_inputs
    n = 96
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    phys = fec.J2Plasticity(*J2_PROPS)
    p = fec.create_parameters(mesh, asm, phys, dirichlet_bcs=uniaxial_bcs())
    inputs = uniaxial_inputs(mesh.nodal_coords, asm.dof.unknown_dofs, p.bc_dofs.cpu().numpy(), 20)
    blocks = blocks_of(mesh)
    X = mesh.nodal_coords
    ne = mesh.num_elements()
    assert ne == 884_736
    props = phys.create_properties()
    threads = orc.max_threads()
    rng = np.random.default_rng(11)
    # sampled nodes: random, the corners, and nodes on the loaded and the symmetry faces
    faces = [mesh.nodeset_nodes[f] - 1 for f in ("left", "right", "bottom", "back")]
    nodes = np.unique(np.concatenate([rng.integers(0, mesh.num_nodes, 16), [0, mesh.num_nodes - 1]] +
                                     [f[rng.integers(0, f.size, 3)] for f in faces]))
    st_o = np.zeros(7 * 8 * ne)
    free = [torch.zeros_like(p.state_old), torch.zeros_like(p.state_old)]   # the library's own state path
    R_abs = np.empty(3 * mesh.num_nodes)
    unknown = asm.dof.unknown_dofs - 1
    plastic = []
    for step, (Uu, bc) in enumerate(inputs, start=1):
        p.bc_vals = torch.from_numpy(bc).cuda()
        Uu_d = torch.from_numpy(Uu).cuda()
        # (1) from the oracle's old state: every output entry by entry
        p.state_old.copy_(torch.from_numpy(st_o))
        R, K = fec.assemble_residual_and_stiffness(asm, Uu_d, p)
        torch.cuda.synchronize()
        U = p.field.cpu().numpy()          # the full field the kernels read (unknowns + Dirichlet values)
        sn_o = np.zeros_like(st_o)
        Rf, _ = orc.assemble(blocks, X, "j2", props, U, st_o, sn_o, want_k=False, threads=threads, abs_out=R_abs)
        e_r = residual_err(R.cpu().numpy(), Rf[unknown], R_abs[unknown])
        e_s = rel_err(p.state_new.cpu().numpy(), sn_o)
        cols, res = sampled_columns(orc, blocks, X, U, "j2", props, nodes, asm.dof.dof_to_unknown, 3, [st_o])
        e_k, e_rs = compare_sampled_columns(K, K.nzval, R, cols, res)
        # (2) carrying its own state: normwise
        saved = (p.state_old, p.state_new)
        p.state_old, p.state_new = free
        Rfree, Kfree = fec.assemble_residual_and_stiffness(asm, Uu_d, p)
        torch.cuda.synchronize()
        e_free = {"residual": rel_err(Rfree.cpu().numpy(), Rf[unknown]),
                  "state": rel_err(p.state_new.cpu().numpy(), sn_o)}
        p.state_old, p.state_new = saved
        free.reverse()
        plastic.append(int((sn_o[6::7] > 0).sum()))
        print(f"step {step:2d}: plastic points {plastic[-1]:7d}  residual {e_r}  state {e_s}  "
              f"sampled columns {e_k}  own state path {e_free}")
        assert max(e_r) <= TOL64, (step, e_r)
        assert max(e_s) <= TOL64, (step, e_s)
        assert max(e_k) <= TOL64, (step, e_k)
        assert max(e_rs[:2]) <= TOL64, (step, e_rs)
        assert max(e_free["residual"][:2]) <= TOL64 and max(e_free["state"][:2]) <= TOL64, (step, e_free)
        st_o = sn_o
    # the nodal noise (N(0, 1e-5^2) at h = 1/96, a strain noise near the yield strain 1.25e-3) makes most
    # points yield from the first step; all of them yield by the end of the path
    assert plastic[-1] == 8 * ne


def test_batched_64_meshes_and_mixed_mesh_full_size(fec, orc):
    torch = _torch()
    from fec_gb300 import batching
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    props = phys.create_properties()
    threads = orc.max_threads()
    sides = batching.lognormal_cube_sides()
    assert len(sides) == 64 and min(sides) >= 8 and max(sides) <= 48
    systems = {"batch64": batching.box_batch(sides), "mixed": None}
    mixed = batching.mixed_mesh(32, 32, 46)
    for name, mesh in (("batch64", systems["batch64"].mesh), ("mixed", mixed)):
        asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
        p = fec.create_parameters(mesh, asm, phys)
        U = stretch_field(mesh.nodal_coords, seed=2).ravel()
        R, K = fec.assemble_residual_and_stiffness(asm, torch.from_numpy(U.copy()).cuda(), p)
        torch.cuda.synchronize()
        blocks = blocks_of(mesh)
        X = mesh.nodal_coords
        R_abs = np.empty(U.size)
        Rf, _ = orc.assemble(blocks, X, "neohookean", props, U, want_k=False, threads=threads, abs_out=R_abs)
        Rg = R.cpu().numpy()
        rng = np.random.default_rng(5)
        if name == "batch64":
            batch = systems["batch64"]
            assert mesh.num_elements() == sum(s ** 3 for s in sides)
            worst_r = worst_k = 0.0
            nodes = []
            for i, s in enumerate(sides):
                n0, n1 = int(batch.node_offsets[i]), int(batch.node_offsets[i + 1])
                # each mesh's own residual entry by entry, and its entry count: 9 (3 s + 1)^3
                e = residual_err(Rg[3 * n0:3 * n1], Rf[3 * n0:3 * n1], R_abs[3 * n0:3 * n1])
                worst_r = max(worst_r, max(e))
                assert int(K.colptr[3 * n1] - K.colptr[3 * n0]) == 9 * (3 * s + 1) ** 3
                nodes += [n0, n1 - 1] + rng.integers(n0, n1, 2).tolist()
            cols, res = sampled_columns(orc, blocks, X, U, "neohookean", props, np.unique(nodes),
                                        asm.dof.dof_to_unknown, 3)
            e_k, e_rs = compare_sampled_columns(K, K.nzval, R, cols, res)
            print(f"batch of 64 meshes ({mesh.num_elements()} elements): worst per-mesh residual {worst_r:.3e}, "
                  f"sampled columns {e_k}")
            assert worst_r <= TOL64 and max(e_k) <= TOL64 and max(e_rs[:2]) <= TOL64
        else:
            counts = [c.shape[0] for _, c in blocks]
            assert counts == [196_608, 196_608, 97_336]
            # per block: the block's nodes (the blocks share none) entry by entry
            nodes = []
            for (et, conns) in blocks:
                bn = np.unique(conns) - 1
                e = residual_err(Rg.reshape(-1, 3)[bn].ravel(), Rf.reshape(-1, 3)[bn].ravel(),
                                 R_abs.reshape(-1, 3)[bn].ravel())
                print(f"mixed mesh, {et} block ({conns.shape[0]} elements): residual {e}")
                assert max(e) <= TOL64
                nodes += bn[rng.integers(0, bn.size, 6)].tolist()
            cols, res = sampled_columns(orc, blocks, X, U, "neohookean", props, np.unique(nodes),
                                        asm.dof.dof_to_unknown, 3)
            e_k, e_rs = compare_sampled_columns(K, K.nzval, R, cols, res)
            print(f"mixed mesh sampled columns {e_k}")
            assert max(e_k) <= TOL64 and max(e_rs[:2]) <= TOL64
        del asm, p, R, K
        torch.cuda.empty_cache()
