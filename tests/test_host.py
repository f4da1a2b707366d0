"""Host-side logic of the product (no GPU): meshes, DOF numbering, the symbolic
phase of libfec_gb300.so through a host-only context, the ABI surface and its
error paths."""
import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

from helpers import blocks_of

ROOT = Path(__file__).resolve().parents[1]
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("n", [2, 3, 5, 9])
def test_structured_hex8_matches_oracle(fec, orc, n):
    m = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    coords, conns = orc.structured_hex8((n, n, n))
    assert np.array_equal(m.nodal_coords, coords)
    assert np.array_equal(m.element_conns["block_1"], conns)
    for face in orc.HEX8_FACES:
        assert np.array_equal(m.nodeset_nodes[face], orc.hex8_nodeset((n, n, n), face))


def test_structured_quad4_known_answer(fec):
    ka = json.loads((GOLD / "known_answers.json").read_text())["structured_quad4_3x3"]
    m = fec.StructuredMesh("quad", (0.0, 0.0), (1.0, 1.0), (3, 3))
    assert np.array_equal(m.nodal_coords.T, np.array(ka["coords"]))
    assert np.array_equal(m.element_conns["block_1"].T, np.array(ka["conns"]))


def test_structured_mesh_bad_input(fec):
    """test/TestMesh.jl: bad element name -> ArgumentError, zero-length side -> BoundsError."""
    with pytest.raises(fec.ArgumentError):
        fec.StructuredMesh("bad element", (0.0, 0.0), (1.0, 1.0), (3, 3))
    with pytest.raises(IndexError):
        fec.StructuredMesh("quad", (0.0, 0.0), (0.0, 1.0), (3, 3))


def test_connectivity_known_answer(fec):
    """test/TestFields.jl: flat multi-block connectivity slices."""
    ka = json.loads((GOLD / "known_answers.json").read_text())["connectivity"]
    b1 = np.array(ka["block_1"], dtype=np.int64).T
    b2 = np.array(ka["block_2"], dtype=np.int64).T
    coords = np.zeros((27, 2))
    mesh = fec.UnstructuredMesh(coords, {"a": ("QUAD4", b1), "b": ("QUAD4", np.c_[b2, b2[:, :1]])})
    V = fec.FunctionSpace(mesh)
    assert V.conn_offsets.tolist() == [1, 13]
    assert V.connectivity(1).shape == (3, 4)
    for blk, e, off, vals in ka["slices"]:
        if blk != 1:
            continue
        base = off + (e - 1) * 4
        assert V.conn_data[base - 1:base + 3].tolist() == vals


def test_dofmanager_size_known_answer(fec):
    """test/TestDofManagers.jl:17-27: a vector function on poisson.g has size (2, 16641)."""
    ka = json.loads((GOLD / "known_answers.json").read_text())["dofmanager_vector_poisson_g"]
    g = np.load(GOLD / "poisson_quad4.npz")
    mesh = fec.UnstructuredMesh(g["coords"], {"block_1": ("QUAD4", g["conn"])})
    dof = fec.DofManager(fec.VectorFunction(fec.FunctionSpace(mesh), "u"))
    assert list(dof.shape) == ka and len(dof) == ka[0] * ka[1]


def test_update_dofs_matches_oracle(fec, orc):
    n = 6
    m = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    u = fec.VectorFunction(fec.FunctionSpace(m), "u")
    dof = fec.DofManager(u)
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom"),
           fec.DirichletBC("u_z", lambda X, t: 0.0, nodeset_name="back")]
    dd = fec.dirichlet_dofs(bcs, m, dof)
    fec.update_dofs(dof, dd)
    ud, dtu = orc.update_dofs(len(dof), dd)
    assert np.array_equal(dof.unknown_dofs, ud) and np.array_equal(dof.dof_to_unknown, dtu)


def _pattern_case(fec, orc, mesh, var_kind, bcs):
    V = fec.FunctionSpace(mesh)
    var = fec.ScalarFunction(V, "u") if var_kind == "scalar" else fec.VectorFunction(V, "u")
    asm = fec.SparseMatrixAssembler(var, device=-1)
    fec.update_dofs_bcs(asm, bcs)
    colptr, rowval = asm.pattern()
    nf = asm.dof.nf
    Is, Js, _ = orc.pattern(blocks_of(mesh), nf, asm.dof.dof_to_unknown)
    n = asm.dof.unknown_dofs.size
    cp, rv, _ = orc.sparse_csc(n, n, Is, Js, np.ones(Is.size))
    assert np.array_equal(colptr, cp)
    assert np.array_equal(rowval, rv)
    return asm


def test_pattern_scalar_hex8_all_faces_dirichlet(fec, orc):
    """Configuration of the Poisson workload (all six faces fixed) at 8^3: colptr/rowval bit-exact."""
    m = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (9, 9, 9))
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f) for f in orc.HEX8_FACES]
    asm = _pattern_case(fec, orc, m, "scalar", bcs)
    assert asm.dof.unknown_dofs.size == 7 ** 3


def test_pattern_vector_hex8_partial_dirichlet(fec, orc):
    m = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (5, 6, 5))
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_z", lambda X, t: 0.0, nodeset_name="front")]
    _pattern_case(fec, orc, m, "vector", bcs)


def test_pattern_mixed_blocks(fec, orc):
    meshes = [fec.meshes.box_tet4((3, 3, 3)), fec.meshes.box_tet10((3, 3, 3)), fec.meshes.box_hex27((3, 3, 3)),
              fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (4, 4, 4))]
    m = fec.meshes.merge_meshes(meshes)
    _pattern_case(fec, orc, m, "vector", [])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pattern_random_shared_blocks_and_dirichlet(fec, orc, seed):
    """hex8 and tet4 blocks cut from the same node grid (so the blocks share nodes),
    in either block order, with random per-component Dirichlet node sets: colptr/rowval
    bit-exact against the oracle's element-ordered COO + sparse!, scalar and vector."""
    rng = np.random.default_rng(seed)
    counts = (5, 4, 5)  # counts[0] == counts[2]: the reference's coordinate loop swaps their bounds
    hexm = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), counts)
    tets = fec.meshes.box_tet4(counts)
    assert np.array_equal(tets.nodal_coords, hexm.nodal_coords)
    h = hexm.element_conns["block_1"]
    t = tets.element_conns["block_1"]
    keep_h = rng.random(h.shape[0]) < 0.5
    keep_t = np.repeat(~keep_h, 6)  # the tets of the other hexes
    blocks = {"hexes": ("HEX8", h[keep_h]), "tets": ("TETRA4", t[keep_t])}
    if seed % 2:
        blocks = dict(reversed(list(blocks.items())))
    nn = hexm.nodal_coords.shape[0]
    sets = {f"s{k}": np.sort(rng.choice(np.arange(1, nn + 1), size=int(rng.integers(1, nn // 3)), replace=False))
            for k in range(3)}
    mesh = fec.UnstructuredMesh(hexm.nodal_coords, blocks, nodesets=sets)
    _pattern_case(fec, orc, mesh, "scalar", [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name="s0")])
    comps = ["u_x", "u_y", "u_z"]
    bcs = [fec.DirichletBC(comps[int(rng.integers(0, 3))], lambda X, t: 0.0, nodeset_name=f"s{k}") for k in range(3)]
    _pattern_case(fec, orc, mesh, "vector", bcs)


def test_pattern_quad4_gold_mesh(fec, orc):
    g = np.load(GOLD / "poisson_quad4.npz")
    mesh = fec.UnstructuredMesh(g["coords"], {"block_1": ("QUAD4", g["conn"])},
                                nodesets={f"nset_{i}": g[f"nset_{i}"] for i in range(1, 5)})
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f"nset_{i}") for i in range(1, 5)]
    _pattern_case(fec, orc, mesh, "scalar", bcs)


def test_abi_exports_every_declared_symbol(fec):
    header = (ROOT / "include" / "fec_gb300.h").read_text()
    declared = set(re.findall(r"^int (fec_\w+)\(", header, re.M))
    lib = fec.load_library()
    from fec_gb300 import _lib
    assert declared == set(_lib.SIGNATURES)
    for name in declared:
        assert hasattr(lib, name)


def test_abi_error_paths_host_only(fec):
    from fec_gb300 import _lib
    lib = fec.load_library()
    h = C.c_void_p()
    assert lib.fec_ctx_create(-1, C.byref(h)) == 0
    try:
        coords = np.zeros((8, 3))
        types = np.array([1], dtype=np.int32)
        ne = np.array([1], dtype=np.int64)
        bad = np.array([1, 2, 3, 4, 5, 6, 7, 9], dtype=np.int64)   # node 9 does not exist
        st = lib.fec_mesh_set(h, 3, 8, coords.ctypes.data, 1, types.ctypes.data, ne.ctypes.data, bad.ctypes.data)
        assert st == _lib.FEC_ERR_ARG and "outside" in _lib.last_error(lib, h)
        rep = np.array([1, 2, 3, 4, 5, 6, 7, 7], dtype=np.int64)   # repeated node
        st = lib.fec_mesh_set(h, 3, 8, coords.ctypes.data, 1, types.ctypes.data, ne.ctypes.data, rep.ctypes.data)
        assert st == _lib.FEC_ERR_ARG and "repeats" in _lib.last_error(lib, h)
        good = np.arange(1, 9, dtype=np.int64)
        assert lib.fec_mesh_set(h, 3, 8, coords.ctypes.data, 1, types.ctypes.data, ne.ctypes.data,
                                good.ctypes.data) == 0
        nnz = C.c_int64()
        assert lib.fec_pattern_build(h, C.byref(nnz)) == _lib.FEC_ERR_STATE
        dtu = np.array([1, 2, -1, 4, 5, 6, 7, 8], dtype=np.int64)  # not consecutive
        assert lib.fec_dofs_set(h, 1, dtu.ctypes.data, 7) == _lib.FEC_ERR_ARG
        dtu = np.array([1, 2, -1, 3, 4, 5, 6, 7], dtype=np.int64)
        assert lib.fec_dofs_set(h, 1, dtu.ctypes.data, 7) == 0
        assert lib.fec_pattern_build(h, C.byref(nnz)) == 0 and nnz.value == 49
        st = lib.fec_assemble(h, 3, 0, 0.0, 0.0, None, None, None, None, None, None, None)
        assert st == _lib.FEC_ERR_STATE and "host-only" in _lib.last_error(lib, h)
        # every device entry point refuses a host-only context instead of touching a GPU
        bad_index = C.c_int64()
        assert lib.fec_check_finite(h, None, None, C.byref(bad_index), None) == _lib.FEC_ERR_STATE
        assert lib.fec_assemble_action(h, 0, 0.0, 0.0, None, None, None, None, None) == _lib.FEC_ERR_STATE
        it, rr = C.c_int(), C.c_double()
        assert lib.fec_cg_solve(h, None, None, None, 10, 1e-8, 0, C.byref(it), C.byref(rr), None) == \
            _lib.FEC_ERR_STATE
        props = np.array([1.0])
        assert lib.fec_physics_set(h, 2, 1, props.ctypes.data, 1) == _lib.FEC_ERR_ARG
        assert lib.fec_physics_set(h, 1, 99, props.ctypes.data, 1) == _lib.FEC_ERR_UNSUPPORTED
        # device outputs of the pattern: NULL is refused before any device work
        st = lib.fec_pattern_get_device(h, None, None, None)
        assert st == _lib.FEC_ERR_ARG and "NULL" in _lib.last_error(lib, h)
        cp = C.c_void_p(16)  # never dereferenced: a host-only context refuses next
        assert lib.fec_pattern_get_device(h, cp, cp, None) == _lib.FEC_ERR_STATE
        assert lib.fec_set_single_launch(h, 1) == 0 and lib.fec_set_single_launch(None, 1) == _lib.FEC_ERR_ARG
    finally:
        lib.fec_ctx_destroy(h)


def test_product_fails_loudly_without_library(fec, tmp_path):
    from fec_gb300 import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(tmp_path / "missing.so")


def test_batch_numbering(fec):
    from fec_gb300 import batching
    sides = batching.lognormal_cube_sides()
    assert len(sides) == 64 and min(sides) >= 8 and max(sides) <= 48
    batch = batching.box_batch([2, 3, 1])
    m = batch.mesh
    assert m.element_block_names == ["block_1"]
    assert batch.node_offsets.tolist() == [0, 27, 91, 99]
    assert batch.elem_offsets.tolist() == [0, 8, 35, 36]
    conn = m.element_conns["block_1"]
    # every element's nodes stay inside its own mesh's node range
    for i in range(3):
        c = conn[batch.elem_offsets[i]:batch.elem_offsets[i + 1]]
        assert c.min() > batch.node_offsets[i] and c.max() <= batch.node_offsets[i + 1]


def test_closure_rows_of_exact_return_map_are_consistent(orc):
    """The closure's training rows rebuilt from the oracle's return map: the exact
    targets lie on the updated yield surface and give back the oracle's stress."""
    import torch
    from fec_gb300 import closure
    props = [200.0, 0.3, 0.25, 2.0]
    rng = np.random.default_rng(5)
    n = 64
    eps = rng.normal(0, 0.001, (n, 6)) * rng.uniform(0.2, 1.5, (n, 1))   # both sides of the yield surface
    st = np.concatenate([rng.normal(0, 5e-5, (n, 6)), rng.uniform(0, 2e-4, (n, 1))], 1)
    ii, jj = [0, 1, 2, 1, 0, 0], [0, 1, 2, 2, 2, 1]
    sig, new = np.zeros((n, 6)), np.zeros((n, 7))
    for k in range(n):
        gu = np.zeros((3, 3))
        for m in range(6):
            gu[ii[m], jj[m]] = gu[jj[m], ii[m]] = eps[k, m]
        P, _, sn = orc.j2_update(gu, props, st[k])
        sig[k] = [P[ii[m] + 3 * jj[m]] for m in range(6)]
        new[k] = sn
    X, Y = closure.sample_rows(props, *(torch.from_numpy(a) for a in (eps, st, sig, new)))
    plastic = X[:, 13] > 0
    assert 0 < int(plastic.sum()) < n
    res = closure.consistency_residual(props, X[plastic], Y[plastic])
    assert float(res.max()) <= 1e-12
    s = closure.deviatoric_stress(props, X, Y) + closure.pressure(props, X[:, :6]) * torch.tensor(
        [1.0, 1, 1, 0, 0, 0], dtype=torch.float64)
    assert np.allclose(s.numpy(), sig, rtol=0, atol=1e-14)
