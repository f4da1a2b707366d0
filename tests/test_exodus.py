"""Exodus II mesh and nodal-field I/O (src/meshes/Exodus.jl, src/PostProcessors.jl):
a write/read round trip, and -- where the reference checkout is present -- its
own mesh and gold files read back against the committed fixtures."""
import os
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
# the reference checkout, when FEC_REFERENCE_DIR names one (its files are read only by the test below)
REF = Path(os.environ["FEC_REFERENCE_DIR"]) if os.environ.get("FEC_REFERENCE_DIR") else None


def test_round_trip_mesh_sets_and_fields(fec, tmp_path):
    hexes = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 2.0, 3.0), (4, 4, 4))
    tets = fec.meshes.box_tet10((2, 2, 2))
    for mesh in (hexes, tets):
        path = tmp_path / "out.exo"
        rng = np.random.default_rng(3)
        u = rng.standard_normal((mesh.num_nodes, 3))
        with fec.ExodusPostProcessor(mesh, path, ["u_x", "u_y", "u_z", "p"]) as pp:
            for k, t in enumerate((0.0, 0.5), start=1):
                pp.write_times(k, t)
                pp.write_field(k, ["u_x", "u_y", "u_z"], (k * u).ravel())
                pp.write_field(k, "p", u[:, 0] - k)
        back = fec.read_exodus(path)
        assert np.array_equal(back.nodal_coords, mesh.nodal_coords)
        assert back.element_block_names == mesh.element_block_names
        for b in mesh.element_block_names:
            assert back.element_types[b] == mesh.element_types[b]
            assert np.array_equal(back.element_conns[b], mesh.element_conns[b])
        assert sorted(back.nodeset_nodes) == sorted(mesh.nodeset_nodes)
        for s in mesh.nodeset_nodes:
            assert np.array_equal(back.nodeset_nodes[s], mesh.nodeset_nodes[s])
        with fec.ExodusFile(path) as f:
            assert f.nodal_variable_names() == ["u_x", "u_y", "u_z", "p"]
            assert np.array_equal(f.times(), [0.0, 0.5])
            for k in (1, 2):
                assert np.array_equal(f.nodal_variable("u_y", k), k * u[:, 1])
                assert np.array_equal(f.nodal_variable("p", k), u[:, 0] - k)


def _ref(rel: str) -> Path:
    if REF is None:
        pytest.skip("FEC_REFERENCE_DIR does not name a reference checkout")
    p = REF / rel
    if not p.exists():
        pytest.skip("reference checkout not present")
    return p


def test_reference_poisson_mesh_and_gold(fec):
    """test/poisson/poisson.g and poisson.gold read back equal the committed fixture
    (made from the same files); the side sets sset_1..4 that TestPoisson.jl:66-69 fixes
    cover exactly the node sets nset_1..4."""
    g = np.load(GOLD / "poisson_quad4.npz")
    mesh = fec.read_exodus(_ref("test/poisson/poisson.g"))
    assert mesh.element_types == {"block_1": "QUAD4"}
    assert np.array_equal(mesh.nodal_coords, g["coords"])
    assert np.array_equal(mesh.element_conns["block_1"], g["conn"])
    for i in range(1, 5):
        assert np.array_equal(mesh.nodeset_nodes[f"nset_{i}"], g[f"nset_{i}"])
        assert np.array_equal(mesh.sideset_nodes[f"sset_{i}"], np.unique(g[f"nset_{i}"]))
    with fec.ExodusFile(_ref("test/poisson/poisson.gold")) as f:
        assert f.nodal_variable_names() == ["u"]
        assert np.array_equal(f.nodal_variable("u", len(f.times())), g["u_gold"])


def test_reference_multi_block_meshes(fec):
    mesh = fec.read_exodus(_ref("test/poisson/multi_block_mesh_quad4_quad4.g"))
    assert mesh.element_block_names == ["block_1", "block_2"]
    for b in mesh.element_block_names:
        c = mesh.element_conns[b]
        assert c.shape[1] == 4 and c.min() >= 1 and c.max() <= mesh.num_nodes
    with pytest.raises(fec.ArgumentError, match="TRI3"):
        fec.read_exodus(_ref("test/poisson/multi_block_mesh_quad4_tri3.g"))
