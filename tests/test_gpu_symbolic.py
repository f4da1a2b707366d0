"""The symbolic phase on the device (fec_pattern_build_device) against the host
one (fec_pattern_build): the same colptr/rowval, and -- because the element
maps and adjacency are the same -- bitwise the same assembled values."""
import numpy as np
import pytest

from helpers import stretch_field

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _pair(fec, mesh, kind, physics, bcs=(), precision="fp64"):
    out = []
    for symbolic in ("host", "device"):
        V = fec.FunctionSpace(mesh)
        var = fec.ScalarFunction(V, "u") if kind == "scalar" else fec.VectorFunction(V, "u")
        asm = fec.SparseMatrixAssembler(var, device=0, precision=precision, symbolic=symbolic)
        p = fec.create_parameters(mesh, asm, physics, dirichlet_bcs=bcs)
        out.append((asm, p))
    return out


def _check(fec, pair, U):
    torch = _torch()
    (ah, ph), (ad, pd) = pair
    ch, rh = ah.pattern()
    cd, rd = ad.pattern()
    assert np.array_equal(ch, cd) and np.array_equal(rh, rd)
    cdd, rdd = ad.pattern_device()
    assert np.array_equal(cdd.cpu().numpy(), ch) and np.array_equal(rdd.cpu().numpy(), rh)
    chd, rhd = ah.pattern_device()  # the device fill from a host-built pattern
    assert np.array_equal(chd.cpu().numpy(), ch) and np.array_equal(rhd.cpu().numpy(), rh)
    res = []
    for asm, p in pair:
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        res.append((R.clone(), K.nzval.clone()))
    torch.cuda.synchronize()
    assert torch.equal(res[0][0], res[1][0]) and torch.equal(res[0][1], res[1][1])


def test_device_symbolic_hex8_vector_with_dirichlet(fec):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (7, 7, 7))
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom"),
           fec.DirichletBC("u_x", lambda X, t: 0.01, nodeset_name="right")]
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    pair = _pair(fec, mesh, "vector", phys, bcs)
    _check(fec, pair, stretch_field(mesh.nodal_coords, seed=3).ravel())


def test_device_symbolic_poisson_all_faces_fixed(fec, orc):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (6, 6, 6))
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f) for f in orc.HEX8_FACES]
    phys = fec.Poisson(1.0)
    pair = _pair(fec, mesh, "scalar", phys, bcs)
    rng = np.random.default_rng(0)
    _check(fec, pair, rng.uniform(-1, 1, mesh.num_nodes))


@pytest.mark.parametrize("kind", ["tet4", "tet10", "hex27"])
def test_device_symbolic_higher_order(fec, kind):
    gen = {"tet4": fec.meshes.box_tet4, "tet10": fec.meshes.box_tet10, "hex27": fec.meshes.box_hex27}[kind]
    mesh = gen((3, 4, 3))
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    pair = _pair(fec, mesh, "vector", phys)
    _check(fec, pair, stretch_field(mesh.nodal_coords, seed=2).ravel())


def test_device_symbolic_mixed_blocks(fec):
    from fec_gb300 import batching
    mesh = batching.mixed_mesh(2, 2, 2)
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    pair = _pair(fec, mesh, "vector", phys)
    _check(fec, pair, stretch_field(mesh.nodal_coords, seed=5).ravel())
