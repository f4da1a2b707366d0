"""fec_assemble_noalloc: assembly for callers that cannot let the library
allocate device memory (their device memory all goes through their own pool,
or their device-memory budget is fixed up front).

The entry point is called through the C ABI and must reproduce fec_assemble,
the allocating entry point, on two calls in a row (the second with a different
displacement, so a stale workspace would show), and must refuse a mesh whose
element workspace does not fit its static array.  This file is collected last
so that a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_err, stretch_field

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _ptr(t):
    return None if t is None else t.data_ptr()


def _setup(fec, n, physics):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    V = fec.FunctionSpace(mesh)
    var = fec.VectorFunction(V, "u") if physics.NF == 3 else fec.ScalarFunction(V, "u")
    asm = fec.SparseMatrixAssembler(var, device=0)
    bcs = [] if physics.NF == 3 else [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name="left")]
    p = fec.create_parameters(mesh, asm, physics, dirichlet_bcs=bcs)
    return mesh, asm, p


def _noalloc(fec, asm, p, precision):
    """Same inputs as the last fec_assemble call, outputs into fresh tensors."""
    torch = _torch()
    lib = fec.load_library()
    R = torch.full((asm.dof.unknown_dofs.size,), float("nan"), dtype=torch.float64, device="cuda")
    nz = torch.full((asm.nnz,), float("nan"), dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    has_state = any(ph.NS for ph in p.physics)
    st = lib.fec_assemble_noalloc(asm._ctx, 3, precision, p.t, p.dt, _ptr(p.field), _ptr(p.field_old),
                                  _ptr(p.state_old) if has_state else None,
                                  _ptr(p.state_new) if has_state else None, _ptr(R), _ptr(nz), stream)
    from fec_gb300 import _lib
    _lib.check(lib, asm._ctx, st)
    torch.cuda.synchronize()
    return R.cpu().numpy(), nz.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_element"])
def test_noalloc_matches_allocating_entry_point_twice(fec, precision):
    torch = _torch()
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    mesh, asm, p = _setup(fec, 9, phys)
    prec = "fp64" if precision == 0 else "fp32_element"
    for seed in (11, 12):   # two calls in a row, different inputs
        U = stretch_field(mesh.nodal_coords, seed=seed).ravel()
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=prec)
        torch.cuda.synchronize()
        R_ref, nz_ref = R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy()
        R2, nz2 = _noalloc(fec, asm, p, precision)
        assert max(rel_err(R2, R_ref)) <= TOL64
        assert max(rel_err(nz2, nz_ref)) <= TOL64


def test_noalloc_poisson_twice(fec):
    torch = _torch()
    mesh, asm, p = _setup(fec, 17, fec.Poisson(1.0))
    for seed in (0, 1):
        U = np.random.default_rng(seed).uniform(-1, 1, mesh.num_nodes)
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        R2, nz2 = _noalloc(fec, asm, p, 0)
        assert max(rel_err(R2, R.cpu().numpy())) <= TOL64
        assert max(rel_err(nz2, K.nzval.cpu().numpy())) <= TOL64


def test_noalloc_rejects_mesh_beyond_static_scratch(fec):
    torch = _torch()
    from fec_gb300 import _lib
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    mesh, asm, p = _setup(fec, 33, phys)   # 32^3 hex8: 32768 * 600 * 8 bytes > 64 MiB
    asm._ensure_pattern()
    for b, (ph, pr) in enumerate(zip(p.physics, p.props), start=1):
        asm._call("fec_physics_set", b, ph.ID, _lib.ptr(pr), int(pr.size))
    lib = fec.load_library()
    R = torch.zeros(asm.dof.unknown_dofs.size, dtype=torch.float64, device="cuda")
    nz = torch.zeros(asm.nnz, dtype=torch.float64, device="cuda")
    st = lib.fec_assemble_noalloc(asm._ctx, 3, 0, 0.0, 0.0, _ptr(p.field), None, None, None, _ptr(R), _ptr(nz),
                                  None)
    assert st == _lib.FEC_ERR_ARG
    assert "static scratch" in _lib.last_error(lib, asm._ctx)
    assert lib.fec_last_launch_count(asm._ctx) == 0
