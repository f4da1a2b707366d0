"""fec_assemble_noalloc: assembly for callers that cannot let the library
allocate device memory (their device memory all goes through their own pool,
or their device-memory budget is fixed up front).

The entry point is called through the C ABI and runs the same kernels as
fec_assemble, the allocating entry point, so it must reproduce it bit for bit
on two calls in a row (the second with a different displacement, so a stale
workspace would show), for Neo-Hookean, Poisson and J2 with state; for the
learned closure it must equal fec_assemble's per-point CUDA-core closure bit for
bit and its tensor-core closure within the closure's tolerance.  It refuses a
mesh whose element workspace does not fit its static array, and keeps working
after the device's primary context is reset (its array is looked up again).
This file is collected last so that a failure here leaves every other test
already run."""
import ctypes as C
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from helpers import rel_err, stretch_field

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
J2_PROPS = [200.0, 0.3, 0.25, 2.0]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _ptr(t):
    return None if t is None else t.data_ptr()


def _setup(fec, n, physics, precision="fp64", bcs=None):
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    V = fec.FunctionSpace(mesh)
    var = fec.VectorFunction(V, "u") if physics.NF == 3 else fec.ScalarFunction(V, "u")
    asm = fec.SparseMatrixAssembler(var, device=0, precision=precision)
    if bcs is None:
        bcs = [] if physics.NF == 3 else [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name="left")]
    p = fec.create_parameters(mesh, asm, physics, dirichlet_bcs=bcs)
    return mesh, asm, p


def _noalloc(fec, asm, p, precision):
    """Same inputs as the last fec_assemble call (field and state already in p),
    outputs into fresh NaN-filled tensors; returns (R, nzval, state_new)."""
    torch = _torch()
    lib = fec.load_library()
    R = torch.full((asm.dof.unknown_dofs.size,), float("nan"), dtype=torch.float64, device="cuda")
    nz = torch.full((asm.nnz,), float("nan"), dtype=torch.float64, device="cuda")
    has_state = any(ph.NS for ph in p.physics)
    sn = torch.full_like(p.state_new, float("nan")) if has_state else None
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.fec_assemble_noalloc(asm._ctx, 3, precision, p.t, p.dt, _ptr(p.field), _ptr(p.field_old),
                                  _ptr(p.state_old) if has_state else None, _ptr(sn), _ptr(R), _ptr(nz), stream)
    from fec_gb300 import _lib
    _lib.check(lib, asm._ctx, st)
    torch.cuda.synchronize()
    return R.cpu().numpy(), nz.cpu().numpy(), None if sn is None else sn.cpu().numpy()


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
        R2, nz2, _ = _noalloc(fec, asm, p, precision)
        assert np.array_equal(R2, R_ref) and np.array_equal(nz2, nz_ref)


def test_noalloc_poisson_twice(fec):
    torch = _torch()
    mesh, asm, p = _setup(fec, 17, fec.Poisson(1.0))
    for seed in (0, 1):
        U = np.random.default_rng(seed).uniform(-1, 1, mesh.num_nodes)
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        R2, nz2, _ = _noalloc(fec, asm, p, 0)
        assert np.array_equal(R2, R.cpu().numpy()) and np.array_equal(nz2, K.nzval.cpu().numpy())


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_element"])
def test_noalloc_j2_with_state_two_steps(fec, precision):
    """J2 with plastic state carried over two load steps: residual, tangent and
    the new state bit for bit those of fec_assemble."""
    torch = _torch()
    from fec_gb300.workloads import uniaxial_path
    phys = fec.J2Plasticity(*J2_PROPS)
    mesh, asm, p = _setup(fec, 7, phys)
    prec = "fp64" if precision == 0 else "fp32_element"
    yielded = 0
    for step in (3, 6):   # two calls in a row along the path
        U = uniaxial_path(mesh.nodal_coords, step, nsteps=6, final_strain=0.01).ravel()
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=prec)
        torch.cuda.synchronize()
        R_ref, nz_ref, sn_ref = R.cpu().numpy().copy(), K.nzval.cpu().numpy().copy(), p.state_new.cpu().numpy()
        R2, nz2, sn2 = _noalloc(fec, asm, p, precision)
        assert np.array_equal(R2, R_ref) and np.array_equal(nz2, nz_ref) and np.array_equal(sn2, sn_ref)
        yielded = max(yielded, int((sn_ref[6::7] > 0).sum()))
        p.swap_states()
    assert yielded > 0


def test_noalloc_learned_closure(fec):
    """FEC_PHYS_J2_MLP hex8 blocks in FP32-element arithmetic: the no-alloc
    entry point evaluates the closure per point on the CUDA cores, bit for bit
    what fec_assemble does with FEC_CLOSURE_ON_CUDA_CORES=1, and within the
    closure's tolerance of fec_assemble's tensor-core closure."""
    torch = _torch()
    from fec_gb300 import closure
    from fec_gb300.workloads import uniaxial_path
    X, Y, plastic = closure.generate_samples(J2_PROPS, n_paths=6000, steps=10, seed=4)
    trained = closure.train(X[plastic], Y[plastic], epochs=8, batch=2048, lr=5e-3)
    tol = 5e-2
    cl = closure.TrainedClosure(trained.params, trained.normalisation, [], tol)
    phys = closure.J2Closure(*J2_PROPS, cl)
    mesh, asm, p = _setup(fec, 7, phys, precision="fp32_element")
    U = uniaxial_path(mesh.nodal_coords, 6, nsteps=6, final_strain=0.01).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    R_tc, K_tc = fec.assemble_residual_and_stiffness(asm, Uu, p)
    torch.cuda.synchronize()
    R_tc, nz_tc = R_tc.cpu().numpy().copy(), K_tc.nzval.cpu().numpy().copy()
    closure.J2Closure.stats(asm, reset=True)
    os.environ["FEC_CLOSURE_ON_CUDA_CORES"] = "1"
    try:
        R_cc, K_cc = fec.assemble_residual_and_stiffness(asm, Uu, p)
        torch.cuda.synchronize()
        R_cc, nz_cc, sn_cc = R_cc.cpu().numpy().copy(), K_cc.nzval.cpu().numpy().copy(), p.state_new.cpu().numpy()
        stats_cc = closure.J2Closure.stats(asm, reset=True)
    finally:
        del os.environ["FEC_CLOSURE_ON_CUDA_CORES"]
    R2, nz2, sn2 = _noalloc(fec, asm, p, 1)
    stats_na = closure.J2Closure.stats(asm, reset=True)
    assert np.array_equal(R2, R_cc) and np.array_equal(nz2, nz_cc) and np.array_equal(sn2, sn_cc)
    assert stats_na == stats_cc and stats_na[0] > 0
    e_r, e_k = rel_err(R2, R_tc), rel_err(nz2, nz_tc)
    print("no-alloc (CUDA-core closure) vs tensor-core closure: residual", e_r, "nzval", e_k, "stats", stats_na)
    assert e_r[1] <= tol and e_k[1] <= tol


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


# Runs in a fresh process without torch: device memory through the driver API in
# the device's primary context (the one the library uses), an assembly through
# both entry points, a reset of the primary context (what cudaDeviceReset or
# CUDA.jl's device_reset! do), and the same again in the new context.
_RESET_SCRIPT = textwrap.dedent(r'''
    import ctypes as C, sys
    import numpy as np
    sys.path[:0] = [sys.argv[1] + "/finiteelementcontainers.jl_gb300", sys.argv[1]]
    import fec_gb300 as fec
    from fec_gb300 import _lib
    from fec_gb300.workloads import stretch_field
    cu = C.CDLL("libcuda.so.1")
    def ck(r, what):
        if r != 0:
            print("DRIVER", what, r); sys.exit(3)
    ck(cu.cuInit(0), "cuInit")
    dev = C.c_int()
    ck(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
    lib = _lib.load()
    n = 6
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n, n, n))
    X = np.ascontiguousarray(mesh.nodal_coords)
    conn = np.ascontiguousarray(mesh.element_conns["block_1"], dtype=np.int64)
    U = stretch_field(X, seed=3).ravel()
    nn, ne = X.shape[0], conn.shape[0]
    dtu = np.arange(1, 3 * nn + 1, dtype=np.int64)
    props = np.array([0.8333333333333334, 0.38461538461538464])

    def one_round(after_reset):
        ctx = C.c_void_p()
        ck(cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "retain")
        ck(cu.cuCtxSetCurrent(ctx), "set current")
        h = C.c_void_p()
        st = lib.fec_ctx_create(0, C.byref(h))
        if st:
            print("LIB create", st, _lib.last_error(lib, None)); sys.exit(4)
        def call(name, *a):
            st = getattr(lib, name)(h, *a)
            if st:
                print("LIB", name, st, _lib.last_error(lib, h))
                # after the reset, a failure before the no-alloc call is the CUDA runtime's, not the entry point's
                sys.exit(6 if after_reset and name != "fec_assemble_noalloc" else 4)
        types = np.array([1], dtype=np.int32); nes = np.array([ne], dtype=np.int64)
        call("fec_mesh_set", 3, nn, _lib.ptr(X), 1, _lib.ptr(types), _lib.ptr(nes), _lib.ptr(conn))
        call("fec_physics_set", 1, 2, _lib.ptr(props), 2)
        call("fec_dofs_set", 3, _lib.ptr(dtu), 3 * nn)
        nnz = C.c_int64()
        call("fec_pattern_build", C.byref(nnz))
        bufs = {}
        for name, count in (("U", U.size), ("R", 3 * nn), ("nz", nnz.value)):
            p = C.c_uint64()
            ck(cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(8 * count)), "alloc")
            bufs[name] = p.value
        ck(cu.cuMemcpyHtoD_v2(C.c_uint64(bufs["U"]), U.ctypes.data, C.c_size_t(8 * U.size)), "HtoD")
        out = []
        for entry in ("fec_assemble", "fec_assemble_noalloc"):
            call(entry, 3, 0, 0.0, 0.0, C.c_void_p(bufs["U"]), None, None, None, C.c_void_p(bufs["R"]),
                 C.c_void_p(bufs["nz"]), None)
            ck(cu.cuCtxSynchronize(), "sync")
            R = np.empty(3 * nn); nz = np.empty(nnz.value)
            ck(cu.cuMemcpyDtoH_v2(R.ctypes.data, C.c_uint64(bufs["R"]), C.c_size_t(8 * R.size)), "DtoH")
            ck(cu.cuMemcpyDtoH_v2(nz.ctypes.data, C.c_uint64(bufs["nz"]), C.c_size_t(8 * nz.size)), "DtoH")
            out.append((R, nz))
        lib.fec_ctx_destroy(h)
        for p in bufs.values():
            ck(cu.cuMemFree_v2(C.c_uint64(p)), "free")
        ck(cu.cuDevicePrimaryCtxRelease_v2(dev), "release")
        return out

    first = one_round(False)
    ck(cu.cuDevicePrimaryCtxReset_v2(dev), "reset")
    second = one_round(True)
    R0, nz0 = first[0]
    ok = all(np.array_equal(R, R0) and np.array_equal(nz, nz0) for R, nz in first + second)
    print("RESULT", "equal" if ok else "different")
    sys.exit(0 if ok else 5)
''')


def test_noalloc_after_primary_context_reset():
    """A reset of the device's primary context between calls: in a fresh
    process, both entry points give the same bits before and after the reset
    (the no-alloc entry point looks its static array up again instead of
    reusing the address of the old context)."""
    _torch()
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, str(ROOT)], capture_output=True, text=True,
                       timeout=600)
    print(r.stdout[-2000:], r.stderr[-2000:])
    if r.returncode == 6:
        pytest.skip("the CUDA runtime linked into the library does not come back after an external reset of the "
                    "primary context (the allocating path fails too): " + r.stdout.strip()[-300:])
    assert r.returncode == 0 and "RESULT equal" in r.stdout
