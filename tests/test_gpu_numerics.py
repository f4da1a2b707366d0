"""The FP64 path's conversions on the device, against host arithmetic.

The FP64 element kernels split doubles into double-float pairs (hi, lo) with
integer operations, and the node gather widens floats back to double the same
way; both must agree with IEEE conversions on every input class."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _inputs():
    rng = np.random.default_rng(7)
    n = 200_000
    special = np.array([
        0.0, -0.0, 1.0, -1.0, 0.5, 3.0,
        2.0 ** -74, -(2.0 ** -74), 2.0 ** -75, 2.0 ** -126, 2.0 ** -149, 2.0 ** -1000, 5e-324, -5e-324,
        2.0 ** 125 * 1.75, 2.0 ** 126, 2.0 ** 127, 3.4e38, 1e300, -1e300, np.inf, -np.inf,
        1.0 + 2.0 ** -24, -(1.0 + 2.0 ** -24), 1.0 + 3.0 * 2.0 ** -25, (2.0 ** 24 - 1.0) / 2.0 ** 24,
        (2.0 ** 53 - 1.0) / 2.0 ** 53, 1.0 - 2.0 ** -25, 1.0 / 3.0, -2.0 / 3.0, np.pi * 1e-8])
    return np.concatenate([
        rng.standard_normal(n) * 10.0 ** rng.integers(-40, 40, n),
        rng.uniform(-1.0, 1.0, n),
        rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64),  # every bit-pattern class
        special])


def test_df64_split_and_widen_match_host_arithmetic(fec):
    torch = _torch()
    from fec_gb300 import _lib
    lib = fec.load_library()
    x = _inputs()
    n = x.size
    xd = torch.from_numpy(x).cuda()
    split = torch.empty(2 * n, dtype=torch.float32, device="cuda")
    wid = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fec_df64_split_check(_lib.ptr(xd), n, _lib.ptr(split), _lib.ptr(wid), s) == 0
    torch.cuda.synchronize()
    sp, wd = split.cpu().numpy(), wid.cpu().numpy()
    hi, lo = sp[0::2], sp[1::2]

    # widening back to double is exact for every float, NaN stays NaN
    for f, w in ((hi, wd[0::2]), (lo, wd[1::2])):
        nan = np.isnan(f)
        assert np.array_equal(np.isnan(w), nan)
        assert np.array_equal(w[~nan].view(np.uint64), f[~nan].astype(np.float64).view(np.uint64))

    with np.errstate(over="ignore", invalid="ignore"):
        hi_ref = x.astype(np.float32)                       # round to nearest, ties to even
        lo_ref = (x - hi_ref.astype(np.float64)).astype(np.float32)
    fast = (np.abs(x) >= 2.0 ** -74) & (np.abs(x) < 2.0 ** 126) & np.isfinite(x)
    other = ~fast & ~np.isnan(x)
    # outside the integer path's range the split is the conversion split, bit for bit
    assert np.array_equal(hi[other].view(np.uint32), hi_ref[other].view(np.uint32))
    lo_o, lo_ro = lo[other], lo_ref[other]
    both_nan = np.isnan(lo_o) & np.isnan(lo_ro)
    assert np.array_equal(lo_o[~both_nan].view(np.uint32), lo_ro[~both_nan].view(np.uint32))
    # inside it: hi is a nearest float (ties may round away from zero), |lo| <= ulp(hi)/2,
    # and hi + lo represents x to 2^-48 relative
    xf, hf, lf = x[fast], hi[fast].astype(np.float64), lo[fast].astype(np.float64)
    ulp = np.spacing(np.abs(hi[fast])).astype(np.float64)
    assert np.all(np.abs(xf - hf) <= 0.5 * ulp)
    differs = hi[fast] != hi_ref[fast]
    assert np.all(np.abs(xf[differs] - hf[differs]) == 0.5 * ulp[differs])  # only exact ties differ
    assert np.all(np.abs(lf) <= 0.5 * ulp)
    assert np.all(np.abs(hf + lf - xf) <= 2.0 ** -48 * np.abs(xf))
    # signed zeros
    z = np.flatnonzero(x == 0.0)
    assert np.array_equal(np.signbit(hi[z]), np.signbit(x[z])) and np.all(lo[z] == 0.0)
