"""ctypes binding of libfec_gb300.so (the C ABI declared in include/fec_gb300.h).

The product path has no CPU fallback: if the library is missing the import of
the assembler raises, telling the caller to build it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

LIB_PATH = _build.LIB

FEC_OK = 0
FEC_ERR_ARG = -1
FEC_ERR_STATE = -2
FEC_ERR_CUDA = -3
FEC_ERR_UNSUPPORTED = -4
FEC_ERR_NONFINITE = -5
FEC_ERR_DEVICE = -6

FEC_HEX8, FEC_QUAD4, FEC_TET4, FEC_TET10, FEC_HEX27 = 1, 2, 6, 7, 8
FEC_PHYS_POISSON, FEC_PHYS_NEOHOOKEAN, FEC_PHYS_J2, FEC_PHYS_J2_MLP = 1, 2, 3, 4
FEC_FP64, FEC_FP32_ELEMENT = 0, 1
FEC_WANT_RESIDUAL, FEC_WANT_STIFFNESS = 1, 2

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol include/fec_gb300.h declares
SIGNATURES = {
    "fec_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "fec_ctx_destroy": (C.c_int, [_vp]),
    "fec_last_error": (C.c_int, [_vp, C.c_char_p, C.c_size_t]),
    "fec_mesh_set": (C.c_int, [_vp, C.c_int, C.c_int64, _vp, C.c_int, _vp, _vp, _vp]),
    "fec_physics_set": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int]),
    "fec_block_reference_set": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp]),
    "fec_block_reference_get": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), _vp, _vp, _vp]),
    "fec_dofs_set": (C.c_int, [_vp, C.c_int, _vp, C.c_int64]),
    "fec_pattern_build": (C.c_int, [_vp, _i64p]),
    "fec_pattern_get": (C.c_int, [_vp, _vp, _vp]),
    "fec_pattern_build_device": (C.c_int, [_vp, _i64p, _vp]),
    "fec_set_single_launch": (C.c_int, [_vp, C.c_int]),
    "fec_pattern_get_device": (C.c_int, [_vp, _vp, _vp, _vp]),
    "fec_update_field": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, _vp, _vp]),
    "fec_assemble": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fec_assemble_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _vp, _vp, _vp, _vp, _vp, _vp,
                                       _vp]),
    "fec_last_launch_count": (C.c_int, [_vp]),
    "fec_sizes": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p, _i64p]),
    "fec_set_profiling": (C.c_int, [_vp, C.c_int]),
    "fec_mlp_param_count": (C.c_int, []),
    "fec_j2_points": (C.c_int, [_vp, C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fec_mlp_forward": (C.c_int, [_vp, _vp, C.c_int64, _vp, _vp]),
    "fec_mlp_eval_tc": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, _vp, _vp]),
    "fec_autotune_report": (C.c_int, [C.c_char_p, C.c_size_t]),
    "fec_assemble_action": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double, _vp, _vp, _vp, _vp, _vp]),
    "fec_check_finite": (C.c_int, [_vp, _vp, _vp, C.POINTER(C.c_int64), _vp]),
    "fec_cg_solve": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int),
                               C.POINTER(C.c_double), _vp]),
    "fec_tensor_core_status": (C.c_int, [C.c_int]),
    "fec_set_wait_budget": (C.c_int, [C.c_longlong]),
    "fec_mlp_gradient": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, C.c_int64, _vp, _vp, _vp]),
    "fec_mlp_adam_step": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_float, _vp, C.c_int64, _vp,
                                    _vp]),
    "fec_closure_set": (C.c_int, [_vp, _vp, _vp, C.c_float]),
    "fec_closure_stats": (C.c_int, [_vp, _i64p, _i64p, C.c_int]),
    "fec_kernel_times": (C.c_int, [_vp, C.POINTER(C.c_float), C.c_int, C.c_char_p, C.c_size_t]),
    "fec_probe_fma_rate": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "fec_df64_split_check": (C.c_int, [_vp, C.c_int64, _vp, _vp, _vp]),
}


class FECError(RuntimeError):
    """An error status returned through the C ABI (the reference raises an
    AbstractFECError subtype, src/FiniteElementContainers.jl:199-202)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"libfec_gb300 status {status}: {message}")
        self.status = status


_LIB = None


def load(path: Path | None = None):
    """Load the shared library once; raise if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def last_error(lib, ctx) -> str:
    buf = C.create_string_buffer(512)
    lib.fec_last_error(ctx, buf, 512)
    return buf.value.decode(errors="replace")


def check(lib, ctx, status: int) -> None:
    if status != FEC_OK:
        raise FECError(status, last_error(lib, ctx))


def ptr(a) -> int | None:
    """Raw address of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
