"""Loader and ctypes signatures of libdropfluid.so (the product).

The library is built in-tree (``dropfluid/_build/libdropfluid.so``).  There
is no fallback: if the shared library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdropfluid.so")

# Every entry point declared in include/dropfluid.h, with its ctypes signature.
P = C.c_void_p
FP = C.POINTER(C.c_float)
SIGNATURES = {
    "dob_abi_version": (C.c_int, []),
    "dob_last_error": (C.c_char_p, [P]),
    "dob_config_reference": (C.c_int, [C.POINTER(abi.DobConfig)]),
    "dob_config_closed_box": (C.c_int, [C.POINTER(abi.DobConfig), C.c_uint32, C.c_uint32, C.c_uint32]),
    "dob_create": (C.c_int, [C.POINTER(abi.DobConfig), C.POINTER(P)]),
    "dob_destroy": (None, [P]),
    "dob_reset": (C.c_int, [P]),
    "dob_set_uniforms": (C.c_int, [P, FP]),
    "dob_inject_sphere": (C.c_int, [P, FP, C.c_float, C.c_float, FP, C.c_float, C.c_uint64]),
    "dob_inject_sphere_soft": (C.c_int, [P, FP, C.c_float, C.c_float, C.c_float, FP, C.c_float, C.c_uint64]),
    "dob_set_parcels": (C.c_int, [P, FP, C.c_uint32, C.c_uint32]),
    "dob_get_parcels": (C.c_int, [P, FP, C.c_uint32, C.c_uint32]),
    "dob_set_high_water": (C.c_int, [P, C.c_uint32]),
    "dob_set_field": (C.c_int, [P, C.c_int, C.c_void_p, C.c_size_t]),
    "dob_get_field": (C.c_int, [P, C.c_int, C.c_void_p, C.c_size_t]),
    "dob_step": (C.c_int, [P, C.c_int, C.c_uint32, C.POINTER(abi.DobStepStats)]),
    "dob_step_uniforms": (C.c_int, [P, FP, C.c_int, C.c_uint32, C.POINTER(abi.DobStepStats)]),
    "dob_run_stage": (C.c_int, [P, C.c_int]),
    "dob_wave_step": (C.c_int, [P]),
    "dob_light_volume": (C.c_int, [P]),
    "dob_set_spectral_lut": (C.c_int, [P, C.c_void_p, C.c_size_t]),
    "dob_render_plume": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t]),
    "dob_sync": (C.c_int, [P]),
    "dob_memory_bytes": (C.c_int, [P, C.POINTER(C.c_uint64)]),
    "dob_launches_per_step": (C.c_int, [P, C.POINTER(C.c_int)]),
    "dob_io_bytes": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "dob_time_steps": (C.c_int, [P, C.c_int, C.c_uint32, FP]),
    "dob_bench_kernel": (C.c_int, [P, C.c_int, C.c_int, FP, C.POINTER(C.c_double)]),
    "dob_save_state": (C.c_int, [P, C.c_int]),
    "dob_load_state": (C.c_int, [P, C.c_int]),
    "dob_eval_math": (C.c_int, [C.c_int, FP, FP, FP, C.c_uint32]),
    "dob_pressure_solve_noalloc": (C.c_int, [C.POINTER(abi.DobConfig), P, P, P]),
    "dob_step_async": (C.c_int, [P, C.c_int]),
    "dob_step_result": (C.c_int, [P, C.c_int, C.POINTER(abi.DobStepStats)]),
    "dob_set_step_stats": (C.c_int, [P, C.c_uint32]),
    "dob_adjoint_stage": (C.c_int, [P, C.c_int]),
    "dob_tape_forward": (C.c_int, [P, C.c_int, C.c_int]),
    "dob_tape_backward": (C.c_int, [P, FP, C.c_size_t]),
    "dob_adjoint_sphere_impulse": (C.c_int, [P, C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float),
                                             C.POINTER(C.c_double)]),
    "dob_adjoint_sphere_soft": (C.c_int, [P, FP, C.c_float, C.c_float, C.c_float, FP, C.c_float, C.c_uint64,
                                          C.POINTER(C.c_double)]),
}

_lib = None


class DropFluidError(RuntimeError):
    """A C-ABI call returned a non-zero dob_status."""

    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        name = abi.STATUS_NAMES.get(status, str(status))
        super().__init__(f"{what} -> {name}" + (f": {detail}" if detail else ""))


def load(path: str | None = None):
    """Load libdropfluid.so and declare every signature; raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"libdropfluid.so not built ({p}); run dropfluid.build.build() or __graft_entry__.build()")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def check(rc: int, what: str, ctx=None):
    if rc != 0:
        detail = ""
        try:
            msg = load().dob_last_error(ctx)
            detail = msg.decode() if msg else ""
        except Exception:
            pass
        raise DropFluidError(rc, what, detail)
