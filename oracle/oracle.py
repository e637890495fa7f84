"""TEST INFRASTRUCTURE — ctypes driver of the oracle (the CPU restatement of
the reference step in dob_oracle.cpp).  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg may use it, and only as the checker.

The API mirrors the product's ``dropfluid.engine.DropFluid`` so a test can
run both on the same inputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdob_oracle.so")

_PKG = os.path.join(os.path.dirname(HERE), "drop-of-blood_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from dropfluid import abi  # noqa: E402

_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (seconds)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(abi.DobConfig), C.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_reset.argtypes = [P]
        L.orc_set_uniforms.argtypes = [P, C.POINTER(C.c_float)]
        L.orc_inject_sphere.argtypes = [P, C.POINTER(C.c_float), C.c_float, C.c_float,
                                        C.POINTER(C.c_float), C.c_float, C.c_uint64]
        L.orc_inject_sphere_soft.argtypes = [P, C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float,
                                             C.POINTER(C.c_float), C.c_float, C.c_uint64]
        L.orc_sphere_soft_grad.argtypes = [P, C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float,
                                           C.POINTER(C.c_float), C.c_float, C.c_uint64, C.POINTER(C.c_double)]
        L.orc_set_parcels.argtypes = [P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32]
        L.orc_get_parcels.argtypes = [P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32]
        L.orc_set_high_water.argtypes = [P, C.c_uint32]
        L.orc_set_field.argtypes = [P, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_get_field.argtypes = [P, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_step.argtypes = [P, C.c_int, C.POINTER(C.c_double)]
        L.orc_run_stage.argtypes = [P, C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_adjoint_stage.argtypes = [P, C.c_int]
        L.orc_wave_step.argtypes = [P]
        L.orc_light_volume.argtypes = [P]
        L.orc_render_plume.argtypes = [P, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.orc_wave_fft2.argtypes = [C.POINTER(C.c_float), C.c_int]
        L.orc_tape_forward.argtypes = [P, C.c_int]
        L.orc_tape_backward.argtypes = [P, C.POINTER(C.c_float), C.c_size_t]
        L.orc_sphere_impulse.argtypes = [P, C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float),
                                         C.POINTER(C.c_double)]
        L.orc_get_field64.argtypes = [P, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_set_field64.argtypes = [P, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_coarse_inverse.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                         C.POINTER(C.c_double)]
        L.orc_eval_math.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.c_uint32]
        _lib = L
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed: {abi.STATUS_NAMES.get(rc, rc)}")


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def wave_fft2(z: np.ndarray, inverse: bool = False) -> np.ndarray:
    """Unitary 2-D transform of a 512x512 complex64 array by the wave passes."""
    a = np.ascontiguousarray(np.asarray(z, np.complex64)).copy()
    assert a.shape == (512, 512)
    f = a.view(np.float32)
    _check(lib().orc_wave_fft2(_fptr(f), int(bool(inverse))), "wave_fft2")
    return a


def eval_math(fn: int, x, y=None) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
    out = np.empty_like(x)
    _check(lib().orc_eval_math(fn, _fptr(x), None if yy is None else _fptr(yy), _fptr(out), x.size),
           "eval_math")
    return out


class OracleSim:
    """CPU restatement of the step; fp64=True is the FP64 oracle."""

    def __init__(self, cfg: abi.DobConfig, fp64: bool = False):
        self.cfg = cfg.copy()
        self._h = lib().orc_create(C.byref(self.cfg), 1 if fp64 else 0)
        if not self._h:
            raise ValueError("oracle rejected the configuration")
        self.fp64 = fp64
        r = cfg.dye_refine
        self.vdims = (cfg.nz, cfg.ny, cfg.nx)
        self.cdims = (cfg.nz * r, cfg.ny * r, cfg.nx * r)

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------------
    def reset(self):
        _check(lib().orc_reset(self._h), "reset")

    def set_uniforms(self, u):
        u = np.ascontiguousarray(u, dtype=np.float32)
        assert u.size == 128
        _check(lib().orc_set_uniforms(self._h, _fptr(u)), "set_uniforms")

    def inject_sphere(self, center, radius, dye, vel, noise_sigma=0.0, seed=0):
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        _check(lib().orc_inject_sphere(self._h, _fptr(c), float(radius), float(dye), _fptr(v),
                                       float(noise_sigma), int(seed)), "inject_sphere")

    def inject_sphere_soft(self, center, radius, edge, dye, vel, noise_sigma=0.0, seed=0):
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        _check(lib().orc_inject_sphere_soft(self._h, _fptr(c), float(radius), float(edge), float(dye), _fptr(v),
                                            float(noise_sigma), int(seed)), "inject_sphere_soft")

    def sphere_soft_grad(self, center, radius, edge, dye, vel, noise_sigma=0.0, seed=0):
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        out = (C.c_double * 4)()
        _check(lib().orc_sphere_soft_grad(self._h, _fptr(c), float(radius), float(edge), float(dye), _fptr(v),
                                          float(noise_sigma), int(seed), out), "sphere_soft_grad")
        return out[0], np.array(out[1:4], dtype=np.float64)

    def set_parcels(self, parcels, offset=0):
        p = np.ascontiguousarray(parcels, dtype=np.float32).reshape(-1, 8)
        _check(lib().orc_set_parcels(self._h, _fptr(p), p.shape[0], offset), "set_parcels")

    def get_parcels(self, n=None, offset=0):
        n = self.cfg.parcel_capacity - offset if n is None else n
        out = np.empty((n, 8), dtype=np.float32)
        _check(lib().orc_get_parcels(self._h, _fptr(out), n, offset), "get_parcels")
        return out

    def set_high_water(self, hw):
        _check(lib().orc_set_high_water(self._h, int(hw)), "set_high_water")

    def _field_shape(self, field):
        ref = self.cfg.bc_mode == abi.DOB_BC_REFERENCE
        return abi.field_shapes(self.vdims, self.cdims, ref)[field]

    def field_shape(self, field):
        return self._field_shape(field)

    def set_field(self, field, arr):
        shape, dt = self._field_shape(field)
        a = np.ascontiguousarray(arr, dtype=dt).reshape(shape)
        _check(lib().orc_set_field(self._h, field, a.ctypes.data, a.nbytes), "set_field")

    def get_field(self, field):
        shape, dt = self._field_shape(field)
        a = np.empty(shape, dtype=dt)
        _check(lib().orc_get_field(self._h, field, a.ctypes.data, a.nbytes), "get_field")
        return a

    # -- stepping ---------------------------------------------------------------------
    def step(self, n=1, stats=False):
        st = (C.c_double * 5)()
        _check(lib().orc_step(self._h, int(n), st if stats else None), "step")
        if stats:
            return {"rhs_l2": st[0], "residual_l2": st[1], "max_div": st[2],
                    "vcycles": int(st[3]), "outer_iters": int(st[4])}
        return None

    def run_stage(self, stage):
        _check(lib().orc_run_stage(self._h, int(stage)), f"run_stage({stage})")

    def wave_step(self):
        """One substep of the 512x512 wave solver on the wave field."""
        _check(lib().orc_wave_step(self._h), "wave_step")

    def light_volume(self):
        """The light volume and brick passes (lighting.ts:19-240)."""
        _check(lib().orc_light_volume(self._h), "light_volume")

    def render_plume(self, width, height, lut):
        """The plume render (render.ts:1593-2109 from fsMain's camera ray):
        (height, width, 8) binary16 as uint16 (radiance rgb, tauTotal,
        transmittance rgb, tauIntact); lut (64, 256, 4) float32."""
        lut = np.ascontiguousarray(lut, np.float32)
        assert lut.shape == (64, 256, 4)
        out = np.zeros((height, width, 8), np.uint16)
        _check(lib().orc_render_plume(self._h, lut.ctypes.data, int(width), int(height), out.ctypes.data),
               "render_plume")
        return out

    # -- discrete adjoint (closed box, dye_refine 1) ---------------------------------------
    def adjoint_stage(self, stage):
        _check(lib().orc_adjoint_stage(self._h, int(stage)), f"adjoint_stage({stage})")

    def tape_forward(self, nsteps, checkpoint_every=None):
        _check(lib().orc_tape_forward(self._h, int(nsteps)), "tape_forward")

    def tape_backward(self, dye_grad):
        shape, _ = self._field_shape(abi.FIELD_ADJ_CONC)
        g = np.ascontiguousarray(dye_grad, dtype=np.float32).reshape(shape)
        _check(lib().orc_tape_backward(self._h, _fptr(g), g.nbytes), "tape_backward")

    def get_field64(self, field):
        shape, _ = self._field_shape(field)
        a = np.empty(shape, dtype=np.float64)
        _check(lib().orc_get_field64(self._h, int(field), a.ctypes.data, a.size), "get_field64")
        return a

    def set_field64(self, field, arr):
        shape, _ = self._field_shape(field)
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(shape)
        _check(lib().orc_set_field64(self._h, int(field), a.ctypes.data, a.size), "set_field64")

    def gradients(self):
        return {"u": self.get_field64(abi.FIELD_ADJ_VEL_U), "v": self.get_field64(abi.FIELD_ADJ_VEL_V),
                "w": self.get_field64(abi.FIELD_ADJ_VEL_W), "dye": self.get_field64(abi.FIELD_ADJ_CONC),
                "p": self.get_field64(abi.FIELD_ADJ_PRESSURE)}

    def sphere_impulse(self, center, radius, vel) -> float:
        c = (C.c_float * 3)(*center)
        v = (C.c_float * 3)(*vel)
        out = C.c_double(0.0)
        _check(lib().orc_sphere_impulse(self._h, c, C.c_float(radius), v, C.byref(out)), "sphere_impulse")
        return out.value


def coarse_inverse(dims, h2, ref, method):
    """Dense coarsest-grid inverse (n x n, natural cell order): method 0
    Gauss-Jordan, 1 the separable form the simulation uses."""
    nx, ny, nz = dims
    n = nx * ny * nz
    out = np.zeros((n, n), np.float64)
    _check(lib().orc_coarse_inverse(nx, ny, nz, float(h2), int(ref), int(method),
                                    out.ctypes.data_as(C.POINTER(C.c_double))), "coarse_inverse")
    return out
