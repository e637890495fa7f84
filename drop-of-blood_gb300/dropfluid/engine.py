"""Host-side mirror of the reference engine's physics interface.

``DropFluid`` owns one libdropfluid context (all device memory of one
simulation) and exposes the operations the reference's ``BloodDropEngine``
performs for the fluid path (src/engine/BloodDropEngine.ts):

  reference                                   here
  ------------------------------------------  ------------------------------------
  BloodDropEngine.create(canvas)  :336        DropFluid(config)
  resetSimulation(seed, offsetXZ) :1682       reset()  (+ set_uniforms for the seed)
  queue.writeBuffer(uniforms)     :2602       set_uniforms(block)
  encodePhysicsStep(enc, spawn)   :1855       step()
  seekToSimTime / multi-substep   :2142,2634  step_uniforms(blocks)
  gpuPassTimingsMs (timestamps)   :2400       time_steps(), stats['stage_ms']
  destroy()                       :2671       close()

Errors follow the reference's engine contract: construction raises, later
calls raise ``DropFluidError`` carrying the library's status and message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import DropFluidError, check, load


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class DropFluid:
    def __init__(self, config: abi.DobConfig):
        self._L = load()
        self.cfg = config.copy()
        h = C.c_void_p()
        rc = self._L.dob_create(C.byref(self.cfg), C.byref(h))
        if rc != 0:
            msg = self._L.dob_last_error(None)
            raise DropFluidError(rc, "dob_create", msg.decode() if msg else "")
        self._h = h
        r = config.dye_refine
        self.vdims = (config.nz, config.ny, config.nx)
        self.cdims = (config.nz * r, config.ny * r, config.nx * r)

    # -- lifecycle ---------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.dob_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        check(rc, what, self._h)

    # -- state ----------------------------------------------------------------------
    def reset(self):
        self._ck(self._L.dob_reset(self._h), "dob_reset")

    def set_uniforms(self, block):
        u = np.ascontiguousarray(block, dtype=np.float32)
        if u.size != 128:
            raise ValueError("the uniform block has 128 floats (512 bytes)")
        self._ck(self._L.dob_set_uniforms(self._h, _fptr(u)), "dob_set_uniforms")

    def inject_sphere(self, center, radius, dye, vel, noise_sigma=0.0, seed=0):
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        self._ck(self._L.dob_inject_sphere(self._h, _fptr(c), float(radius), float(dye), _fptr(v),
                                           float(noise_sigma), int(seed)), "dob_inject_sphere")

    def inject_sphere_soft(self, center, radius, edge, dye, vel, noise_sigma=0.0, seed=0):
        """Soft-edged additive drop (dob_inject_sphere_soft)."""
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        self._ck(self._L.dob_inject_sphere_soft(self._h, _fptr(c), float(radius), float(edge), float(dye), _fptr(v),
                                                float(noise_sigma), int(seed)), "dob_inject_sphere_soft")

    def set_parcels(self, parcels, offset=0):
        p = np.ascontiguousarray(parcels, dtype=np.float32).reshape(-1, abi.PARCEL_FLOATS)
        self._ck(self._L.dob_set_parcels(self._h, _fptr(p), p.shape[0], int(offset)), "dob_set_parcels")

    def get_parcels(self, n=None, offset=0):
        n = self.cfg.parcel_capacity - offset if n is None else n
        out = np.empty((n, abi.PARCEL_FLOATS), dtype=np.float32)
        self._ck(self._L.dob_get_parcels(self._h, _fptr(out), n, int(offset)), "dob_get_parcels")
        return out

    def set_high_water(self, hw):
        self._ck(self._L.dob_set_high_water(self._h, int(hw)), "dob_set_high_water")

    def field_shape(self, field):
        ref = self.cfg.bc_mode == abi.DOB_BC_REFERENCE
        return abi.field_shapes(self.vdims, self.cdims, ref)[field]

    def set_field(self, field, arr):
        shape, dt = self.field_shape(field)
        a = np.ascontiguousarray(arr, dtype=dt).reshape(shape)
        self._ck(self._L.dob_set_field(self._h, int(field), a.ctypes.data, a.nbytes), "dob_set_field")

    def get_field(self, field):
        shape, dt = self.field_shape(field)
        a = np.empty(shape, dtype=dt)
        self._ck(self._L.dob_get_field(self._h, int(field), a.ctypes.data, a.nbytes), "dob_get_field")
        return a

    # -- stepping ----------------------------------------------------------------------
    def step(self, n=1, stats=False, timing=False, graph=True):
        flags = (abi.STEP_STATS if stats else 0) | (abi.STEP_TIMING if timing else 0) | \
                (0 if graph else abi.STEP_NO_GRAPH)
        st = abi.DobStepStats()
        want = stats or timing
        self._ck(self._L.dob_step(self._h, int(n), flags, C.byref(st) if want else None), "dob_step")
        if not want:
            return None
        return self._stats_dict(st)

    @staticmethod
    def _stats_dict(st):
        return {
            "steps_done": st.steps_done, "vcycles": st.vcycles, "outer_iters": st.outer_iters,
            "rhs_l2": st.rhs_l2, "residual_l2": st.residual_l2, "max_div": st.max_div,
            "parcels_alive": st.parcels_alive,
            "stage_ms": {abi.STAGE_NAMES[k]: st.stage_ms[k] for k in range(abi.STAGE_COUNT)},
        }

    def step_async(self, slot):
        """Enqueue one step with statistics into result slot 0..7."""
        self._ck(self._L.dob_step_async(self._h, int(slot)), "dob_step_async")

    def step_result(self, slot):
        """Wait for the step of `slot` and return its statistics."""
        st = abi.DobStepStats()
        st.struct_size = C.sizeof(abi.DobStepStats)
        self._ck(self._L.dob_step_result(self._h, int(slot), C.byref(st)), "dob_step_result")
        return self._stats_dict(st)

    def set_step_stats(self, mask):
        """Statistics a step with statistics forms (dob_set_step_stats):
        abi.STATS_ALL, or a mask of STATS_RESIDUAL / STATS_PARCELS over the
        always-formed max |div| and ||b||."""
        self._ck(self._L.dob_set_step_stats(self._h, int(mask)), "dob_set_step_stats")

    def run_pipelined(self, n, depth=2):
        """n steps, each step's statistics read back while the next runs."""
        out = []
        for k in range(n):
            self.step_async(k % 8)
            if k >= depth - 1:
                out.append(self.step_result((k - depth + 1) % 8))
        for k in range(max(0, n - depth + 1), n):
            out.append(self.step_result(k % 8))
        return out

    def step_uniforms(self, blocks, stats=False):
        b = np.ascontiguousarray(blocks, dtype=np.float32).reshape(-1, 128)
        st = abi.DobStepStats()
        flags = abi.STEP_STATS if stats else 0
        self._ck(self._L.dob_step_uniforms(self._h, _fptr(b), b.shape[0], flags,
                                           C.byref(st) if stats else None), "dob_step_uniforms")

    def run_stage(self, stage):
        self._ck(self._L.dob_run_stage(self._h, int(stage)), f"dob_run_stage({stage})")

    def wave_step(self):
        """One substep of the 512x512 wave solver (contexts made with DOB_PHYS_WAVE)."""
        self._ck(self._L.dob_wave_step(self._h), "dob_wave_step")

    def light_volume(self):
        """Light volume and brick occupancy from the current dye and wave
        (reference mode); read them with FIELD_LIGHT / FIELD_BRICKS."""
        self._ck(self._L.dob_light_volume(self._h), "dob_light_volume")

    def set_spectral_lut(self, lut):
        """The renderer's 256 x 64 spectral transmittance table, (64, 256, 4)
        float32 (u fastest)."""
        a = np.ascontiguousarray(lut, np.float32)
        if a.shape != (64, 256, 4):
            raise ValueError("spectral table must be (64, 256, 4)")
        self._ck(self._L.dob_set_spectral_lut(self._h, a.ctypes.data, a.nbytes), "dob_set_spectral_lut")

    def render_plume(self, width, height):
        """The plume render of the current state (dob_render_plume): (height,
        width, 8) binary16 as uint16 -- radiance rgb, total optical depth,
        transmittance rgb, intact-cell optical depth."""
        out = np.zeros((int(height), int(width), 8), np.uint16)
        self._ck(self._L.dob_render_plume(self._h, int(width), int(height), out.ctypes.data, out.nbytes),
                 "dob_render_plume")
        return out

    def sync(self):
        self._ck(self._L.dob_sync(self._h), "dob_sync")

    def memory_bytes(self) -> int:
        b = C.c_uint64()
        self._ck(self._L.dob_memory_bytes(self._h, C.byref(b)), "dob_memory_bytes")
        return int(b.value)

    def io_bytes(self):
        """(host->device bytes per step, device->host bytes of the statistics)."""
        a, b = C.c_uint64(), C.c_uint64()
        self._ck(self._L.dob_io_bytes(self._h, C.byref(a), C.byref(b)), "dob_io_bytes")
        return int(a.value), int(b.value)

    def launches_per_step(self) -> int:
        n = C.c_int()
        self._ck(self._L.dob_launches_per_step(self._h, C.byref(n)), "dob_launches_per_step")
        return int(n.value)

    def time_steps(self, n, graph=True) -> float:
        ms = C.c_float()
        flags = 0 if graph else abi.STEP_NO_GRAPH
        self._ck(self._L.dob_time_steps(self._h, int(n), flags, C.byref(ms)), "dob_time_steps")
        return float(ms.value)

    def bench_kernel(self, which=0, reps=10):
        ms = C.c_float()
        by = C.c_double()
        self._ck(self._L.dob_bench_kernel(self._h, int(which), int(reps), C.byref(ms), C.byref(by)),
                 "dob_bench_kernel")
        return float(ms.value), float(by.value)

    # -- discrete adjoint (closed box, FP32 or mixed, dye_refine 1) ---------------------------
    def adjoint_stage(self, stage):
        """Transpose of the Jacobian of one stage at the current forward state
        (field conventions of dob_adjoint_stage)."""
        self._ck(self._L.dob_adjoint_stage(self._h, int(stage)), f"dob_adjoint_stage({stage})")

    def tape_forward(self, nsteps, checkpoint_every=8):
        self._ck(self._L.dob_tape_forward(self._h, int(nsteps), int(checkpoint_every)), "dob_tape_forward")

    def tape_backward(self, dye_grad):
        shape, _ = self.field_shape(abi.FIELD_ADJ_CONC)
        g = np.ascontiguousarray(dye_grad, dtype=np.float32).reshape(shape)
        self._ck(self._L.dob_tape_backward(self._h, _fptr(g), g.nbytes), "dob_tape_backward")

    def gradients(self):
        """d loss / d (initial u, v, w, dye, pressure) after tape_backward."""
        return {"u": self.get_field(abi.FIELD_ADJ_VEL_U), "v": self.get_field(abi.FIELD_ADJ_VEL_V),
                "w": self.get_field(abi.FIELD_ADJ_VEL_W), "dye": self.get_field(abi.FIELD_ADJ_CONC),
                "p": self.get_field(abi.FIELD_ADJ_PRESSURE)}

    def sphere_impulse(self, center, radius, vel) -> float:
        c = (C.c_float * 3)(*center)
        v = (C.c_float * 3)(*vel)
        out = C.c_double(0.0)
        self._ck(self._L.dob_adjoint_sphere_impulse(self._h, c, C.c_float(radius), v, C.byref(out)),
                 "dob_adjoint_sphere_impulse")
        return out.value

    def sphere_soft_grad(self, center, radius, edge, dye, vel, noise_sigma=0.0, seed=0):
        """(d loss / d s at s = 1 for injected velocity s vel, d loss / d centre[3])
        of a soft drop, from the adjoint fields (dob_adjoint_sphere_soft)."""
        c = np.asarray(center, dtype=np.float32)
        v = np.asarray(vel, dtype=np.float32)
        out = (C.c_double * 4)()
        self._ck(self._L.dob_adjoint_sphere_soft(self._h, _fptr(c), float(radius), float(edge), float(dye), _fptr(v),
                                                 float(noise_sigma), int(seed), out), "dob_adjoint_sphere_soft")
        return out[0], np.array(out[1:4], dtype=np.float64)

    def save_state(self, slot):
        self._ck(self._L.dob_save_state(self._h, int(slot)), "dob_save_state")

    def load_state(self, slot):
        self._ck(self._L.dob_load_state(self._h, int(slot)), "dob_load_state")


def eval_math(fn: int, x, y=None) -> np.ndarray:
    """Evaluate the library's own elementary function `fn` on the device."""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
    out = np.empty_like(x)
    rc = L.dob_eval_math(int(fn), _fptr(x), None if yy is None else _fptr(yy), _fptr(out), x.size)
    check(rc, "dob_eval_math")
    return out
