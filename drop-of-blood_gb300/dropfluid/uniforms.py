"""The reference's 512-byte SimUniforms block (src/shaders/common.ts:26-43)
and its packer (src/sim/uniformLayout.ts:6-190), restated for the host.

Only the fields the fluid step reads matter to this library; the camera
matrices [0..31] and optics fields are packed for layout fidelity.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SIM_UNIFORM_FLOATS = 128                      # uniformLayout.ts:6
SIM_UNIFORM_BYTES = SIM_UNIFORM_FLOATS * 4    # uniformLayout.ts:7
DOMAIN_HALF_XZ = 0.48                         # uniformLayout.ts:9
DOMAIN_Y_MIN = -0.98                          # uniformLayout.ts:10
WATER_SURFACE_Y = 0.30                        # dropKinematics.ts:5
DOMAIN_Y_MAX = WATER_SURFACE_Y                # uniformLayout.ts:11
FRONT_PANE_DIST = 1.10                        # uniformLayout.ts:12
MAX_ACTIVE_DROPS = 8                          # common.ts:17
FIXED_SIM_DT = 1.0 / 60.0                     # BloodDropEngine.ts:82
PARTICLE_COUNT = 393216                       # common.ts:18
PARCELS_PER_REF_DROP = 49152                  # particles.ts:12
INITIAL_PARCEL_VOXEL_MASS = 0.134             # particles.ts:14
SPLAT_FP_SCALE = 65536.0                      # common.ts:20
INITIAL_DROP_RADIUS = 0.058                   # dropKinematics.ts:7
PENDANT_MIN_RADIUS = 0.018                    # dropKinematics.ts:8

# Offsets of the fields inside the block (common.ts:31-42).
OFF = {
    "invViewProj": 0, "viewProj": 16, "cameraPos": 32, "simTime": 35,
    "viewport": 36, "dt": 38, "frameIndex": 39, "surfaceY": 40, "marangoni": 41,
    "activeCount": 42, "globalSeed": 43, "vorticityConf": 44, "buoyancy": 45,
    "velDamp": 46, "concSharpness": 47, "extinction": 48, "scatterAlbedo": 49,
    "caustic": 50, "lightingMode": 51, "halfXZ": 52, "yMin": 53, "yMax": 54,
    "frontPane": 55, "focalDistance": 56, "aperture": 57, "cassonYield": 58,
    "hemolysisRate": 59, "schlieren": 60, "spawnCursor": 61, "spawnCount": 62,
    "neckCapillaryLen": 63, "drops": 64,
}


@dataclass
class FluidOpticalConfig:
    """uniformLayout.ts:14-46 (DEFAULT_FLUID_OPTICAL_CONFIG)."""
    vorticityConfinement: float = 1.02
    buoyancyStrength: float = 0.48
    velocityDamping: float = 0.9993
    concSharpness: float = 0.995
    extinctionScale: float = 1.0
    scatterAlbedo: float = 1.0
    causticStrength: float = 1.0
    lightingMode: float = 0.0
    marangoniStrength: float = 1.0
    apertureRadius: float = 0.0032
    cassonYield: float = 1.0
    hemolysisRate: float = 0.088
    schlierenStrength: float = 0.032
    neckCapillaryLength: float = 0.028


@dataclass
class DropSlot:
    """The fields of a DropSlotState that reach the GPU (uniformLayout.ts:161-187)."""
    active: bool = False
    center: tuple = (0.0, 0.0, 0.0)
    radius: float = 0.0
    vel_y: float = 0.0
    oscillation: float = 0.0
    vol_drain_rate: float = 0.0
    pipette_presence: float = 0.0
    pendant: bool = False
    seed: float = 1.0


@dataclass
class DropSnapshot:
    sim_time: float = 0.0
    active_count: int = 0
    slots: list = field(default_factory=lambda: [DropSlot() for _ in range(MAX_ACTIVE_DROPS)])


class SimUniformPacker:
    """Zero-allocation packer: every call reuses the same 512-byte buffer
    (uniformLayout.ts:52-55; the reuse is pinned by the reference test at
    tests/simulation.test.ts:687-724)."""

    def __init__(self):
        self.buffer = bytearray(SIM_UNIFORM_BYTES)
        self.f32 = np.frombuffer(self.buffer, dtype=np.float32)

    def pack(self, *, drops: DropSnapshot, dt: float, frame_index: int = 0, global_seed: float = 1.0,
             spawn_cursor: int = 0, spawn_count: int = 0, config: FluidOpticalConfig | None = None,
             inv_view_proj=None, view_proj=None, camera_pos=(0.0, 0.0, 2.0), camera_target=(0.0, 0.0, 0.0),
             viewport_width: float = 1.0, viewport_height: float = 1.0) -> np.ndarray:
        cfg = config or FluidOpticalConfig()
        out = self.f32
        out[0:16] = np.eye(4, dtype=np.float32).ravel() if inv_view_proj is None else np.asarray(inv_view_proj).ravel()
        out[16:32] = np.eye(4, dtype=np.float32).ravel() if view_proj is None else np.asarray(view_proj).ravel()
        out[32:35] = camera_pos
        out[35] = drops.sim_time
        out[36] = max(1.0, viewport_width)
        out[37] = max(1.0, viewport_height)
        out[38] = dt
        out[39] = frame_index
        out[40] = WATER_SURFACE_Y
        out[41] = cfg.marangoniStrength
        out[42] = drops.active_count
        out[43] = global_seed
        out[44] = cfg.vorticityConfinement
        out[45] = cfg.buoyancyStrength
        out[46] = cfg.velocityDamping
        out[47] = cfg.concSharpness
        out[48] = cfg.extinctionScale
        out[49] = cfg.scatterAlbedo
        out[50] = cfg.causticStrength
        out[51] = cfg.lightingMode
        out[52] = DOMAIN_HALF_XZ
        out[53] = DOMAIN_Y_MIN
        out[54] = DOMAIN_Y_MAX
        out[55] = FRONT_PANE_DIST
        d = [camera_target[k] - camera_pos[k] for k in range(3)]
        focal = max(0.20, math.hypot(*d))
        out[56] = focal
        macro = min(1.0, math.pow(max(focal, 0.20) / 0.82, 1.25))
        out[57] = max(0.0, cfg.apertureRadius) * macro
        out[58] = cfg.cassonYield
        out[59] = cfg.hemolysisRate
        out[60] = cfg.schlierenStrength
        out[61] = spawn_cursor
        out[62] = spawn_count
        out[63] = cfg.neckCapillaryLength
        for i in range(MAX_ACTIVE_DROPS):
            base = 64 + 8 * i
            s = drops.slots[i] if i < len(drops.slots) else None
            if s is not None and s.active:
                out[base + 0:base + 3] = s.center
                out[base + 3] = s.radius
                out[base + 4] = s.vel_y
                out[base + 5] = s.oscillation
                out[base + 6] = s.vol_drain_rate if s.vol_drain_rate > 0.0 else -max(0.0, s.pipette_presence)
                out[base + 7] = -abs(s.seed) if s.pendant else abs(s.seed)
            else:
                out[base:base + 8] = 0.0
        return out


def default_block(dt: float = FIXED_SIM_DT, sim_time: float = 0.0, global_seed: float = 1.0) -> np.ndarray:
    """A block with the default config, no drops, and the given dt/time/seed."""
    p = SimUniformPacker()
    return p.pack(drops=DropSnapshot(sim_time=sim_time), dt=dt, global_seed=global_seed).copy()


def camera_matrices(eye, target, fovy_deg: float = 40.0, aspect: float = 16.0 / 9.0, near: float = 0.01,
                    far: float = 20.0):
    """(view_proj, inv_view_proj) of a right-handed look-at camera with a
    WebGPU clip range (z in [0, 1]), each 16 float32 in column-major order as
    the uniform block stores them (the block's matrices are gl-matrix mat4s);
    y is up."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    up = np.array([0.0, 1.0, 0.0]) if abs(f[1]) < 0.99 else np.array([1.0, 0.0, 0.0])
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    t = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    proj = np.zeros((4, 4))
    proj[0, 0] = t / aspect
    proj[1, 1] = t
    proj[2, 2] = far / (near - far)
    proj[2, 3] = near * far / (near - far)
    proj[3, 2] = -1.0
    vp = proj @ view
    return (vp.T.ravel().astype(np.float32), np.linalg.inv(vp).T.ravel().astype(np.float32))


def synthetic_spectral_lut(seed: int = 0) -> np.ndarray:
    """A stand-in for the renderer's 256 x 64 spectral transmittance table
    (its shape and axes: u = tau / (0.012 + 0.996 tau), v = oxygenated
    fraction; rgb transmittance falling with tau, blue and green faster than
    red), (64, 256, 4) float32.  The reference builds its table from
    tabulated absorption spectra on the host; a caller of the renderer
    passes that table instead."""
    rng = np.random.default_rng(seed)
    u = (np.arange(256) + 0.5) / 256.0
    tau = 0.012 * u / np.maximum(1.0 - 0.996 * u, 1e-6)
    v = (np.arange(64) + 0.5) / 64.0
    k = np.array([0.9, 5.5, 7.0]) * (1.0 + 0.05 * rng.standard_normal(3))
    ox = np.array([0.4, -1.2, 0.6])
    out = np.ones((64, 256, 4), np.float32)
    for c in range(3):
        out[:, :, c] = np.exp(-tau[None, :] * k[c] * (1.0 + 0.3 * ox[c] * v[:, None]))
    return out
