"""Seeded synthetic drop scenes (the benchmark configurations) and a runner
that plays them on any engine with the DropFluid interface.

Generator: SplitMix64 (Steele, Lea & Flood 2014) for uniforms in [0, 1),
Box-Muller for normals; every number is derived from the scene seed, so the
device run and the CPU restatement see identical inputs.

Scenes (velocity grid, closed box, dx = 1, dt = 0.02; "w" is the vertical
(y) velocity, given in cells/step and converted to world units as
w * dx / dt):
  box48    48x64x48, one sphere r=4 at (24,56,24), dye 1, w=-2, 8192 parcels
           uniform in the sphere (seed 0), 20 steps, 4 V-cycles of 2+2 sweeps.
  box192   192x256x192, three spheres r=12, centres uniform in the top 20 % of
           the box, released at steps 0/40/80 with w=-1.5 plus N(0, 0.05) per
           face, 393216 parcels split evenly, 200 steps.
  box192_mixed   box192 with FP16 dye and the mixed pressure solve: an
           error-free residual of the double-float pressure, then V-cycles on
           the correction (BF16 levels 2-3; three untested, then tested after
           each further cycle's finest-level pre-smoothing) until max |div|
           dt/dx <= 1e-5
           (box192_mixed_1e8: also ||b - A p|| / ||b|| <= 1e-8).
  box96    96x128x96, one sphere r=8 with a seeded centre, w=-1.5 plus
           N(0, 0.05) per face like box192, 32 steps (the adjoint scene:
           without the face noise a uniform drop in fluid at exact rest puts
           the dye limiter at exact ties, where the loss has no derivative).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
PARCEL_MASS = 0.134  # particles.ts:14


def splitmix64(x: np.ndarray) -> np.ndarray:
    """The SplitMix64 output function of state x + golden (vectorised, mod 2^64)."""
    with np.errstate(over="ignore"):
        z = (np.asarray(x, dtype=np.uint64) + GOLDEN).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


class SplitMix64:
    """Sequential stream: output k uses state seed + (k+1)*golden."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed)

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            k = np.arange(n, dtype=np.uint64)
            states = (self.state + k * GOLDEN).astype(np.uint64)
            out = splitmix64(states)
            self.state = (self.state + np.uint64(n) * GOLDEN).astype(np.uint64)
        return out

    def uniform(self, n: int) -> np.ndarray:
        """Doubles in [0, 1) from the top 53 bits."""
        return (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def normal(self, n: int) -> np.ndarray:
        u1 = 1.0 - self.uniform(n)  # (0, 1]
        u2 = self.uniform(n)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def parcels_in_sphere(center, radius, n, seed) -> np.ndarray:
    """n parcels uniform in the sphere (rejection sampling in the bounding cube)."""
    rng = SplitMix64(seed)
    pts = np.empty((0, 3))
    while pts.shape[0] < n:
        m = max(64, int((n - pts.shape[0]) * 2.1))
        q = (rng.uniform(3 * m).reshape(m, 3) * 2.0 - 1.0) * radius
        q = q[np.einsum("ij,ij->i", q, q) <= radius * radius]
        pts = np.concatenate([pts, q], axis=0)
    pts = pts[:n] + np.asarray(center, dtype=np.float64)
    out = np.zeros((n, 8), dtype=np.float32)
    out[:, 0:3] = pts
    out[:, 3] = PARCEL_MASS
    return out


@dataclass
class Drop:
    center: tuple
    radius: float
    w_cells_per_step: float
    noise_cells_per_step: float
    release_step: int
    seed: int
    n_parcels: int
    parcel_seed: int
    edge_cells: float = 0.0  # > 0: soft-edged additive drop (dob_inject_sphere_soft) of this edge width


@dataclass
class Scene:
    name: str
    config: abi.DobConfig
    steps: int
    drops: list = field(default_factory=list)

    def parcel_offset(self, k: int) -> int:
        return sum(d.n_parcels for d in self.drops[:k])

    def release(self, engine, k: int):
        """Inject drop k (dye + velocity) and place its parcels."""
        d = self.drops[k]
        c = self.config
        scale = c.dx / c.dt  # cells/step -> world units
        if d.edge_cells > 0.0:
            engine.inject_sphere_soft(d.center, d.radius, d.edge_cells * c.dx, 1.0,
                                      (0.0, d.w_cells_per_step * scale, 0.0), d.noise_cells_per_step * scale, d.seed)
        else:
            engine.inject_sphere(d.center, d.radius, 1.0, (0.0, d.w_cells_per_step * scale, 0.0),
                                 d.noise_cells_per_step * scale, d.seed)
        if d.n_parcels:
            engine.set_parcels(parcels_in_sphere(d.center, d.radius, d.n_parcels, d.parcel_seed),
                               self.parcel_offset(k))

    def releases_at(self, step: int):
        return [k for k, d in enumerate(self.drops) if d.release_step == step]


def run(scene: Scene, engine, steps: int | None = None, start: int = 0, stats: bool = False):
    """Play steps [start, start+steps) of the scene on `engine`; returns the
    last step's statistics when `stats` is set."""
    steps = scene.steps if steps is None else steps
    last = None
    for k in range(start, start + steps):
        for d in scene.releases_at(k):
            scene.release(engine, d)
        last = engine.step(1, stats=stats) if stats else engine.step(1)
    return last


def box48() -> Scene:
    cfg = abi.config_closed_box(48, 64, 48)
    cfg.parcel_capacity = 8192
    return Scene("box48", cfg, 20, [Drop((24.0, 56.0, 24.0), 4.0, -2.0, 0.0, 0, 1, 8192, 0)])


def box192(precision: int = abi.DOB_PREC_FP32, seed: int = 2024) -> Scene:
    cfg = abi.config_closed_box(192, 256, 192)
    cfg.precision_mode = precision
    cfg.parcel_capacity = 393216
    if precision == abi.DOB_PREC_MIXED:
        cfg.mg_cycles = 3  # V-cycles of the first round before its first convergence test
    rng = SplitMix64(seed)
    r = 12.0
    drops = []
    for k, rel in enumerate((0, 40, 80)):
        u = rng.uniform(3)
        cx = r + 1.0 + u[0] * (cfg.nx - 2 * r - 2.0)
        cy = 0.8 * cfg.ny + u[1] * (0.2 * cfg.ny - r - 1.0)
        cz = r + 1.0 + u[2] * (cfg.nz - 2 * r - 2.0)
        drops.append(Drop((float(cx), float(cy), float(cz)), r, -1.5, 0.05, rel, seed + 17 * (k + 1), 131072,
                          seed + 1000 + k))
    return Scene("box192" if precision == abi.DOB_PREC_FP32 else "box192_mixed", cfg, 200, drops)


def box96(seed: int = 7, impulse_scale: float = 1.0) -> Scene:
    cfg = abi.config_closed_box(96, 128, 96)
    cfg.parcel_capacity = 16384
    rng = SplitMix64(seed)
    r = 8.0
    u = rng.uniform(3)
    c = (r + 1.0 + u[0] * (cfg.nx - 2 * r - 2.0), 0.8 * cfg.ny + u[1] * (0.2 * cfg.ny - r - 1.0),
         r + 1.0 + u[2] * (cfg.nz - 2 * r - 2.0))
    return Scene("box96", cfg, 32, [Drop(tuple(float(v) for v in c), r, -1.5 * impulse_scale, 0.05, 0, seed + 1,
                                         16384, seed + 2)])


def box192_adjoint(impulse_scale=(1.0, 1.0, 1.0), shift=((0.0, 0.0, 0.0),) * 3, edge_cells: float = 2.0,
                   precision: int = abi.DOB_PREC_FP32) -> Scene:
    """The box192 drops, all released at step 0 as soft-edged drops (edge
    `edge_cells` wide, so the loss is differentiable in their centres), 64
    steps: the full-size forward + adjoint case.  impulse_scale / shift
    perturb each drop's velocity and centre (for targets and differences);
    precision DOB_PREC_MIXED gives the box192_mixed solve and storage."""
    sc = box192(precision)
    sc.name = "box192_adjoint" if precision == abi.DOB_PREC_FP32 else "box192_adjoint_mixed"
    sc.steps = 64
    for k, d in enumerate(sc.drops):
        d.release_step = 0
        d.edge_cells = edge_cells
        d.w_cells_per_step *= impulse_scale[k]
        d.center = tuple(float(d.center[j] + shift[k][j]) for j in range(3))
    return sc


def box192_mixed_1e8() -> Scene:
    sc = box192(abi.DOB_PREC_MIXED)
    sc.name = "box192_mixed_1e8"
    sc.config.mg_rel_tol = 1e-8
    sc.config.mg_max_outer = 32
    return sc


SCENES = {"box48": box48, "box192": box192, "box96": box96, "box192_adjoint": box192_adjoint,
          "box192_mixed": lambda: box192(abi.DOB_PREC_MIXED), "box192_mixed_1e8": box192_mixed_1e8}
