"""The physics side of the reference engine's frame loop: what
`BloodDropEngine` does on the host between two fluid steps, so that a
reference-mode context sees the uniform blocks and parcel spawn counts the
reference would give it.

* `reset_simulation` (BloodDropEngine.ts:1682-1763): time, spawn cursor,
  high-water mark and fractional parcel carry to zero, the drop seed set or
  advanced, the drop system reset (one drop released from the pipette
  height), and the block the reset's velocity initialisation reads;
* `advance_substep` (BloodDropEngine.ts:1821-1844): one drop-system step,
  then spawnCount = floor(drained / V_ref * 49152 + carry) capped at 8192,
  the carry kept, the cursor advanced modulo the ring and the high-water
  mark raised; the block packs the cursor from before the advance;
* `seek_blocks` (BloodDropEngine.ts:2142-2179): the blocks of the fixed
  1/60 s substeps that reach a target time, with the auto-squeezed pendant
  drop updated before each;
* drop triggers (BloodDropEngine.ts:1572-1783): `trigger_additional_drop`,
  `spawn_drop`, `begin_pendant_drop`, `release_pendant_drop`, with the
  engine's seed sequence.

Screen raycasting, the camera, the renderer and the auto-loop are not part
of the fluid step and are left to the caller (drops are placed by their
x/z offset on the meniscus).
"""
from __future__ import annotations

import math

import numpy as np

from . import kinematics as K
from .uniforms import (FIXED_SIM_DT, PARCELS_PER_REF_DROP, PARTICLE_COUNT, FluidOpticalConfig,
                       SimUniformPacker)

MAX_SPAWN_PER_SUBSTEP = 8192  # BloodDropEngine.ts:1835 (PARTICLE_EMIT's per-substep limit)


class SubstepSequencer:
    """Host state of the reference engine that feeds the fluid step."""

    def __init__(self, config: FluidOpticalConfig | None = None, parcel_capacity: int = PARTICLE_COUNT,
                 seed: float = 1.0):
        self.config = config or FluidOpticalConfig()
        self.capacity = int(parcel_capacity)
        self.drops = K.MultiDropSystem()
        self.packer = SimUniformPacker()
        self.drop_seed = 1.0
        self.sim_time = 0.0
        self.frame_index = 0
        self.spawn_cursor = 0
        self.high_water = 0
        self.parcel_carry = 0.0
        self.reset_simulation(seed)

    # ---- seeds and drops ------------------------------------------------------------------------
    def next_seed(self) -> float:
        """BloodDropEngine.ts:1572-1575."""
        self.drop_seed = math.fmod(self.drop_seed * 2.7182818 + 1.37, 100.0) + 0.5
        return self.drop_seed

    def reset_simulation(self, seed: float | None = None, offset_xz=(0.0, 0.0)) -> np.ndarray:
        """Returns the block uploaded at the reset (dt = 1/60, cursor 0,
        spawn 0), which the velocity initialisation reads (its globalSeed)."""
        self.sim_time = 0.0
        self.spawn_cursor = 0
        self.high_water = 0
        self.parcel_carry = 0.0
        if seed is not None:
            self.drop_seed = max(0.5, seed)
        else:
            self.drop_seed = math.fmod(self.drop_seed * 1.6180339 + 1.0, 100.0) + 0.5
        self.drops.reset(self.drop_seed, offset_xz)
        return self.block(FIXED_SIM_DT, 0, 0)

    def trigger_additional_drop(self, offset_xz=(0.0, 0.0), radius: float | None = None) -> K.DropState:
        """A drop of radius 0.053-0.063 (from its seed) released from the
        pipette height (BloodDropEngine.ts:1770-1783)."""
        seed = self.next_seed()
        frac = math.fmod(math.sin(seed * 12.9898) * 43758.5453, 1.0)
        unit = frac + 1.0 if frac < 0.0 else frac
        r = radius if radius is not None else 0.053 + unit * 0.010
        return self.drops.spawn_aerial_drop(offset_xz, r, seed)

    def spawn_drop(self, offset_xz, radius: float = K.INITIAL_DROP_RADIUS) -> K.DropState:
        """spawnDropAtNdc with the meniscus point given (BloodDropEngine.ts:1595-1601)."""
        return self.drops.spawn_aerial_drop(offset_xz, radius, self.next_seed())

    def begin_pendant_drop(self, offset_xz, quick_radius: float | None = None) -> K.DropState:
        """Press-and-hold pendant drop, or a quick-squeezed one of the given
        radius (BloodDropEngine.ts:1605-1640)."""
        if quick_radius is None:
            return self.drops.begin_pendant_drop(offset_xz, self.next_seed())
        return self.drops.begin_quick_pipette_drop(offset_xz, quick_radius, self.next_seed())

    def release_pendant_drop(self):
        return self.drops.release_pendant_drop()

    # ---- blocks ---------------------------------------------------------------------------------
    def block(self, dt: float, cursor: int, spawn: int, result: K.StepResult | None = None) -> np.ndarray:
        res = result or self.drops.snapshot()
        return self.packer.pack(drops=res.snapshot, dt=dt, frame_index=self.frame_index,
                                global_seed=self.drop_seed, spawn_cursor=cursor, spawn_count=spawn,
                                config=self.config).copy()

    def advance_substep(self, dt: float = FIXED_SIM_DT):
        """One substep's host work: returns (block, spawn_count, drop step result)."""
        self.frame_index += 1
        res = self.drops.step(dt)
        self.sim_time = res.sim_time
        exact = res.drained_volume / K.REFERENCE_DROP_VOLUME * PARCELS_PER_REF_DROP + self.parcel_carry
        spawn = min(MAX_SPAWN_PER_SUBSTEP, max(0, math.floor(exact)))
        self.parcel_carry = max(0.0, exact - spawn)
        before = self.spawn_cursor
        self.spawn_cursor = (self.spawn_cursor + spawn) % self.capacity
        self.high_water = min(self.capacity, self.high_water + spawn)
        return self.block(dt, before, spawn, res), spawn, res

    def seek_blocks(self, target_time: float) -> list:
        """Blocks of the fixed substeps from the current time to
        `target_time` (BloodDropEngine.ts:2150-2158)."""
        n = max(0, math.floor((target_time - self.sim_time) / FIXED_SIM_DT + 0.5))  # JS Math.round
        out = []
        for _ in range(n):
            if self.drops.has_auto_squeeze_pendant_drop():
                self.drops.update_pendant_drop(FIXED_SIM_DT)
            out.append(self.advance_substep(FIXED_SIM_DT)[0])
        return out
