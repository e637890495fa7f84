"""Host-side drop lifecycle: up to eight drops moving through pendant ->
aerial -> coalescing, producing the per-slot state the step's uniform block
carries (centre, radius, fall speed, oscillation, drain rate or pipette
presence, signed seed) and the volume drained into the tank each substep,
from which the parcel spawn count is derived.

This restates `MultiDropSystem` of the reference
(src/sim/dropKinematics.ts:202-749) in Python double precision, which is the
arithmetic of the reference's JavaScript numbers.  The constants and the
closed-form laws (free fall, the meniscus contact time, the Rayleigh
oscillation, the pendant swelling, the two-part drainage curve, the slump
of the crater dome, merging by volume) must be the reference's for the
uniform sequences to match; the code is organised around this library's
needs.  Left out, because nothing of the fluid step reads them: the plume
trackers and inspection subjects (camera focus) and the phase label (UI).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

from .uniforms import MAX_ACTIVE_DROPS, DropSlot, DropSnapshot

# dropKinematics.ts:5-18
WATER_SURFACE_Y = 0.30
PIPETTE_TIP_Y = 0.55
INITIAL_DROP_RADIUS = 0.058
PENDANT_MIN_RADIUS = 0.018
PENDANT_MAX_RADIUS = 0.078
PENDANT_GROWTH_DURATION = 2.2
SHOT_CYCLE_DURATION = 22.0
MAX_DROP_OFFSET_XZ = 0.26
Y_START = 0.495
V_START = -0.075
G_SLOW = -0.155
REFERENCE_DROP_VOLUME = (4.0 / 3.0) * math.pi * math.pow(INITIAL_DROP_RADIUS, 3)  # dropKinematics.ts:20
BASE_COALESCE_DURATION = 1.26                                               # dropKinematics.ts:21


def _clamp(v, lo, hi):
    return lo if v < lo else hi if v > hi else v


def _smoothstep(e0, e1, x):
    t = _clamp((x - e0) / (e1 - e0), 0.0, 1.0)
    return t * t * (3.0 - 2.0 * t)


def _finite_or(v, alt):
    return v if isinstance(v, (int, float)) and math.isfinite(v) else alt


def _impact_time() -> float:
    """Contact time of the first drop's bottom with the meniscus: the earlier
    root of y0 + v0 t + g t^2 / 2 - R0 = surface (dropKinematics.ts:24-30)."""
    a, b = 0.5 * G_SLOW, V_START
    c = Y_START - INITIAL_DROP_RADIUS - WATER_SURFACE_Y
    disc = max(0.0, b * b - 4.0 * a * c)
    return (-b - math.sqrt(disc)) / (2.0 * a)


IMPACT_TIME = _impact_time()


def sphere_volume(radius: float) -> float:
    r = max(0.0, radius)
    return (4.0 / 3.0) * math.pi * r * r * r


def radius_from_volume(volume: float) -> float:
    return 0.0 if volume <= 0.0 else math.cbrt((3.0 * volume) / (4.0 * math.pi))


def clamp_drop_disk_xz(x: float, z: float, max_r: float = MAX_DROP_OFFSET_XZ):
    """Non-finite offsets become 0; offsets beyond max_r are scaled onto the
    disk edge (dropKinematics.ts:50-59)."""
    sx, sz = _finite_or(x, 0.0), _finite_or(z, 0.0)
    r = math.hypot(sx, sz)
    if r <= max_r or r < 1e-8:
        return sx, sz
    s = max_r / r
    return sx * s, sz * s


def rayleigh_oscillation(age: float, radius: float, seed: float, boost: float) -> float:
    """Damped l=2 and l=3 shape modes plus late aerodynamic flattening
    (dropKinematics.ts:182-192)."""
    ratio = math.pow(INITIAL_DROP_RADIUS / max(radius, 0.020), 1.5)
    w2, w3 = 9.6 * ratio, 18.4 * ratio
    damp = math.exp(-age * 0.36)
    a2, a3 = 0.092 + boost, 0.022 + 0.35 * boost
    flat = -0.020 * _smoothstep(0.25, 0.90, age)
    return (a2 * math.cos(age * w2 + seed) + a3 * math.sin(age * w3 + seed * 1.7)) * damp + flat


def _coalesce_duration(radius: float) -> float:
    return _clamp(BASE_COALESCE_DURATION * (radius / INITIAL_DROP_RADIUS), 0.48, 1.54)


INACTIVE, PENDANT, AERIAL, COALESCING = "inactive", "pendant", "aerial", "coalescing"


@dataclass
class DropState:
    """One drop slot (DropSlotState, dropKinematics.ts:104-130)."""
    active: bool = False
    mode: str = INACTIVE
    center: list = field(default_factory=lambda: [0.0, Y_START, 0.0])
    vel: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    radius: float = 0.0
    impact_radius: float = 0.0
    impact_vel_y: float = 0.0
    volume: float = 0.0                 # aerialVolume
    coalesce_volume0: float = 0.0       # initialCoalesceVolume
    age: float = 0.0                    # ageInPhase
    coalesce_duration: float = BASE_COALESCE_DURATION
    oscillation: float = 0.0
    osc_boost: float = 0.0
    osc_at_contact: float = 0.0
    vol_drain_rate: float = 0.0         # -dV/dt / REFERENCE_DROP_VOLUME
    step_drained: float = 0.0           # volume drained during the last step
    pipette_presence: float = 0.0
    auto_release_volume: float = 0.0
    seed: float = 1.0

    def clear(self):
        """clearSlot (dropKinematics.ts:233-245): position, velocity and seed stay."""
        self.active = False
        self.mode = INACTIVE
        self.radius = 0.0
        self.volume = 0.0
        self.coalesce_volume0 = 0.0
        self.vol_drain_rate = 0.0
        self.step_drained = 0.0
        self.pipette_presence = 0.0
        self.auto_release_volume = 0.0
        self.oscillation = 0.0
        self.osc_boost = 0.0

    def gpu_slot(self) -> DropSlot:
        """The DropGpuSlot fields the packer writes (uniformLayout.ts:161-187)."""
        return DropSlot(active=self.active, center=tuple(self.center), radius=self.radius, vel_y=self.vel[1],
                        oscillation=self.oscillation, vol_drain_rate=self.vol_drain_rate,
                        pipette_presence=self.pipette_presence, pendant=self.mode == PENDANT, seed=self.seed)


@dataclass
class StepResult:
    """What one step hands to the engine: the drops as the GPU sees them and
    the volume drained into the tank (MultiDropSnapshot's fields the step
    uses)."""
    sim_time: float
    active_count: int
    drained_volume: float
    snapshot: DropSnapshot


class MultiDropSystem:
    """Concurrent drops with pendant swelling, free fall, meniscus contact,
    coalescence and volume-conserving drainage (dropKinematics.ts:202-749)."""

    def __init__(self, seed: float = 1.0, offset_xz=(0.0, 0.0)):
        self.slots = [DropState() for _ in range(MAX_ACTIVE_DROPS)]
        self.sim_time = 0.0
        self.last_spawn_time = 0.0
        self._pendant = -1
        self._recycled_volume = 0.0
        self.reset(seed, offset_xz)

    # ---- slots ---------------------------------------------------------------------------------
    def _acquire(self) -> int:
        """A free slot, else the non-pendant slot with the least volume, whose
        remaining volume is carried into the next draining step
        (dropKinematics.ts:248-270)."""
        for i, s in enumerate(self.slots):
            if not s.active:
                return i
        best, smallest = 0, math.inf
        for i, s in enumerate(self.slots):
            if i != self._pendant and s.volume < smallest:
                smallest, best = s.volume, i
        ev = self.slots[best]
        if ev.active and ev.mode != PENDANT and ev.volume > 0.0:
            self._recycled_volume += ev.volume
            ev.volume = 0.0
        return best

    def reset(self, seed: float = 1.0, offset_xz=(0.0, 0.0)) -> StepResult:
        """All slots cleared, then the first drop released from the pipette
        height (dropKinematics.ts:272-285)."""
        self.sim_time = 0.0
        self.last_spawn_time = 0.0
        self._pendant = -1
        self._recycled_volume = 0.0
        for s in self.slots:
            s.clear()
        hero = self.spawn_aerial_drop(offset_xz, INITIAL_DROP_RADIUS, seed, Y_START, V_START)
        hero.pipette_presence = 1.0
        return self._result(0.0)

    def spawn_aerial_drop(self, offset_xz, radius=INITIAL_DROP_RADIUS, seed=1.0, start_y=Y_START,
                          vel_y=V_START) -> DropState:
        """dropKinematics.ts:354-392."""
        s = self.slots[self._acquire()]
        cx, cz = clamp_drop_disk_xz(offset_xz[0], offset_xz[1])
        r = _clamp(radius, PENDANT_MIN_RADIUS, 0.095)
        vol = sphere_volume(r)
        s.active, s.mode = True, AERIAL
        s.center[:] = [cx, start_y, cz]
        s.vel[:] = [0.0, vel_y, 0.0]
        s.radius = s.impact_radius = r
        s.impact_vel_y = vel_y
        s.volume = s.coalesce_volume0 = vol
        s.age = 0.0
        s.coalesce_duration = _coalesce_duration(r)
        s.osc_boost = 0.024
        s.oscillation = rayleigh_oscillation(0.0, r, seed, s.osc_boost)
        s.osc_at_contact = s.oscillation
        s.vol_drain_rate = s.step_drained = 0.0
        s.pipette_presence = s.auto_release_volume = 0.0
        s.seed = max(0.5, abs(seed))
        self.last_spawn_time = self.sim_time
        return s

    def begin_pendant_drop(self, offset_xz, seed=1.0) -> DropState:
        """A drop hanging from the pipette tip; an earlier pendant drop is
        released (quick squeeze) or cancelled (dropKinematics.ts:398-440)."""
        if self.has_active_pendant_drop():
            if self.slots[self._pendant].auto_release_volume > 0.0:
                self.release_pendant_drop()
            else:
                self.cancel_pendant_drop()
        idx = self._acquire()
        self._pendant = idx
        s = self.slots[idx]
        cx, cz = clamp_drop_disk_xz(offset_xz[0], offset_xz[1])
        r = PENDANT_MIN_RADIUS
        s.active, s.mode = True, PENDANT
        s.center[:] = [cx, PIPETTE_TIP_Y - 1.04 * r, cz]
        s.vel[:] = [0.0, 0.0, 0.0]
        s.radius = s.impact_radius = r
        s.impact_vel_y = 0.0
        s.volume = s.coalesce_volume0 = sphere_volume(r)
        s.age = 0.0
        s.coalesce_duration = _coalesce_duration(r)
        s.osc_boost = 0.0
        s.oscillation = s.osc_at_contact = 0.03
        s.vol_drain_rate = s.step_drained = 0.0
        s.pipette_presence = 1.0
        s.auto_release_volume = 0.0
        s.seed = max(0.5, abs(seed))
        return s

    def begin_quick_pipette_drop(self, offset_xz, target_radius=INITIAL_DROP_RADIUS, seed=1.0) -> DropState:
        """A pendant drop squeezed out in 0.15 s (dropKinematics.ts:446-455)."""
        s = self.begin_pendant_drop(offset_xz, seed)
        s.auto_release_volume = sphere_volume(_clamp(target_radius, 0.030, PENDANT_MAX_RADIUS))
        return s

    def update_pendant_drop(self, dt_real: float) -> bool:
        """Volume grows linearly to the pinch-off volume (or the quick
        squeeze's target); the bulb sags below the tip; reaching the volume
        releases the drop.  True when it pinched off (dropKinematics.ts:463-500)."""
        if self._pendant < 0:
            return False
        s = self.slots[self._pendant]
        if not s.active or s.mode != PENDANT:
            self._pendant = -1
            return False
        s.age += max(0.0, _finite_or(dt_real, 0.0))
        v_min = sphere_volume(PENDANT_MIN_RADIUS)
        quick = s.auto_release_volume > 0.0
        v_target = max(v_min + 1e-8, s.auto_release_volume) if quick else sphere_volume(PENDANT_MAX_RADIUS)
        frac = min(1.0, s.age / (0.15 if quick else PENDANT_GROWTH_DURATION))
        vol = v_min + (v_target - v_min) * frac
        r = radius_from_volume(vol)
        s.radius = s.impact_radius = r
        s.volume = s.coalesce_volume0 = vol
        s.pipette_presence = 1.0
        bond = _smoothstep(0.12, 1.0, frac)
        osc = 0.03 + (0.14 if quick else 0.24) * bond * bond
        s.oscillation = osc
        s.center[1] = PIPETTE_TIP_Y - r * (1.01 + osc) - 0.036 * bond * bond
        if frac >= 1.0 - 1e-6:
            self.release_pendant_drop()
            return True
        return False

    def release_pendant_drop(self):
        """The neck snaps: the drop falls with a small downward speed and a
        recoil boost of its shape modes (dropKinematics.ts:505-526)."""
        if self._pendant < 0:
            return None
        s = self.slots[self._pendant]
        self._pendant = -1
        if not s.active or s.mode != PENDANT:
            return None
        quick = s.auto_release_volume > 0.0
        s.auto_release_volume = 0.0
        s.mode = AERIAL
        s.vel[1] = -0.068 if quick else -0.042
        s.age = 0.0
        s.osc_boost = 0.062
        s.oscillation = rayleigh_oscillation(0.0, s.radius, s.seed, s.osc_boost)
        s.coalesce_duration = _coalesce_duration(s.radius)
        s.pipette_presence = 1.0
        self.last_spawn_time = self.sim_time
        return s

    def cancel_pendant_drop(self):
        if self._pendant < 0:
            return
        self.slots[self._pendant].clear()
        self._pendant = -1

    def has_active_pendant_drop(self) -> bool:
        return self._pendant >= 0 and self.slots[self._pendant].active

    def has_auto_squeeze_pendant_drop(self) -> bool:
        return self.has_active_pendant_drop() and self.slots[self._pendant].auto_release_volume > 0.0

    def effective_cycle_duration(self, base=SHOT_CYCLE_DURATION) -> float:
        """dropKinematics.ts:757-762."""
        return base if self.last_spawn_time <= 0.0 else max(base, self.last_spawn_time + 9.0)

    # ---- time stepping ------------------------------------------------------------------------
    def _drain(self, s: DropState, dt: float):
        """Coalescing drop: 62 % of the volume drains over the first 62 % of
        the coalescence time (a cubic core), 38 % over all of it (a wake);
        the dome slumps into the crater (dropKinematics.ts:550-602)."""
        if dt <= 0.0:
            return
        prev = s.volume
        s.age += dt
        s.pipette_presence = 0.0
        u = _clamp(s.age / max(s.coalesce_duration, 0.08), 0.0, 1.0)
        uc = _clamp(u / 0.62, 0.0, 1.0)
        om_c, om_w = 1.0 - uc, 1.0 - u
        core = om_c * om_c * om_c * (1.0 + 3.0 * uc)
        wake = om_w * om_w * (1.0 + 0.65 * u)
        nxt = 0.0 if u >= 0.9999 else s.coalesce_volume0 * (0.62 * core + 0.38 * wake)
        s.volume = nxt
        s.step_drained += max(0.0, prev - nxt)
        s.radius = radius_from_volume(nxt) if nxt > 0.0 else 0.0
        tau = _clamp(0.20 * (s.impact_radius / INITIAL_DROP_RADIUS), 0.14, 0.24)
        sn = min(1.0, s.age / tau)
        slump = _smoothstep(0.0, 1.0, sn)
        v_imp = min(s.impact_vel_y, -0.18)
        s.vel[1] = v_imp * (1.0 - 0.78 * _smoothstep(0.0, 1.0, u))
        s.center[1] = (WATER_SURFACE_Y + s.impact_radius + v_imp * min(s.age, tau)
                       - 1.98 * s.impact_radius * slump * slump - 0.095 * max(0.0, s.age - tau))
        s.oscillation = ((s.osc_at_contact * (1.0 - _smoothstep(0.0, 0.35, sn)) - 0.14 * math.sin(sn * math.pi))
                         * (1.0 - slump))
        if u >= 0.9999 or s.radius <= 1e-5:
            s.active, s.mode = False, INACTIVE
            s.radius = s.volume = s.oscillation = 0.0

    def _merge(self):
        """Drops closer than 0.88 (Ra + Rb) merge by volume: volume-weighted
        centre and velocity, R = (Ra^3 + Rb^3)^(1/3); a merge with a
        coalescing drop restarts the coalescence (dropKinematics.ts:620-666)."""
        for i in range(MAX_ACTIVE_DROPS):
            a = self.slots[i]
            if not a.active or a.mode == PENDANT:
                continue
            for j in range(i + 1, MAX_ACTIVE_DROPS):
                b = self.slots[j]
                if not b.active or b.mode == PENDANT:
                    continue
                d = math.hypot(b.center[0] - a.center[0], b.center[1] - a.center[1], b.center[2] - a.center[2])
                if d >= 0.88 * (a.radius + b.radius):
                    continue
                vsum = a.volume + b.volume
                if vsum > 1e-12:
                    wa, wb = a.volume / vsum, b.volume / vsum
                    for k in range(3):
                        a.center[k] = a.center[k] * wa + b.center[k] * wb
                        a.vel[k] = a.vel[k] * wa + b.vel[k] * wb
                    a.volume = vsum
                    a.radius = radius_from_volume(vsum)
                    a.osc_boost = min(0.11, a.osc_boost + 0.065)
                    a.pipette_presence = max(a.pipette_presence, b.pipette_presence)
                    if a.mode == COALESCING or b.mode == COALESCING:
                        a.mode = COALESCING
                        a.impact_radius = a.radius
                        a.impact_vel_y = min(a.vel[1], -0.12)
                        a.coalesce_volume0 = vsum
                        a.age = 0.0
                        a.coalesce_duration = _coalesce_duration(a.radius)
                        a.osc_at_contact = a.oscillation
                        a.pipette_presence = 0.0
                b.clear()

    def _fall(self, s: DropState, dt: float):
        """Free fall; on the step that reaches the meniscus the exact contact
        time splits the step into fall and coalescence
        (dropKinematics.ts:674-728)."""
        y0, v0, r0 = s.center[1], s.vel[1], s.radius
        y1 = y0 + v0 * dt + 0.5 * G_SLOW * dt * dt
        if y1 - r0 <= WATER_SURFACE_Y:
            t_air = 0.0
            if y0 - r0 > WATER_SURFACE_Y:
                qa, qb, qc = 0.5 * G_SLOW, v0, y0 - r0 - WATER_SURFACE_Y
                disc = max(0.0, qb * qb - 4.0 * qa * qc)
                t_air = _clamp((-qb - math.sqrt(disc)) / (2.0 * qa), 0.0, dt)
            osc = rayleigh_oscillation(s.age + t_air, r0, s.seed, s.osc_boost)
            s.center[0] += s.vel[0] * t_air
            s.center[1] = WATER_SURFACE_Y + r0
            s.center[2] += s.vel[2] * t_air
            s.vel[1] = v0 + G_SLOW * t_air
            s.mode = COALESCING
            s.impact_radius = r0
            s.impact_vel_y = s.vel[1]
            s.coalesce_volume0 = s.volume
            s.age = 0.0
            s.coalesce_duration = _coalesce_duration(r0)
            s.oscillation = s.osc_at_contact = osc
            s.pipette_presence = 0.0
            self._drain(s, dt - t_air)
        else:
            s.center[0] += s.vel[0] * dt
            s.center[1] = y1
            s.center[2] += s.vel[2] * dt
            s.vel[1] = v0 + G_SLOW * dt
            s.age += dt
            s.oscillation = rayleigh_oscillation(s.age, r0, s.seed, s.osc_boost)
            s.vol_drain_rate = 0.0
            if s.pipette_presence > 0.0:
                s.pipette_presence = max(0.0, s.pipette_presence - dt / 0.24)

    def step(self, dt: float) -> StepResult:
        """Advance every released drop by dt (dropKinematics.ts:608-749).
        A zero, negative or non-finite dt changes nothing but the per-step
        drainage, which is cleared."""
        dt = max(0.0, dt) if isinstance(dt, (int, float)) and math.isfinite(dt) else 0.0
        self.sim_time += dt
        for s in self.slots:
            s.step_drained = 0.0
            if not s.active:
                s.vol_drain_rate = 0.0
        if dt <= 0.0:
            return self._result(0.0)
        self._merge()
        drained = 0.0
        for s in self.slots:
            if not s.active or s.mode == PENDANT:
                s.vol_drain_rate = 0.0
                continue
            if s.mode == AERIAL:
                self._fall(s, dt)
            elif s.mode == COALESCING:
                self._drain(s, dt)
            s.vol_drain_rate = s.step_drained / (dt * REFERENCE_DROP_VOLUME) if dt > 1e-8 else 0.0
            drained += s.step_drained
        if self._recycled_volume > 0.0 and drained > 1e-9:
            drained += self._recycled_volume
            self._recycled_volume = 0.0
        return self._result(drained)

    def snapshot(self) -> StepResult:
        return self._result(0.0)

    def _result(self, drained: float) -> StepResult:
        snap = DropSnapshot(sim_time=self.sim_time, active_count=sum(1 for s in self.slots if s.active),
                            slots=[s.gpu_slot() for s in self.slots])
        return StepResult(self.sim_time, snap.active_count, drained, snap)
