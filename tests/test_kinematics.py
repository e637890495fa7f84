"""The drop-lifecycle restatement (dropfluid.kinematics, dropKinematics.ts)
and the engine's substep sequencing (dropfluid.sequencer,
BloodDropEngine.ts:1682-1844) against the invariants the reference's own
tests pin (tests/simulation.test.ts:112-291, 864-886): impact time, monotone
descent and complete drainage, continuity across contact, pendant swelling
and cancellation, clamping, merging by volume and momentum, bad time steps,
slot recycling and volume conservation.  Host only."""
import math

import numpy as np
import pytest

from dropfluid import kinematics as K
from dropfluid import uniforms as U
from dropfluid.sequencer import SubstepSequencer


def close(a, b, digits):
    """vitest toBeCloseTo(b, digits): |a - b| < 10^-digits / 2."""
    return abs(a - b) < 0.5 * 10.0 ** (-digits)


def step_to(sys, t, dt=1 / 240):
    while sys.sim_time + dt * 0.5 < t:
        sys.step(dt)
    rem = t - sys.sim_time
    if rem > 1e-9:
        sys.step(rem)


def test_first_drop_meets_meniscus_at_impact_time():
    assert 0.8 < K.IMPACT_TIME < 1.4
    sys = K.MultiDropSystem()
    sys.reset(1.0)
    step_to(sys, K.IMPACT_TIME - 1e-5)
    s = sys.slots[0]
    assert s.mode == K.AERIAL
    assert close(s.center[1] - s.radius, K.WATER_SURFACE_Y, 3)
    assert s.vel[1] < -0.2


@pytest.mark.parametrize("r0", [K.PENDANT_MIN_RADIUS, K.INITIAL_DROP_RADIUS, K.PENDANT_MAX_RADIUS])
@pytest.mark.parametrize("dt", [1 / 60, 1 / 120])
def test_descends_and_drains_all_volume(r0, dt):
    sys = K.MultiDropSystem()
    sys.slots[0].active = False
    s = sys.spawn_aerial_drop((0.04, -0.03), r0, 1.7)
    prev_y, drained, coalesced = math.inf, 0.0, False
    for _ in range(300):
        if s.active and s.mode == K.AERIAL:
            assert s.center[1] < prev_y
            assert close(s.radius, r0, 6)
            assert abs(s.oscillation) < 0.15
            prev_y = s.center[1]
        drained += sys.step(dt).drained_volume
        if s.active and s.mode == K.COALESCING:
            coalesced = True
            if s.age >= 0.03:
                assert s.center[1] - s.radius * (1.0 + s.oscillation) < K.WATER_SURFACE_Y
    assert coalesced and not s.active and s.radius == 0.0
    assert close(drained, K.sphere_volume(r0), 9)


def test_continuous_across_contact_and_sinks():
    for seed in (0.5, 1.0, 2.718, 4.2):
        sys = K.MultiDropSystem()
        sys.reset(seed)
        step_to(sys, K.IMPACT_TIME - 1e-4)
        osc0, y0 = sys.slots[0].oscillation, sys.slots[0].center[1]
        sys.step(2e-4)
        assert sys.slots[0].mode == K.COALESCING
        assert abs(sys.slots[0].oscillation - osc0) < 1e-3
        assert abs(sys.slots[0].center[1] - y0) < 1e-3
    sys = K.MultiDropSystem()
    sys.reset(1.0)
    step_to(sys, K.IMPACT_TIME + 0.30, 1 / 120)
    assert sys.slots[0].active and sys.slots[0].center[1] < K.WATER_SURFACE_Y


def test_pendant_swells_pinches_off_and_cancels():
    sys = K.MultiDropSystem()
    p = sys.begin_pendant_drop((0.08, -0.05), 2.5)
    assert sys.has_active_pendant_drop() and p.mode == K.PENDANT
    assert close(p.radius, K.PENDANT_MIN_RADIUS, 6) and close(p.pipette_presence, 1.0, 6)
    assert sys.update_pendant_drop(0.5) is False
    assert K.PENDANT_MIN_RADIUS + 0.025 < p.radius < K.PENDANT_MAX_RADIUS
    sys.step(1 / 60)
    assert p.mode == K.PENDANT and p.step_drained == 0.0
    assert sys.update_pendant_drop(K.PENDANT_GROWTH_DURATION) is True
    assert not sys.has_active_pendant_drop()
    assert p.mode == K.AERIAL and close(p.radius, K.PENDANT_MAX_RADIUS, 5) and p.vel[1] < 0
    q = sys.begin_pendant_drop((-0.06, 0.04), 3.1)
    sys.update_pendant_drop(0.3)
    assert q.active
    sys.cancel_pendant_drop()
    assert not sys.has_active_pendant_drop() and not q.active and q.radius == 0.0


def test_eight_drops_clamping_and_midair_merge():
    sys = K.MultiDropSystem()
    c = sys.spawn_aerial_drop((0.95, -0.95), 0.055, 2.0)
    assert close(math.hypot(c.center[0], c.center[2]), K.MAX_DROP_OFFSET_XZ, 6)
    n = sys.spawn_aerial_drop((math.nan, 0.09), 0.052, 3.0)
    assert n.center[0] == 0.0 and close(n.center[2], 0.09, 6)
    for k in range(5):
        a = k * 2 * math.pi / 5
        sys.spawn_aerial_drop((0.16 * math.cos(a), 0.16 * math.sin(a)), 0.050, 4.0 + k)
    assert sys.snapshot().active_count == U.MAX_ACTIVE_DROPS

    m = K.MultiDropSystem()
    m.slots[0].active = False
    d1 = m.spawn_aerial_drop((0.0, 0.0), 0.050, 1.2, 0.48, -0.22)
    d2 = m.spawn_aerial_drop((0.01, 0.0), 0.062, 2.4, 0.46, -0.06)
    v1, v2 = K.sphere_volume(0.050), K.sphere_volume(0.062)
    res = m.step(1 / 240)
    assert res.active_count == 1 and not d2.active and d1.active
    assert close(d1.radius, K.radius_from_volume(v1 + v2), 6)
    assert close(d1.vel[1], (v1 * -0.22 + v2 * -0.06) / (v1 + v2) + -0.155 / 240, 5)
    m.sim_time = 19.0
    m.spawn_aerial_drop((0.02, -0.02), K.INITIAL_DROP_RADIUS, 5.0)
    assert m.effective_cycle_duration(K.SHOT_CYCLE_DURATION) >= 27.5


def test_bad_time_steps_change_nothing():
    sys = K.MultiDropSystem()
    y0 = sys.slots[0].center[1]
    for bad in (0.0, -0.5, math.nan):
        res = sys.step(bad)
        assert res.sim_time == 0.0 and res.drained_volume == 0.0
        assert sys.slots[0].center[1] == y0


def test_ninth_drop_recycles_smallest_and_keeps_pendant():
    sys = K.MultiDropSystem()
    pend = sys.begin_pendant_drop((0.0, 0.0), 2.0)
    tiny = sys.spawn_aerial_drop((0.18, 0.0), 0.032, 3.0)
    for i in range(5):
        a = (i + 1) * math.pi / 3
        sys.spawn_aerial_drop((0.22 * math.cos(a), 0.22 * math.sin(a)), 0.068, 4.0 + i)
    assert sys.snapshot().active_count == 8
    ninth = sys.spawn_aerial_drop((-0.15, 0.12), 0.060, 9.5)
    assert ninth is tiny
    assert sys.has_active_pendant_drop() and pend.mode == K.PENDANT


def test_volume_conserved_when_rapid_drops_recycle_slots():
    sys = K.MultiDropSystem()
    spawned, drained = K.sphere_volume(K.INITIAL_DROP_RADIUS), 0.0
    for i in range(10):
        a = i / 10 * 2 * math.pi
        sys.spawn_aerial_drop((0.24 * math.cos(a), 0.24 * math.sin(a)), 0.048, 10 + i * 1.7)
        spawned += K.sphere_volume(0.048)
        for _ in range(8):
            drained += sys.step(1 / 240).drained_volume
    for _ in range(240 * 5):
        drained += sys.step(1 / 240).drained_volume
    assert close(drained / spawned, 1.0, 5)


# ---- the engine's substep sequencing -------------------------------------------------------------
def test_reset_block_carries_seed_and_first_drop():
    seq = SubstepSequencer(seed=1.0)
    blk = seq.reset_simulation(3.25, (0.05, -0.02))
    assert blk.dtype == np.float32 and blk.size == 128
    assert blk[U.OFF["globalSeed"]] == np.float32(3.25)
    assert blk[U.OFF["dt"]] == np.float32(U.FIXED_SIM_DT)
    assert blk[U.OFF["spawnCursor"]] == 0 and blk[U.OFF["spawnCount"]] == 0
    assert blk[U.OFF["activeCount"]] == 1
    d = blk[64:72]
    assert np.allclose(d[:4], [0.05, K.Y_START, -0.02, K.INITIAL_DROP_RADIUS])
    assert d[4] == np.float32(K.V_START)
    assert d[6] == np.float32(-1.0)  # no drainage yet: -pipettePresence
    assert d[7] == np.float32(3.25)  # free drop: positive seed
    seq.reset_simulation()  # seed advanced by the golden-ratio rule
    assert math.isclose(seq.drop_seed, math.fmod(3.25 * 1.6180339 + 1.0, 100.0) + 0.5)


def test_spawn_counts_follow_drained_volume():
    """Over a whole impact the spawned parcels plus the fractional carry
    equal the drained volume in parcels (49152 per reference drop); the
    cursor and high-water mark advance by the spawn counts; each block packs
    the cursor from before its substep."""
    seq = SubstepSequencer(seed=1.0)
    total_spawn, drained, cursor = 0, 0.0, 0
    for _ in range(240):  # 4 s: impact at 0.92 s, drainage within 1.3 s of it
        blk, spawn, res = seq.advance_substep()
        assert blk[U.OFF["spawnCursor"]] == cursor and blk[U.OFF["spawnCount"]] == spawn
        assert 0 <= spawn <= 8192
        cursor = (cursor + spawn) % U.PARTICLE_COUNT
        total_spawn += spawn
        drained += res.drained_volume
    assert seq.spawn_cursor == cursor and seq.high_water == min(U.PARTICLE_COUNT, total_spawn)
    want = drained / K.REFERENCE_DROP_VOLUME * U.PARCELS_PER_REF_DROP
    assert abs(total_spawn + seq.parcel_carry - want) < 1e-6
    assert close(drained, K.sphere_volume(K.INITIAL_DROP_RADIUS), 9)
    assert total_spawn == math.floor(want + 1e-9)


def test_block_drop_slots_follow_the_lifecycle():
    """Drain rate positive while coalescing (the neck branch of the kernels),
    negative pipette presence while falling, zero when inactive."""
    seq = SubstepSequencer(seed=2.0)
    seen = set()
    for _ in range(200):
        blk, spawn, res = seq.advance_substep()
        z = float(blk[64 + 6])
        mode = seq.drops.slots[0].mode
        if mode == K.AERIAL:
            assert z <= 0.0
        elif mode == K.COALESCING:
            assert z > 0.0 and spawn >= 0
        else:
            assert np.all(blk[64:72] == 0.0)
        seen.add(mode)
    assert {K.AERIAL, K.COALESCING, K.INACTIVE} <= seen


def test_seek_blocks_and_quick_pendant():
    seq = SubstepSequencer(seed=1.0)
    seq.begin_pendant_drop((0.1, 0.0), quick_radius=0.05)
    blocks = seq.seek_blocks(0.5)
    assert len(blocks) == 30
    assert all(b[U.OFF["dt"]] == np.float32(U.FIXED_SIM_DT) for b in blocks)
    assert not seq.drops.has_active_pendant_drop()  # squeezed out within 0.15 s, then released
    assert math.isclose(seq.sim_time, 0.5, rel_tol=1e-12)
    d = seq.trigger_additional_drop((0.0, 0.1))
    assert 0.053 <= d.radius <= 0.063 and d.mode == K.AERIAL
