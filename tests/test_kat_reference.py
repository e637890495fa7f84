"""Known-answer tests taken from the reference's own test-suite
(tests/simulation.test.ts) for the pieces of this path it pins: the 512-byte
uniform layout, the parcel ring / fixed-point splat bounds, the 4-point
splat weights, the even azimuthal modes and the binary16 encoder's edge
values.  The reference's tests pin no numeric output of the step itself."""
import math

import numpy as np

from dropfluid import uniforms as U


def test_uniform_block_layout():
    """tests/simulation.test.ts:395-452 — 128 floats / 512 B with fields at
    fixed offsets, 8 drop slots, pendant seed negative."""
    assert U.SIM_UNIFORM_FLOATS == 128
    assert U.SIM_UNIFORM_BYTES == 512
    assert U.SIM_UNIFORM_BYTES % 256 == 0
    assert U.DOMAIN_Y_MAX == U.WATER_SURFACE_Y
    assert U.DOMAIN_Y_MIN == -0.98
    assert U.DOMAIN_HALF_XZ == 0.48
    snap = U.DropSnapshot(sim_time=0.25, active_count=2)
    snap.slots[0] = U.DropSlot(active=True, center=(0.03, 0.4, -0.02), radius=U.INITIAL_DROP_RADIUS,
                               vel_y=-0.1, seed=1.5)
    snap.slots[1] = U.DropSlot(active=True, center=(-0.08, 0.53, 0.06), radius=U.PENDANT_MIN_RADIUS,
                               pendant=True, seed=3.25)
    p = U.SimUniformPacker()
    out = p.pack(drops=snap, dt=1 / 60, frame_index=42, global_seed=2.5, spawn_cursor=12000, spawn_count=640,
                 viewport_width=0, viewport_height=-10, camera_pos=(0.0, 0.2, 1.6), camera_target=(0.0, 0.0, 0.0))
    assert out.nbytes == 512
    assert math.isclose(out[35], 0.25, abs_tol=1e-5)
    assert out[36] == 1 and out[37] == 1
    assert out[39] == 42
    assert math.isclose(out[40], U.WATER_SURFACE_Y, abs_tol=1e-5)
    assert out[42] == 2
    assert math.isclose(out[52], U.DOMAIN_HALF_XZ, abs_tol=1e-5)
    assert out[56] > 0.25
    assert math.isclose(out[57], U.FluidOpticalConfig().apertureRadius, abs_tol=1e-6)
    assert out[61] == 12000 and out[62] == 640
    assert math.isclose(out[64 + 0], 0.03, abs_tol=1e-5)
    assert math.isclose(out[64 + 3], U.INITIAL_DROP_RADIUS, abs_tol=1e-5)
    assert math.isclose(out[64 + 7], 1.5, abs_tol=1e-5)
    assert math.isclose(out[72 + 0], -0.08, abs_tol=1e-5)
    assert math.isclose(out[72 + 3], U.PENDANT_MIN_RADIUS, abs_tol=1e-5)
    assert math.isclose(out[72 + 7], -3.25, abs_tol=1e-5)
    # inactive slots are zero
    assert not out[80:128].any()


def test_packer_reuses_one_buffer():
    """tests/simulation.test.ts:687-724."""
    p = U.SimUniformPacker()
    a = p.pack(drops=U.DropSnapshot(), dt=1 / 60, frame_index=1)
    b = p.pack(drops=U.DropSnapshot(), dt=1 / 60, frame_index=2, spawn_cursor=128, spawn_count=64)
    assert a is b
    assert a.base is not None and np.shares_memory(a, np.frombuffer(p.buffer, np.float32))


def test_parcel_ring_and_splat_overflow_bound():
    """tests/simulation.test.ts:726-736: 8 reference drops fill the ring
    exactly and u32 splat sums cannot overflow."""
    assert U.PARCELS_PER_REF_DROP * U.MAX_ACTIVE_DROPS == U.PARTICLE_COUNT == 393216
    assert U.PARTICLE_COUNT * U.INITIAL_PARCEL_VOXEL_MASS * U.SPLAT_FP_SCALE < 0xFFFFFFFF


def test_four_point_splat_weights_partition_of_unity():
    """tests/simulation.test.ts:846-851 (weights 0.21/0.29/0.29/0.21)."""
    assert math.isclose(0.21 + 0.29 + 0.29 + 0.21, 1.0, abs_tol=1e-12)


def test_even_azimuthal_modes_have_no_dipole(oracle_mod):
    """tests/simulation.test.ts:738-768, evaluated with this library's own
    single-precision cos/sin: the m=1 Fourier projection of azim^p vanishes
    to float precision for p = 1, 2, 3."""
    n = 512
    theta = (2.0 * np.pi * np.arange(n) / n).astype(np.float32)
    for seed in (1.0, 2.718, 5.13):
        a1 = oracle_mod.eval_math(1, (4.0 * theta + seed * 1.73).astype(np.float32)).astype(np.float64)
        a2 = oracle_mod.eval_math(1, (6.0 * theta - seed * 2.31).astype(np.float32)).astype(np.float64)
        a3 = oracle_mod.eval_math(0, (8.0 * theta + seed * 0.89).astype(np.float32)).astype(np.float64)
        azim = 1.0 + 0.058 * a1 + 0.044 * a2 + 0.028 * a3
        c = oracle_mod.eval_math(1, theta).astype(np.float64)
        s = oracle_mod.eval_math(0, theta).astype(np.float64)
        for pw in (1, 2, 3):
            f = azim ** pw
            assert abs((f * c).mean()) < 1e-6
            assert abs((f * s).mean()) < 1e-6


def test_binary16_encoder_edge_values(oracle_mod):
    """tests/simulation.test.ts:676-685 edge values through the library's
    binary16 store rounding.  One deliberate difference: the reference's LUT
    encoder saturates 999999 to 0x7bff, while an IEEE store (what an
    rgba16float texture write and this library do) rounds it to +inf."""
    x = np.array([0.0, 1.0, -1.0, 0.5, np.inf, -np.inf, np.nan, 999999.0], np.float32)
    y = oracle_mod.eval_math(7, x).astype(np.float16).view(np.uint16)
    assert list(y[:6]) == [0x0000, 0x3C00, 0xBC00, 0x3800, 0x7C00, 0xFC00]
    assert y[6] == 0x7E00
    assert y[7] == 0x7C00
