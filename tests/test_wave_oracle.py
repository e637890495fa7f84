"""The oracle's 512x512 wave solver (wave.ts:55-388): its radix-2 passes
against numpy's FFT (an independent statement of the same transform), still
water staying still, a drop at the surface excavating a crater and laying a
surfactant film, and the wave texture holding half-precision values."""
import numpy as np

from dropfluid import abi

# float32 radix-2 with nine stages on O(1) data: a few ulps of the largest
# coefficient
FFT_TOL = 1e-5


def _ref_cfg(flags):
    c = abi.config_reference()
    c.nx, c.ny, c.nz = 16, 24, 16
    c.mg_levels = 2
    c.parcel_capacity = 1024
    c.physics_flags = flags
    return c


def _drop_block():
    from dropfluid import uniforms as U
    snap = U.DropSnapshot(sim_time=0.4, active_count=1)
    snap.slots[0] = U.DropSlot(active=True, center=(0.03, 0.285, -0.02), radius=0.05, vel_y=-0.3,
                               oscillation=0.01, vol_drain_rate=0.42, seed=1.5)
    return U.SimUniformPacker().pack(drops=snap, dt=1.0 / 60.0, global_seed=1.5).copy()


def test_wave_fft_matches_numpy(oracle_mod):
    rng = np.random.default_rng(0)
    z = (rng.standard_normal((512, 512)) + 1j * rng.standard_normal((512, 512))).astype(np.complex64)
    z64 = z.astype(np.complex128)
    fwd = oracle_mod.wave_fft2(z)
    inv = oracle_mod.wave_fft2(z, inverse=True)
    assert np.abs(fwd - np.fft.fft2(z64) / 512).max() < FFT_TOL
    assert np.abs(inv - np.fft.ifft2(z64) * 512).max() < FFT_TOL
    assert np.abs(oracle_mod.wave_fft2(fwd, inverse=True) - z).max() < FFT_TOL


def test_still_water_stays_still(oracle_mod):
    o = oracle_mod.OracleSim(_ref_cfg(abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE))
    o.reset()
    for _ in range(3):
        o.wave_step()
    assert not np.any(o.get_field(abi.FIELD_WAVE))


def test_drop_excavates_crater_and_film(oracle_mod):
    o = oracle_mod.OracleSim(_ref_cfg(abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE))
    o.set_uniforms(_drop_block())
    o.reset()
    for _ in range(4):
        o.wave_step()
    w = o.get_field(abi.FIELD_WAVE).reshape(512, 512, 4)
    # texel of the drop centre (x 0.03, z -0.02) on the 3.2 m wave grid
    ix = int((0.03 + 1.6) / 3.2 * 512)
    iz = int((-0.02 + 1.6) / 3.2 * 512)
    assert w[iz, ix, 0] < 0.0 and w[iz, ix, 1] < 0.0      # the impulse pushes the surface down
    assert w[iz, ix, 3] > 0.05                            # surfactant film under the drop
    assert w[10, 10, 3] == 0.0                            # none at the far corner
    assert np.all(w == w.astype(np.float16).astype(np.float32))  # rgba16float texture
    # the propagation keeps the field real and drops the mean: the surface
    # integral of eta stays small against its magnitude
    assert abs(float(w[..., 0].astype(np.float64).mean())) < 1e-2 * float(np.abs(w[..., 0]).max())


def test_wave_step_inside_step_only_with_flag(oracle_mod):
    blk = _drop_block()
    on = oracle_mod.OracleSim(_ref_cfg(abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE))
    off = oracle_mod.OracleSim(_ref_cfg(abi.DOB_PHYS_REFERENCE_ALL))
    for o in (on, off):
        o.set_uniforms(blk)
        o.reset()
        o.step(1)
    assert np.any(on.get_field(abi.FIELD_WAVE))
    assert not np.any(off.get_field(abi.FIELD_WAVE))
