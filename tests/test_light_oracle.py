"""The oracle's light volume and brick passes (lighting.ts:19-240) on the
host: the properties the reference's shader comments state, checked on
small reference-mode grids (no GPU)."""
import numpy as np
import pytest

from dropfluid import abi
from dropfluid import uniforms as U


def _cfg(nx=32, ny=48, nz=32):
    c = abi.config_reference()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.mg_levels = 3
    c.parcel_capacity = 256
    return c


def _sim(oracle_mod, conc=None, block=None):
    cfg = _cfg()
    o = oracle_mod.OracleSim(cfg)
    o.set_uniforms(U.default_block() if block is None else block)
    o.reset()
    if conc is not None:
        o.set_field(abi.FIELD_CONC, conc)
    o.light_volume()
    return cfg, o


def _blob(cfg, center_uvw, radius_uvw, value=0.8, channel=0):
    r = cfg.dye_refine
    nz, ny, nx = cfg.nz * r, cfg.ny * r, cfg.nx * r
    z, y, x = np.meshgrid(*[(np.arange(n) + 0.5) / n for n in (nz, ny, nx)], indexing="ij")
    d2 = (x - center_uvw[0]) ** 2 + (y - center_uvw[1]) ** 2 + (z - center_uvw[2]) ** 2
    conc = np.zeros((nz, ny, nx, 4), np.float32)
    conc[..., channel] = np.where(d2 < radius_uvw ** 2, value, 0.0)
    return conc


def test_empty_tank_is_fully_lit_and_unoccupied(oracle_mod):
    cfg, o = _sim(oracle_mod)
    light = o.get_field(abi.FIELD_LIGHT)
    assert light.shape == (cfg.nz, cfg.ny, cfg.nx, 4)
    np.testing.assert_array_equal(light[..., 0], 1.0)
    np.testing.assert_array_equal(light[..., 1], 1.0)
    np.testing.assert_array_equal(light[..., 2:], 0.0)
    assert not o.get_field(abi.FIELD_BRICKS_RAW).any() and not o.get_field(abi.FIELD_BRICKS).any()


def test_blob_shadows_lights_and_occupies_bricks(oracle_mod):
    cfg = _cfg()
    conc = _blob(cfg, (0.5, 0.55, 0.5), 0.12)
    _, o = _sim(oracle_mod, conc)
    light = o.get_field(abi.FIELD_LIGHT)
    # every stored value is a binary16 (rgba16float texture)
    np.testing.assert_array_equal(light, light.astype(np.float16).astype(np.float32))
    cz, cy, cx = cfg.nz // 2, int(0.55 * cfg.ny), cfg.nx // 2
    assert light[cz, cy, cx, 3] > 0.5           # filtered total inside the blob
    assert light[cz, cy, cx, 2] > 0.0           # intact cells scatter
    # the key light comes from above: a voxel under the blob is in its
    # shadow, one the same distance above it is not
    below, above = light[cz, cy - 12, cx, 0], light[cz, cy + 12, cx, 0]
    assert light[cz, cy - 12, cx, 3] < 2.8e-5 and below == 1.0  # empty voxels are stored as fully lit
    inside_low = light[cz, cy - 4, cx, 0]
    inside_high = light[cz, cy + 4, cx, 0]
    assert inside_low < inside_high <= 1.38
    # outside the |x|, |z| <= 0.462 margin the voxel is not evaluated
    half = U.DOMAIN_HALF_XZ
    xs = -half + (np.arange(cfg.nx) + 0.5) / cfg.nx * 2 * half
    edge = np.abs(xs) > 0.462
    np.testing.assert_array_equal(light[:, :, edge, 0], 1.0)
    raw = o.get_field(abi.FIELD_BRICKS_RAW)
    bricks = o.get_field(abi.FIELD_BRICKS)
    assert raw.shape == (cfg.nz // 4, cfg.ny // 4, cfg.nx // 4)
    occ = light[..., 3].reshape(cfg.nz // 4, 4, cfg.ny // 4, 4, cfg.nx // 4, 4).max(axis=(1, 3, 5))
    np.testing.assert_array_equal(raw, (occ >= np.float32(0.000028)).astype(np.float32))
    # dilation: 2 within one brick (Chebyshev) of an occupied brick, 1 within two
    occupied = np.argwhere(raw > 0.5)
    assert len(occupied)
    for idx in np.ndindex(*raw.shape):
        d = np.abs(occupied - np.array(idx)).max(axis=1).min()
        assert bricks[idx] == (2.0 if d <= 1 else 1.0 if d <= 2 else 0.0), idx


def test_lysed_dye_absorbs_less_and_does_not_scatter(oracle_mod):
    """Free haemoglobin (.g) attenuates by 0.78 against 1.16 for intact cells
    (.r) and adds nothing to the multiple-scattering channel."""
    cfg = _cfg()
    lights = {}
    for ch in (0, 1):
        _, o = _sim(oracle_mod, _blob(cfg, (0.5, 0.55, 0.5), 0.12, 0.8, ch))
        lights[ch] = o.get_field(abi.FIELD_LIGHT)
    cz, cy, cx = cfg.nz // 2, int(0.55 * cfg.ny) - 4, cfg.nx // 2
    assert lights[1][cz, cy, cx, 0] > lights[0][cz, cy, cx, 0]
    assert lights[1][..., 2].max() == 0.0 and lights[0][..., 2].max() > 0.0


def test_dark_mode_and_drop_shadow(oracle_mod):
    cfg = _cfg()
    conc = _blob(cfg, (0.5, 0.4, 0.5), 0.10)
    snap = U.DropSnapshot(sim_time=0.3, active_count=1)
    blk_plain = U.SimUniformPacker().pack(drops=snap, dt=U.FIXED_SIM_DT).copy()
    # a drop above the surface on the key light's ray through the blob's centre
    key_dir = np.array([0.22, 0.95, 0.20]) / np.linalg.norm([0.22, 0.95, 0.20])
    py = U.DOMAIN_Y_MIN + 0.4 * (U.DOMAIN_Y_MAX - U.DOMAIN_Y_MIN)
    t = (0.45 - py) / key_dir[1]
    snap.slots[0] = U.DropSlot(active=True, center=(key_dir[0] * t, 0.45, key_dir[2] * t), radius=0.06,
                               vel_y=-0.1, seed=1.0)
    blk_drop = U.SimUniformPacker().pack(drops=snap, dt=U.FIXED_SIM_DT).copy()
    key = {}
    for name, blk in (("plain", blk_plain), ("drop", blk_drop)):
        _, o = _sim(oracle_mod, conc, blk)
        key[name] = o.get_field(abi.FIELD_LIGHT)[..., 0]
    # a drop hanging above the tank casts a ball-lens pattern on the key light
    assert (key["drop"] != key["plain"]).any()
    dark = blk_plain.copy()
    dark[U.OFF["lightingMode"]] = 1.0
    _, o = _sim(oracle_mod, conc, dark)
    assert (o.get_field(abi.FIELD_LIGHT)[..., 0] != key["plain"]).any()


def test_light_volume_needs_reference_mode(oracle_mod):
    cfg = abi.config_closed_box(32, 32, 32)
    cfg.mg_levels = 3
    o = oracle_mod.OracleSim(cfg)
    with pytest.raises(RuntimeError):
        o.light_volume()
