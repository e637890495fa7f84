"""The oracle's plume render (render.ts:1593-2109 from fsMain's camera ray,
the submerged primary march): clear-water rays leave untouched, rays through
the dye pick up optical depth, transmittance and in-scattered light, and
more dye means more depth.  Runs on the host only."""
import numpy as np
import pytest

from dropfluid import abi
from dropfluid import uniforms as U

W, H = 40, 24


def render_case(oracle_mod, scale=1.0, seed=3, lighting_mode=0.0):
    cfg = abi.config_reference()
    cfg.nx, cfg.ny, cfg.nz = 32, 48, 32
    cfg.mg_levels = 3
    cfg.parcel_capacity = 1024
    o = oracle_mod.OracleSim(cfg)
    vp, ivp = U.camera_matrices((0.05, -0.32, 1.05), (0.0, -0.36, 0.0), 40.0, W / H)
    snap = U.DropSnapshot(sim_time=0.5, active_count=0)
    oc = U.FluidOpticalConfig(lightingMode=lighting_mode)
    blk = U.SimUniformPacker().pack(drops=snap, dt=1.0 / 60.0, frame_index=7, config=oc, inv_view_proj=ivp,
                                    view_proj=vp, camera_pos=(0.05, -0.32, 1.05), camera_target=(0.0, -0.36, 0.0),
                                    viewport_width=W, viewport_height=H).copy()
    o.set_uniforms(blk)
    rng = np.random.default_rng(seed)
    nz, ny, nx = 64, 96, 64
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    r2 = ((x - 30) / 9.0) ** 2 + ((y - 42) / 16.0) ** 2 + ((z - 33) / 9.0) ** 2
    blob = np.exp(-r2 * 1.5)
    conc = np.zeros((nz, ny, nx, 4), np.float32)
    conc[..., 0] = 0.030 * scale * blob
    conc[..., 1] = 0.012 * scale * blob * (1.0 + 0.2 * rng.standard_normal(blob.shape)).clip(0.5, 1.5)
    conc[..., 2] = 0.4 * blob
    conc[..., 3] = 0.0
    o.set_field(abi.FIELD_CONC, conc)
    return o, o.render_plume(W, H, U.synthetic_spectral_lut())


def halves(img):
    return img.view(np.float16).astype(np.float32)


def test_render_clear_and_plume_pixels(oracle_mod):
    o, img = render_case(oracle_mod)
    f = halves(img)
    rad, tau, trans, taui = f[..., 0:3], f[..., 3], f[..., 4:7], f[..., 7]
    assert np.isfinite(f).all()
    hit = tau > 0
    assert hit.any() and (~hit).any()
    # a ray that gathers no depth keeps the transmittance and radiance it started with
    assert (trans[~hit] == 1.0).all() and (rad[~hit] == 0.0).all() and (taui[~hit] == 0.0).all()
    assert (trans[hit].min(axis=-1) < 1.0).all()
    assert (rad[hit].max(axis=-1) > 0.0).any()
    assert (taui <= tau + 1e-3).all()
    # the blob sits at the image centre
    assert hit[H // 2, W // 2]


def test_render_more_dye_more_depth(oracle_mod):
    _, a = render_case(oracle_mod, 1.0)
    _, b = render_case(oracle_mod, 2.0)
    ta, tb = halves(a)[..., 3], halves(b)[..., 3]
    both = (ta > 0.001) & (tb > 0.001)
    assert both.sum() > 20
    assert np.median(tb[both] / ta[both]) > 1.3


def test_render_dark_field_mode(oracle_mod):
    _, img = render_case(oracle_mod, lighting_mode=1.0)
    f = halves(img)
    assert np.isfinite(f).all() and (f[..., 3] > 0).any()


def test_camera_matrices_round_trip():
    vp, ivp = U.camera_matrices((0.1, 0.2, 1.5), (0.0, 0.0, 0.0), 45.0, 1.5)
    M = ivp.reshape(4, 4).T  # column-major storage
    pc = M @ np.array([0.0, 0.0, 0.5, 1.0])
    d = pc[:3] / pc[3] - np.array([0.1, 0.2, 1.5])
    d /= np.linalg.norm(d)
    t = -np.array([0.1, 0.2, 1.5]) / np.linalg.norm([0.1, 0.2, 1.5])
    assert np.dot(d, t) > 0.9999
    assert np.allclose(vp.reshape(4, 4).T @ M, np.eye(4), atol=1e-4)


def test_render_upward_rays_end_at_the_waves(oracle_mod):
    """A camera below the meniscus looking up: rays steeper than 0.052 end
    where they cross the wave surface (intersectWaterSurface), so a raised
    wave field changes the depth the rays gather through a plume that
    reaches the surface; a flat field gives the flat-plane image."""
    cfg = abi.config_reference()
    cfg.nx, cfg.ny, cfg.nz = 32, 48, 32
    cfg.mg_levels = 3
    cfg.parcel_capacity = 1024
    eye, target = (0.02, -0.12, 0.95), (0.0, 0.05, 0.0)
    vp, ivp = U.camera_matrices(eye, target, 40.0, W / H)
    blk = U.SimUniformPacker().pack(drops=U.DropSnapshot(sim_time=0.5, active_count=0), dt=1.0 / 60.0,
                                    frame_index=7, config=U.FluidOpticalConfig(), inv_view_proj=ivp, view_proj=vp,
                                    camera_pos=eye, camera_target=target, viewport_width=W,
                                    viewport_height=H).copy()
    nz, ny, nx = 64, 96, 64
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    blob = np.exp(-(((x - 32) / 10.0) ** 2 + ((y - 80) / 30.0) ** 2 + ((z - 31) / 10.0) ** 2) * 1.5)
    conc = np.zeros((nz, ny, nx, 4), np.float32)
    conc[..., 0] = 0.6 * blob
    conc[..., 1] = 0.2 * blob
    conc[..., 2] = 0.5 * blob
    lut = U.synthetic_spectral_lut()
    wave = np.zeros((512, 512, 4), np.float32)
    i = np.linspace(0, 6 * np.pi, 512)
    wave[..., 0] = 0.03 * np.sin(i[None, :]) * np.cos(0.7 * i[:, None])
    out = []
    for w in (np.zeros_like(wave), wave):
        o = oracle_mod.OracleSim(cfg)
        o.set_uniforms(blk)
        o.set_field(abi.FIELD_CONC, conc)
        o.set_field(abi.FIELD_WAVE, w)
        out.append(halves(o.render_plume(W, H, lut)))
    flat, wavy = out
    assert np.isfinite(wavy).all()
    assert (flat[..., 3] > 0).mean() > 0.05
    changed = (flat[..., 3] != wavy[..., 3])
    assert changed.mean() > 0.05
