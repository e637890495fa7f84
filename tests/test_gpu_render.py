"""The plume render (k_render.cu, dob_render_plume) against the oracle's
restatement (oracle/dob_oracle_render.inc): the same state, camera and
spectral table give the same binary16 image bits, in FP32 and with the
reference's binary16 storage, in both lighting modes, on a reduced grid
and on the reference's own 96x128x96 / 192x256x192 grids."""
import numpy as np
import pytest

from dropfluid import abi
from dropfluid import uniforms as U

pytestmark = pytest.mark.gpu


def _block(W, H, eye, target, lighting_mode=0.0, frame=7, drops=None):
    vp, ivp = U.camera_matrices(eye, target, 40.0, W / H)
    snap = drops or U.DropSnapshot(sim_time=0.5, active_count=0)
    oc = U.FluidOpticalConfig(lightingMode=lighting_mode)
    return U.SimUniformPacker().pack(drops=snap, dt=1.0 / 60.0, frame_index=frame, config=oc, inv_view_proj=ivp,
                                     view_proj=vp, camera_pos=eye, camera_target=target, viewport_width=W,
                                     viewport_height=H).copy()


def _blob_conc(shape, seed, centre, radii, scale=1.0):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    r2 = ((x - centre[0]) / radii[0]) ** 2 + ((y - centre[1]) / radii[1]) ** 2 + ((z - centre[2]) / radii[2]) ** 2
    blob = np.exp(-r2 * 1.5)
    conc = np.zeros((nz, ny, nx, 4), np.float32)
    conc[..., 0] = 0.030 * scale * blob
    conc[..., 1] = 0.012 * scale * blob * (1.0 + 0.2 * rng.standard_normal(blob.shape)).clip(0.5, 1.5)
    conc[..., 2] = (0.4 + 0.3 * rng.random(blob.shape)) * blob
    conc[..., 3] = 0.02 * blob
    return conc


def _wave(seed):
    rng = np.random.default_rng(seed)
    w = np.zeros((512, 512, 4), np.float32)
    i = np.linspace(0, 6 * np.pi, 512)
    w[..., 0] = 0.004 * np.sin(i[None, :] + rng.random()) * np.cos(0.7 * i[:, None])
    w[..., 2] = 0.002 * np.cos(1.3 * i[None, :])
    return w


def _compare(gpu_lib, oracle_mod, cfg, conc, blk, W, H, fp16):
    from dropfluid import DropFluid
    lut = U.synthetic_spectral_lut(5)
    g = DropFluid(cfg)
    o = oracle_mod.OracleSim(cfg)
    if fp16:  # the device stores binary16: the oracle starts from the same values
        conc = conc.astype(np.float16).astype(np.float32)
    wave = _wave(2)
    for e in (g, o):
        e.set_uniforms(blk)
        e.set_field(abi.FIELD_CONC, conc)
        e.set_field(abi.FIELD_WAVE, wave)
    g.set_spectral_lut(lut)
    a = g.render_plume(W, H)
    b = o.render_plume(W, H, lut)
    diff = (a != b).any(axis=-1)
    assert not diff.any(), (int(diff.sum()), np.argwhere(diff)[:5])
    f = a.view(np.float16).astype(np.float32)
    assert (f[..., 3] > 0).mean() > 0.05  # the plume is in the picture
    g.close()
    return f


@pytest.mark.parametrize("prec,mode", [(abi.DOB_PREC_FP32, 0.0), (abi.DOB_PREC_REFERENCE_FP16, 0.0),
                                       (abi.DOB_PREC_FP32, 1.0)])
def test_render_bit_exact_reduced(gpu_lib, oracle_mod, prec, mode):
    cfg = abi.config_reference()
    cfg.nx, cfg.ny, cfg.nz = 32, 48, 32
    cfg.mg_levels = 3
    cfg.parcel_capacity = 1024
    cfg.precision_mode = prec
    W, H = 64, 40
    conc = _blob_conc((64, 96, 64), 3, (30, 42, 33), (9.0, 16.0, 9.0))
    blk = _block(W, H, (0.05, -0.32, 1.05), (0.0, -0.36, 0.0), mode)
    _compare(gpu_lib, oracle_mod, cfg, conc, blk, W, H, prec == abi.DOB_PREC_REFERENCE_FP16)


def test_render_bit_exact_reference_grids(gpu_lib, oracle_mod):
    """The reference's own grids (96x128x96 light volume, 192x256x192 dye),
    a dense plume that reaches the meniscus (the wave-height clip and the
    cubic B-spline dye both active) seen from below the surface, and a
    drop at the surface (the collar and orifice terms)."""
    cfg = abi.config_reference()
    cfg.parcel_capacity = 1024
    W, H = 96, 54
    conc = _blob_conc((192, 256, 192), 4, (96, 200, 92), (14.0, 60.0, 14.0), scale=20.0)
    snap = U.DropSnapshot(sim_time=0.9, active_count=1)
    snap.slots[0] = U.DropSlot(active=True, center=(0.0, 0.29, -0.01), radius=0.04, vel_y=-0.2, oscillation=0.0,
                               vol_drain_rate=0.3, seed=1.5)
    blk = _block(W, H, (0.02, -0.12, 0.95), (0.0, 0.05, 0.0), 0.0, drops=snap)
    f = _compare(gpu_lib, oracle_mod, cfg, conc, blk, W, H, False)
    assert f[..., 0].max() > 0.0
