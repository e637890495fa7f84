"""Parity of the CUDA path (through the C ABI) with the oracle.

Each stage of the step runs on the same seeded inputs on the device and in
the CPU restatement; fields must agree to the tolerance stated per test
(FP32 arithmetic with and without multiply-add contraction differs in the
last bits, so stage results are compared in relative L2).  Parcel positions
and splat accumulators are compared bit for bit.
"""
import numpy as np
import pytest

from helpers import bits_equal, rel_l2, smooth_field

pytestmark = pytest.mark.gpu

STAGE_TOL = 2e-5      # one stage, FP32 with vs without FMA contraction
STEP_TOL = 1e-4       # relative L2 bar after N full steps


def _abi():
    from dropfluid import abi
    return abi


def ref_block(sim_time=0.4, spawn=2048, cursor=0, dt=1.0 / 60.0):
    from dropfluid import uniforms as U
    snap = U.DropSnapshot(sim_time=sim_time, active_count=2)
    snap.slots[0] = U.DropSlot(active=True, center=(0.03, 0.285, -0.02), radius=0.05, vel_y=-0.3,
                               oscillation=0.01, vol_drain_rate=0.42, seed=1.5)
    snap.slots[1] = U.DropSlot(active=True, center=(-0.12, 0.31, 0.09), radius=0.03, vel_y=-0.5,
                               oscillation=0.0, vol_drain_rate=0.05, seed=2.7)
    return U.SimUniformPacker().pack(drops=snap, dt=dt, global_seed=1.5, spawn_cursor=cursor,
                                     spawn_count=spawn).copy()


def ref_config(nx=32, ny=48, nz=32, prec=0):
    abi = _abi()
    c = abi.config_reference()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.mg_levels = 3
    c.parcel_capacity = 16384
    c.precision_mode = prec
    return c


def box_config(n=(32, 32, 32), prec=0):
    abi = _abi()
    c = abi.config_closed_box(*n)
    c.mg_levels = 3
    c.parcel_capacity = 4096
    c.precision_mode = prec
    return c


def ref_state(cfg, seed=0):
    """Seeded reference-mode state: velocities ~0.3 m/s, positive conc, a
    small wave field, parcels around the drops."""
    abi = _abi()
    nz, ny, nx = cfg.nz, cfg.ny, cfg.nx
    r = cfg.dye_refine
    st = {}
    st[abi.FIELD_VEL_U] = smooth_field((nz, ny, nx), seed + 1, 0.3)
    st[abi.FIELD_VEL_V] = smooth_field((nz, ny, nx), seed + 2, 0.3)
    st[abi.FIELD_VEL_W] = smooth_field((nz, ny, nx), seed + 3, 0.3)
    cen = np.zeros((nz, ny, nx, 4), np.float32)
    for k in range(3):
        cen[..., k] = smooth_field((nz, ny, nx), seed + 10 + k, 0.3)
    st[abi.FIELD_VEL_CENTER] = cen
    curl = np.zeros((nz, ny, nx, 4), np.float32)
    for k in range(3):
        curl[..., k] = smooth_field((nz, ny, nx), seed + 20 + k, 2.0)
    curl[..., 3] = np.sqrt((curl[..., :3] ** 2).sum(-1))
    st[abi.FIELD_CURL] = curl
    st[abi.FIELD_PRESSURE] = smooth_field((nz, ny, nx), seed + 30, 0.01)
    conc = np.zeros((nz * r, ny * r, nx * r, 4), np.float32)
    for k in range(4):
        conc[..., k] = np.abs(smooth_field((nz * r, ny * r, nx * r), seed + 40 + k, 0.6))
    st[abi.FIELD_CONC] = conc
    wave = np.zeros((512, 512, 4), np.float32)
    wave[..., 0] = smooth_field((512, 512), seed + 50, 0.01)
    wave[..., 1] = smooth_field((512, 512), seed + 51, 0.05)
    wave[..., 2] = smooth_field((512, 512), seed + 52, 0.01)
    wave[..., 3] = np.abs(smooth_field((512, 512), seed + 53, 0.9))
    st[abi.FIELD_WAVE] = wave
    return st


def ref_parcels(n, seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 8), np.float32)
    p[:, 0] = rng.uniform(-0.3, 0.3, n)
    p[:, 1] = rng.uniform(-0.95, 0.29, n)
    p[:, 2] = rng.uniform(-0.3, 0.3, n)
    p[:, 3] = np.where(rng.uniform(size=n) < 0.9, 0.134, 0.0)
    p[:, 4:7] = rng.normal(0, 0.004, (n, 3))
    p[:, 7] = np.floor(rng.uniform(0, 4000, n)) + rng.uniform(0, 0.9, n)
    return p


def load_state(eng, st):
    for f, a in st.items():
        eng.set_field(f, a)


@pytest.fixture(scope="module")
def both(oracle_mod, gpu_lib):
    from dropfluid import DropFluid

    def make(cfg):
        return DropFluid(cfg), oracle_mod.OracleSim(cfg)
    return make


# ---------------------------------------------------------------------------------------------
def test_eval_math_bit_exact(oracle_mod, gpu_lib):
    """The library's own elementary functions give the same bits on the
    device and on the host (the basis of bit-exact parcel bins)."""
    from dropfluid import eval_math
    rng = np.random.default_rng(5)
    cases = {
        0: rng.uniform(-200, 200, 20000), 1: rng.uniform(-200, 200, 20000), 2: rng.uniform(-80, 80, 20000),
        3: np.exp(rng.uniform(-80, 80, 20000)), 6: rng.uniform(-10, 10, 20000),
        7: rng.normal(0, 100, 20000), 8: rng.normal(0, 1e5, 20000),
    }
    for fn, x in cases.items():
        x = x.astype(np.float32)
        assert bits_equal(eval_math(fn, x), oracle_mod.eval_math(fn, x)), fn
    x = rng.uniform(0, 3, 20000).astype(np.float32)
    y = rng.uniform(0, 2, 20000).astype(np.float32)
    assert bits_equal(eval_math(4, x, y), oracle_mod.eval_math(4, x, y))
    a = rng.normal(0, 1, 20000).astype(np.float32)
    b = rng.normal(0, 1, 20000).astype(np.float32)
    assert bits_equal(eval_math(5, a, b), oracle_mod.eval_math(5, a, b))


def test_division_by_launch_constants_is_ieee(gpu_lib):
    """The kernels divide by launch constants (grid dims, domain size, 2 dx,
    dx^2) through the correctly rounded reciprocal and one exact remainder
    correction: every quotient equals the IEEE float32 division, over
    dividends across many binades and both signs."""
    from dropfluid import eval_math
    rng = np.random.default_rng(11)
    n = 1 << 20
    a = (rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-40, 13, n))).astype(np.float32)
    a[::2] *= -1
    a[:4] = [0.0, 1.0, 0.5, 191.5]
    for d in (192.0, 256.0, 96.0, 128.0, 48.0, 64.0, 24.0, 12.0, 2.0, 1.0, 3.0, 0.02, 7.0, 1.7, 0.3):
        y = np.full(n, d, np.float32)
        want = a / y
        assert want.dtype == np.float32
        assert bits_equal(eval_math(9, a, y), want), d


def test_binary16_store_matches_host_rounding(oracle_mod, gpu_lib):
    """__float2half_rn on the device == the host IEEE RNE restatement,
    including subnormals, ties and overflow."""
    from dropfluid import eval_math
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.normal(0, s, 5000) for s in (1e-7, 1e-5, 1e-2, 1, 1e3, 7e4)]).astype(np.float32)
    x = np.concatenate([x, np.array([0.0, -0.0, 1.0, 65504.0, 65520.0, 65519.99, 5.96e-8, 2.98e-8, 1e-9],
                                    np.float32)])
    dev = eval_math(7, x)
    assert bits_equal(dev, oracle_mod.eval_math(7, x))
    np.testing.assert_array_equal(dev, x.astype(np.float16).astype(np.float32))


# ---- closed box, stage by stage ------------------------------------------------------------
def box_state(cfg, seed=0, amp=40.0):
    abi = _abi()
    nz, ny, nx = cfg.nz, cfg.ny, cfg.nx
    st = {abi.FIELD_VEL_U: smooth_field((nz, ny, nx), seed + 1, amp),
          abi.FIELD_VEL_V: smooth_field((nz, ny, nx), seed + 2, amp),
          abi.FIELD_VEL_W: smooth_field((nz, ny, nx), seed + 3, amp)}
    cen = np.zeros((nz, ny, nx, 4), np.float32)
    for k in range(3):
        cen[..., k] = smooth_field((nz, ny, nx), seed + 10 + k, amp)
    st[abi.FIELD_VEL_CENTER] = cen
    st[abi.FIELD_PRESSURE] = smooth_field((nz, ny, nx), seed + 30, 1.0)
    st[abi.FIELD_CONC] = np.abs(smooth_field((nz, ny, nx), seed + 40, 1.0))
    return st


BOX_STAGE_OUT = {
    0: ("VEL_U", "VEL_V", "VEL_W"), 1: ("VEL_CENTER",), 3: ("VEL_U", "VEL_V", "VEL_W"), 4: ("RHS",),
    6: ("VEL_U", "VEL_V", "VEL_W"), 10: ("CONC_PRED",),
}


@pytest.mark.parametrize("stage", sorted(BOX_STAGE_OUT))
def test_box_stage_parity(both, stage):
    abi = _abi()
    cfg = box_config()
    g, o = both(cfg)
    st = box_state(cfg)
    load_state(g, st)
    load_state(o, st)
    g.run_stage(stage)
    o.run_stage(stage)
    for name in BOX_STAGE_OUT[stage]:
        f = getattr(abi, "FIELD_" + name)
        err = rel_l2(g.get_field(f), o.get_field(f))
        assert err < STAGE_TOL, (stage, name, err)


def test_box_pressure_solve_parity(both):
    abi = _abi()
    cfg = box_config()
    g, o = both(cfg)
    st = box_state(cfg)
    load_state(g, st)
    load_state(o, st)
    for e in (g, o):
        e.run_stage(abi.STAGE_MAC_RHS)
        e.run_stage(abi.STAGE_PRESSURE_SOLVE)
    assert rel_l2(g.get_field(abi.FIELD_PRESSURE), o.get_field(abi.FIELD_PRESSURE)) < STAGE_TOL
    # the FP64 compatibility sum leaves a zero-mean right-hand side and pressure
    assert abs(float(g.get_field(abi.FIELD_RHS).astype(np.float64).mean())) < 1e-5
    assert abs(float(g.get_field(abi.FIELD_PRESSURE).astype(np.float64).mean())) < 1e-5


def test_box_dye_resolve_parity(both):
    abi = _abi()
    cfg = box_config()
    g, o = both(cfg)
    st = box_state(cfg)
    st[abi.FIELD_CONC_PRED] = np.abs(smooth_field((cfg.nz, cfg.ny, cfg.nx), 77, 1.0))
    load_state(g, st)
    load_state(o, st)
    g.run_stage(abi.STAGE_CONC_RESOLVE)
    o.run_stage(abi.STAGE_CONC_RESOLVE)
    assert rel_l2(g.get_field(abi.FIELD_CONC), o.get_field(abi.FIELD_CONC)) < STAGE_TOL


def test_box_parcels_bit_exact(both):
    """Same centre velocity + parcels -> identical positions and splat bins."""
    abi = _abi()
    from dropfluid import scenes
    cfg = box_config()
    g, o = both(cfg)
    st = box_state(cfg)
    load_state(g, st)
    load_state(o, st)
    p = scenes.parcels_in_sphere((16.0, 20.0, 15.0), 6.0, 4096, 3)
    g.set_parcels(p)
    o.set_parcels(p)
    for e in (g, o):
        e.run_stage(abi.STAGE_CLEAR_SPLATS)
        e.run_stage(abi.STAGE_PARCEL_ADVECT)
    assert bits_equal(g.get_parcels(), o.get_parcels())
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_INTACT), o.get_field(abi.FIELD_SPLAT_INTACT))


# ---- reference mode, stage by stage -----------------------------------------------------------
REF_STAGE_OUT = {
    0: ("VEL_U", "VEL_V", "VEL_W"), 1: ("VEL_CENTER",), 2: ("CURL",), 3: ("VEL_U", "VEL_V", "VEL_W"),
    4: ("RHS",), 6: ("VEL_U", "VEL_V", "VEL_W"), 10: ("CONC_PRED",),
}


@pytest.mark.parametrize("stage", sorted(REF_STAGE_OUT))
def test_reference_stage_parity(both, stage):
    abi = _abi()
    cfg = ref_config()
    g, o = both(cfg)
    st = ref_state(cfg)
    blk = ref_block()
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
        e.run_stage(stage)
    for name in REF_STAGE_OUT[stage]:
        f = getattr(abi, "FIELD_" + name)
        err = rel_l2(g.get_field(f), o.get_field(f))
        assert err < STAGE_TOL, (stage, name, err)


def test_reference_pressure_solve_parity(both):
    abi = _abi()
    cfg = ref_config()
    g, o = both(cfg)
    st = ref_state(cfg)
    blk = ref_block()
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
        e.run_stage(abi.STAGE_MAC_RHS)
        e.run_stage(abi.STAGE_PRESSURE_SOLVE)
    assert rel_l2(g.get_field(abi.FIELD_PRESSURE), o.get_field(abi.FIELD_PRESSURE)) < STAGE_TOL


def test_reference_conc_resolve_parity(both):
    abi = _abi()
    cfg = ref_config()
    g, o = both(cfg)
    st = ref_state(cfg)
    r = cfg.dye_refine
    shape = (cfg.nz * r, cfg.ny * r, cfg.nx * r)
    st[abi.FIELD_CONC_PRED] = np.abs(smooth_field(shape, 91, 0.5))
    rng = np.random.default_rng(4)
    st[abi.FIELD_SPLAT_INTACT] = np.where(rng.uniform(size=shape) < 0.3, rng.integers(0, 20000, shape), 0).astype(np.uint32)
    st[abi.FIELD_SPLAT_LYSED] = np.where(rng.uniform(size=shape) < 0.3, rng.integers(0, 9000, shape), 0).astype(np.uint32)
    blk = ref_block()
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
        e.run_stage(abi.STAGE_CONC_RESOLVE)
    assert rel_l2(g.get_field(abi.FIELD_CONC), o.get_field(abi.FIELD_CONC)) < STAGE_TOL


def test_reference_parcels_bit_exact(both):
    """PARTICLE_EMIT + PARTICLE_ADVECT_SPLAT: parcels, and therefore their
    splat bins and fixed-point sums, identical to the host restatement."""
    abi = _abi()
    cfg = ref_config()
    g, o = both(cfg)
    st = ref_state(cfg)
    blk = ref_block(spawn=2048, cursor=1000)
    p = ref_parcels(cfg.parcel_capacity, 1)
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
        e.set_parcels(p)
        e.run_stage(abi.STAGE_CLEAR_SPLATS)
        e.run_stage(abi.STAGE_PARCEL_EMIT)
    assert bits_equal(g.get_parcels(), o.get_parcels())
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_LYSED), o.get_field(abi.FIELD_SPLAT_LYSED))
    for e in (g, o):
        e.run_stage(abi.STAGE_PARCEL_ADVECT)
    gp, op = g.get_parcels(), o.get_parcels()
    assert bits_equal(gp, op), int((gp.view(np.uint32) != op.view(np.uint32)).any(axis=1).sum())
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_INTACT), o.get_field(abi.FIELD_SPLAT_INTACT))
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_LYSED), o.get_field(abi.FIELD_SPLAT_LYSED))
    assert g.get_field(abi.FIELD_SPLAT_INTACT).sum() > 0
    # the device clears only the bricks its splats marked: everything is zero
    # again, and a second round matches the host's
    g.run_stage(abi.STAGE_CLEAR_SPLATS)
    assert not g.get_field(abi.FIELD_SPLAT_INTACT).any() and not g.get_field(abi.FIELD_SPLAT_LYSED).any()
    for e in (g, o):
        e.run_stage(abi.STAGE_CLEAR_SPLATS)
        e.run_stage(abi.STAGE_PARCEL_EMIT)
        e.run_stage(abi.STAGE_PARCEL_ADVECT)
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_INTACT), o.get_field(abi.FIELD_SPLAT_INTACT))
    assert bits_equal(g.get_field(abi.FIELD_SPLAT_LYSED), o.get_field(abi.FIELD_SPLAT_LYSED))
    # splats written from outside: every brick may hold them until the next clear
    g.set_field(abi.FIELD_SPLAT_INTACT, np.full(g.get_field(abi.FIELD_SPLAT_INTACT).shape, 7.0, np.float32))
    g.run_stage(abi.STAGE_CLEAR_SPLATS)
    assert not g.get_field(abi.FIELD_SPLAT_INTACT).any() and not g.get_field(abi.FIELD_SPLAT_LYSED).any()


# ---- full steps ------------------------------------------------------------------------------
def test_box48_scene_parity_and_divergence(oracle_mod, gpu_lib):
    """The 48x64x48 drop scene, 20 full steps: every field within relative L2
    1e-4 of the FP32 oracle, error against the FP64 oracle reported, and the
    projected velocity's max |div u| dt/dx <= 1e-5 at the end."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    g = DropFluid(sc.config)
    o32 = oracle_mod.OracleSim(sc.config)
    o64 = oracle_mod.OracleSim(sc.config, fp64=True)
    for e in (g, o32, o64):
        scenes.run(sc, e)
    for name in ("VEL_U", "VEL_V", "VEL_W", "PRESSURE", "CONC"):
        f = getattr(abi, "FIELD_" + name)
        e32 = rel_l2(g.get_field(f), o32.get_field(f))
        e64 = rel_l2(g.get_field(f), o64.get_field(f))
        print(f"box48 {name}: rel L2 vs FP32 oracle {e32:.2e}, vs FP64 oracle {e64:.2e}")
        assert e32 < STEP_TOL, (name, e32)
        assert e64 < 1e-3, (name, e64)
    gp, op = g.get_parcels()[:, :3], o32.get_parcels()[:, :3]
    assert rel_l2(gp, op) < STEP_TOL
    st = g.step(1, stats=True)
    assert st["max_div"] <= 1e-5, st


def test_step_statistics_match_fields(gpu_lib):
    """The closed-box step forms max |div u| dt/dx inside the projection
    kernel and ||rhs|| inside the mean removal: both equal the same
    quantities formed from the fields it leaves (the divergence with the
    same float32 operations, so exactly; the norm to FP64 summation order),
    with and without the captured graph."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    c = sc.config
    g = DropFluid(c)
    sc.release(g, 0)
    g.step(3)
    for graph in (True, False):
        st = g.step(1, stats=True, graph=graph)
        u = g.get_field(abi.FIELD_VEL_U).reshape(c.nz, c.ny, c.nx)
        v = g.get_field(abi.FIELD_VEL_V).reshape(c.nz, c.ny, c.nx)
        w = g.get_field(abi.FIELD_VEL_W).reshape(c.nz, c.ny, c.nx)
        f32 = np.float32
        uR = u.copy(); uR[:, :, -1] = 0
        vU = v.copy(); vU[:, -1, :] = 0
        wF = w.copy(); wF[-1, :, :] = 0
        uL = np.zeros_like(u); uL[:, :, 1:] = uR[:, :, :-1]
        vD = np.zeros_like(v); vD[:, 1:, :] = vU[:, :-1, :]
        wB = np.zeros_like(w); wB[1:, :, :] = wF[:-1, :, :]
        d = ((uR - uL) + (vU - vD)) + (wF - wB)
        assert d.dtype == f32
        md = float(np.max(np.abs(d) * (f32(c.dt) / f32(c.dx))))
        assert np.float32(st["max_div"]) == np.float32(md), (graph, st["max_div"], md)
        rhs = g.get_field(abi.FIELD_RHS).astype(np.float64)
        assert abs(st["rhs_l2"] - np.sqrt(np.sum(rhs * rhs))) <= 1e-9 * st["rhs_l2"], (graph, st["rhs_l2"])
    g.close()


def test_step_statistics_selection(gpu_lib):
    """dob_set_step_stats: without DOB_STATS_RESIDUAL / DOB_STATS_PARCELS a
    step with statistics skips the residual pass and the parcel count
    (reported as -1 and 0), keeps max |div| and ||b||, and leaves the same
    field bits; pipelined and synchronous; a bad mask is refused."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    from dropfluid._lib import DropFluidError
    sc = scenes.box48()
    a, b = DropFluid(sc.config), DropFluid(sc.config)
    b.set_step_stats(0)
    for e in (a, b):
        sc.release(e, 0)
    sa = [a.step(1, stats=True) for _ in range(2)] + a.run_pipelined(4)
    sb = [b.step(1, stats=True) for _ in range(2)] + b.run_pipelined(4)
    for x, y in zip(sa, sb):
        assert x["residual_l2"] > 0 and x["parcels_alive"] > 0
        assert y["residual_l2"] == -1.0 and y["parcels_alive"] == 0
        # ||b|| sums FP64 block partials with atomics: equal to summation order
        assert x["max_div"] == y["max_div"] and abs(x["rhs_l2"] - y["rhs_l2"]) <= 1e-12 * x["rhs_l2"]
    for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W, abi.FIELD_PRESSURE, abi.FIELD_CONC):
        assert bits_equal(a.get_field(f), b.get_field(f)), f
    b.set_step_stats(abi.STATS_ALL)
    assert b.step(1, stats=True)["residual_l2"] > 0
    with pytest.raises(DropFluidError):
        b.set_step_stats(8)
    a.close()
    b.close()


def test_reference_mode_steps_parity(oracle_mod, gpu_lib):
    """Reference setup (Dirichlet free-surface top, drops, parcels, 2x dye),
    8 substeps at a reduced grid: relative L2 <= 1e-4 against the oracle."""
    abi = _abi()
    from dropfluid import DropFluid
    cfg = ref_config()
    g = DropFluid(cfg)
    o = oracle_mod.OracleSim(cfg)
    st = ref_state(cfg, seed=3)
    del st[abi.FIELD_CURL]
    for k, e in enumerate((g, o)):
        e.set_uniforms(ref_block(sim_time=0.5, spawn=0))
        e.reset()
        e.set_field(abi.FIELD_WAVE, st[abi.FIELD_WAVE])
    for k in range(8):
        blk = ref_block(sim_time=0.5 + k / 60.0, spawn=512, cursor=512 * k)
        for e in (g, o):
            e.set_uniforms(blk)
            e.step(1)
    for name in ("VEL_U", "VEL_V", "VEL_W", "PRESSURE", "CONC"):
        f = getattr(abi, "FIELD_" + name)
        err = rel_l2(g.get_field(f), o.get_field(f))
        print(f"reference {name}: rel L2 {err:.2e}")
        assert err < STEP_TOL, (name, err)


def test_wave_solver_bit_exact(oracle_mod, gpu_lib):
    """The wave substep (force, row/column FFTs, spectral propagation,
    finalize; wave.ts:55-388) equals the oracle bit for bit over five
    substeps, from a seeded half-valued wave field with two drops at the
    surface and the v faces feeding the subsurface term; the dt changes at
    the fourth substep."""
    abi = _abi()
    from dropfluid import DropFluid
    cfg = ref_config()
    cfg.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE
    g = DropFluid(cfg)
    o = oracle_mod.OracleSim(cfg)
    st = ref_state(cfg, seed=5)
    del st[abi.FIELD_CURL]
    st[abi.FIELD_WAVE] = st[abi.FIELD_WAVE].astype(np.float16).astype(np.float32)
    for e in (g, o):
        e.set_uniforms(ref_block(sim_time=0.5, spawn=0))
        e.reset()
        load_state(e, st)
    for k, dt in enumerate((1.0 / 60.0, 1.0 / 60.0, 1.0 / 60.0, 1.0 / 120.0, 1.0 / 120.0)):
        blk = ref_block(sim_time=0.5 + k / 60.0, spawn=0, dt=dt)
        for e in (g, o):
            e.set_uniforms(blk)
            e.wave_step()
        a, b = g.get_field(abi.FIELD_WAVE), o.get_field(abi.FIELD_WAVE)
        assert np.abs(a).max() > 0
        assert bits_equal(a, b), (k, int(np.count_nonzero(a != b)), float(np.abs(a - b).max()))


def test_reference_steps_with_wave_solver(oracle_mod, gpu_lib):
    """Reference-mode steps with the wave solver at their start
    (BloodDropEngine.ts:1886-1912): the wave after the first step is the
    oracle's bit for bit (it reads the loaded faces); after 6 steps the
    wave and the fields are within the step tolerance."""
    abi = _abi()
    from dropfluid import DropFluid
    cfg = ref_config()
    cfg.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE
    g = DropFluid(cfg)
    o = oracle_mod.OracleSim(cfg)
    st = ref_state(cfg, seed=6)
    del st[abi.FIELD_CURL]
    st[abi.FIELD_WAVE] = st[abi.FIELD_WAVE].astype(np.float16).astype(np.float32)
    for e in (g, o):
        e.set_uniforms(ref_block(sim_time=0.5, spawn=0))
        e.reset()
        load_state(e, st)
    for k in range(6):
        blk = ref_block(sim_time=0.5 + k / 60.0, spawn=512, cursor=512 * k)
        for e in (g, o):
            e.set_uniforms(blk)
            e.step(1)
        if k == 0:
            assert bits_equal(g.get_field(abi.FIELD_WAVE), o.get_field(abi.FIELD_WAVE))
    # the wave texture stores halves: once the faces differ in their last
    # bits, a texel whose value flips one half ulp moves by 2^-11 relative
    wave_tol = 1e-3
    for name in ("WAVE", "VEL_U", "VEL_V", "VEL_W", "PRESSURE", "CONC"):
        f = getattr(abi, "FIELD_" + name)
        err = rel_l2(g.get_field(f), o.get_field(f))
        print(f"reference + wave {name}: rel L2 {err:.2e}")
        assert err < (wave_tol if name == "WAVE" else STEP_TOL), (name, err)


def test_graph_replay_equals_stage_launches(gpu_lib):
    """A step replayed from the captured graph gives the same bits as the
    same step launched stage by stage."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    a, b = DropFluid(sc.config), DropFluid(sc.config)
    sc.release(a, 0)
    sc.release(b, 0)
    a.step(5, graph=True)
    b.step(5, graph=False)
    for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_PRESSURE, abi.FIELD_CONC):
        assert bits_equal(a.get_field(f), b.get_field(f)), f
    assert bits_equal(a.get_parcels(), b.get_parcels())


@pytest.mark.parametrize("rel_tol", [0.0, 1e-8])
def test_mixed_graph_replay_equals_stage_launches(gpu_lib, rel_tol):
    """The mixed solve captured into the step graph (a while-node of V-cycles
    per round, an if-node for each round after the first) gives the bits and
    the round / V-cycle counts of the same steps enqueued without a graph
    (every round launched, returning at once after convergence): with the
    divergence target alone (one round) and with the relative target 1e-8
    (several rounds)."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    cfg = sc.config
    cfg.precision_mode = abi.DOB_PREC_MIXED
    cfg.mg_cycles = 1
    cfg.mg_rel_tol = rel_tol
    cfg.mg_div_tol = 1e-5
    cfg.mg_max_outer = 4
    a, b = DropFluid(cfg), DropFluid(cfg)
    sc.release(a, 0)
    sc.release(b, 0)
    rounds = []
    for _ in range(4):
        sa = a.step(1, stats=True, graph=True)
        sb = b.step(1, stats=True, graph=False)
        assert (sa["outer_iters"], sa["vcycles"]) == (sb["outer_iters"], sb["vcycles"])
        rounds.append(sa["outer_iters"])
    if rel_tol > 0:
        assert max(rounds) >= 2, rounds
    for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_PRESSURE, abi.FIELD_CONC):
        assert bits_equal(a.get_field(f), b.get_field(f)), f
    a.close()
    b.close()


def test_fused_projection_equals_separate_stages(gpu_lib):
    """The closed-box step leaves out the centre pass after advection (no
    reader) and runs projection + centre as one out-of-place kernel; a step
    made of the separate stages (dob_run_stage, in-place projection, then the
    centre pass) gives the same bits in every field, the centre velocity
    included, over several steps of alternating velocity buffers."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    # the separate stages run the plain V-cycle schedule: compare against
    # steps without the extra cycles after an injection
    sc.config.mg_cycles_injected = 0
    a, b = DropFluid(sc.config), DropFluid(sc.config)
    sc.release(a, 0)
    sc.release(b, 0)
    order = [abi.STAGE_ADVECT_MAC, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CASSON_FORCES, abi.STAGE_MAC_RHS,
             abi.STAGE_PRESSURE_SOLVE, abi.STAGE_PROJECT, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CLEAR_SPLATS,
             abi.STAGE_PARCEL_EMIT, abi.STAGE_PARCEL_ADVECT, abi.STAGE_CONC_PREDICT, abi.STAGE_CONC_RESOLVE]
    for _ in range(3):
        a.step(1)
        for stage in order:
            b.run_stage(stage)
        for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W, abi.FIELD_VEL_CENTER, abi.FIELD_PRESSURE,
                  abi.FIELD_CONC):
            assert bits_equal(a.get_field(f), b.get_field(f)), f
    assert bits_equal(a.get_parcels(), b.get_parcels())


def test_closed_box_sparse_dye_equals_stage_launches(gpu_lib):
    """The closed-box step skips clear water in the dye predictor (blocks
    whose departure points, bounded by the projection's largest centre
    velocity, reach no dye brick) and in the resolve (voxels whose tap
    bracket is two zeros): the same bits as the stages launched one by one
    (dense), over 10 steps of box96 with a second injection (flags reset to
    "may hold dye") halfway."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box96()
    sc.config.mg_cycles_injected = 0  # the stages run the plain V-cycle schedule
    a, b = DropFluid(sc.config), DropFluid(sc.config)
    sc.release(a, 0)
    sc.release(b, 0)
    order = [abi.STAGE_ADVECT_MAC, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CASSON_FORCES, abi.STAGE_MAC_RHS,
             abi.STAGE_PRESSURE_SOLVE, abi.STAGE_PROJECT, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CLEAR_SPLATS,
             abi.STAGE_PARCEL_EMIT, abi.STAGE_PARCEL_ADVECT, abi.STAGE_CONC_PREDICT, abi.STAGE_CONC_RESOLVE]
    for k in range(10):
        if k == 5:
            for e in (a, b):
                e.inject_sphere((40.0, 70.0, 50.0), 6.0, 1.0, (0.0, -0.5, 0.0), 0.0, 99)
        a.step(1)
        for stage in order:
            b.run_stage(stage)
        for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W, abi.FIELD_PRESSURE, abi.FIELD_CONC):
            assert bits_equal(a.get_field(f), b.get_field(f)), (k, f)
    conc = a.get_field(abi.FIELD_CONC)
    assert (conc > 0).mean() < 0.5  # most of the box is clear water: the skips ran
    a.close()
    b.close()


def test_injection_step_runs_more_cycles(gpu_lib, oracle_mod):
    """The two steps after a drop's injection run mg_cycles_injected V-cycles
    (closed-box default 8): their projections hold max |div| dt/dx <= 1e-5,
    their results match the oracle following the same rule, and the third
    step is back to mg_cycles (a graph captured without the extra cycles)."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    assert sc.config.mg_cycles_injected == 2 * sc.config.mg_cycles
    g = DropFluid(sc.config)
    o = oracle_mod.OracleSim(sc.config)
    for e in (g, o):
        sc.release(e, 0)
    for _ in range(2):
        st = g.step(1, stats=True)
        ost = o.step(1, stats=True)
        assert st["vcycles"] == sc.config.mg_cycles_injected, st
        assert ost["vcycles"] == sc.config.mg_cycles_injected, ost
        assert st["max_div"] <= 1e-5, st
        for f in (abi.FIELD_VEL_V, abi.FIELD_PRESSURE):
            assert rel_l2(g.get_field(f), o.get_field(f)) < STEP_TOL, f
    st = g.step(1, stats=True)
    ost = o.step(1, stats=True)
    assert st["vcycles"] == sc.config.mg_cycles, st
    assert ost["vcycles"] == sc.config.mg_cycles, ost
    g.close()


def test_save_load_state_roundtrip(gpu_lib):
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    a = DropFluid(sc.config)
    sc.release(a, 0)
    a.step(2)
    a.save_state(0)
    a.step(3)
    u5 = a.get_field(abi.FIELD_VEL_V)
    a.load_state(0)
    a.step(3)
    assert bits_equal(a.get_field(abi.FIELD_VEL_V), u5)


def test_fp16_reference_storage_parity(both):
    """rgba16float storage (reference-faithful mode): the device's binary16
    stores match the oracle's emulated RNE rounding."""
    abi = _abi()
    cfg = ref_config(prec=abi.DOB_PREC_REFERENCE_FP16)
    g, o = both(cfg)
    st = ref_state(cfg, seed=8)
    blk = ref_block()
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
    for stage in (abi.STAGE_ADVECT_MAC, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CASSON_FORCES):
        g.run_stage(stage)
        o.run_stage(stage)
        for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W):
            assert rel_l2(g.get_field(f), o.get_field(f)) < 2e-3, (stage, f)


def test_mixed_precision_defect_loop(both):
    """Mixed mode: the error-free residual of the double-float pressure and
    one V-cycle per iteration (BF16 levels 2-3) reach a relative residual of
    1e-8, like the oracle's restatement with a double pressure."""
    abi = _abi()
    cfg = box_config(prec=abi.DOB_PREC_MIXED)
    cfg.mg_cycles = 1
    cfg.mg_rel_tol = 1e-8
    cfg.mg_div_tol = 1e-5
    cfg.mg_max_outer = 30
    g, o = both(cfg)
    st = box_state(cfg)
    load_state(g, st)
    load_state(o, st)
    for e in (g, o):
        e.run_stage(abi.STAGE_MAC_RHS)
        e.run_stage(abi.STAGE_PRESSURE_SOLVE)
    # both converged to 1e-8: they agree far below the FP32 rounding floor of
    # an FP32-only solve (~1e-5 here)
    assert rel_l2(g.get_field(abi.FIELD_PRESSURE), o.get_field(abi.FIELD_PRESSURE)) < 1e-6


def test_mixed_precision_steps_meet_targets(gpu_lib, oracle_mod):
    """box48 in the mixed mode: every step ends with ||b - A p|| / ||b|| <=
    1e-8 and max |div| dt/dx <= 1e-5; after 12 steps velocity agrees with an
    FP64 run with a fully converged pressure to 1e-4 (relative L2) and the
    FP16-stored dye to 2e-3."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    sc = scenes.box48()
    cfg = sc.config
    cfg.precision_mode = abi.DOB_PREC_MIXED
    cfg.mg_cycles = 1
    cfg.mg_rel_tol = 1e-8
    cfg.mg_div_tol = 1e-5
    cfg.mg_max_outer = 30
    ref_cfg = scenes.box48().config
    ref_cfg.mg_cycles = 40
    g = DropFluid(cfg)
    o = oracle_mod.OracleSim(ref_cfg, fp64=True)
    for k in range(12):
        for j in sc.releases_at(k):
            sc.release(g, j)
            sc.release(o, j)
        stg = g.step(1, stats=True)
        o.step(1)
        assert stg["residual_l2"] <= 1.05e-8 * stg["rhs_l2"], (k, stg)
        assert stg["max_div"] <= 1e-5, (k, stg)
    for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W):
        assert rel_l2(g.get_field(f), o.get_field(f)) < 1e-4, f
    assert rel_l2(g.get_field(abi.FIELD_CONC), o.get_field(abi.FIELD_CONC)) < 2e-3
    g.close()


def test_error_paths(gpu_lib):
    abi = _abi()
    from dropfluid import DropFluid, DropFluidError
    bad = abi.config_closed_box(30, 32, 32)
    bad.mg_levels = 3  # 30 is not divisible by 2^3: odd coarse grids
    with pytest.raises(DropFluidError) as ei:
        DropFluid(bad)
    assert ei.value.status == abi.DOB_EINVAL
    cfg = box_config()
    g = DropFluid(cfg)
    small = np.zeros(10, np.float32)
    assert g._L.dob_set_field(g._h, abi.FIELD_VEL_U, small.ctypes.data, small.nbytes) == abi.DOB_EINVAL
    assert g._L.dob_get_field(g._h, 99, small.ctypes.data, small.nbytes) == abi.DOB_EINVAL
    with pytest.raises(ValueError):
        g.set_field(abi.FIELD_VEL_U, small)
    with pytest.raises(DropFluidError) as ei:
        g.set_parcels(np.zeros((cfg.parcel_capacity + 1, 8), np.float32))
    assert ei.value.status == abi.DOB_EINVAL
    r = DropFluid(ref_config())
    with pytest.raises(DropFluidError) as ei:
        r.inject_sphere((0, 0, 0), 0.1, 1.0, (0, 0, 0))
    assert ei.value.status == abi.DOB_ESTATE
    blk = ref_block()
    blk[38] = np.nan
    with pytest.raises(DropFluidError) as ei:
        r.set_uniforms(blk)
    assert ei.value.status == abi.DOB_EINVAL


@pytest.mark.parametrize("mode", ["box", "ref"])
def test_pressure_solve_parity_wide_tiles(both, mode):
    """A wide, deep grid (128x64x96, five grids in the closed box): the
    4-cells-per-thread smoother on levels whose rows fill several warps, the
    paired transfers and the exact coarsest solve (closed box) or the
    cluster's coarse sweeps (reference mode) reproduce the oracle's
    in-place sweeps."""
    abi = _abi()
    if mode == "box":
        cfg = box_config(n=(128, 64, 96))
        cfg.mg_levels = 5
        st = box_state(cfg, seed=5)
    else:
        cfg = ref_config(nx=128, ny=64, nz=96)
        cfg.mg_levels = 4
        cfg.reference_schedule = 1
        st = ref_state(cfg, seed=6)
    g, o = both(cfg)
    for e in (g, o):
        if mode == "ref":
            e.set_uniforms(ref_block())
        load_state(e, st)
        e.run_stage(abi.STAGE_MAC_RHS)
        e.run_stage(abi.STAGE_PRESSURE_SOLVE)
    assert rel_l2(g.get_field(abi.FIELD_PRESSURE), o.get_field(abi.FIELD_PRESSURE)) < STAGE_TOL


def test_pipelined_steps_match_synchronous(gpu_lib):
    """dob_step_async / dob_step_result give the same steps and statistics
    as dob_step with statistics, and refuse a slot that is still pending or
    was never filled."""
    abi = _abi()
    from dropfluid import DropFluid, DropFluidError, scenes
    sc = scenes.box48()
    a, b = DropFluid(sc.config), DropFluid(sc.config)
    for e in (a, b):
        sc.release(e, 0)
    sync = [a.step(1, stats=True) for _ in range(5)]
    piped = b.run_pipelined(5, depth=2)
    assert [s["max_div"] for s in sync] == [s["max_div"] for s in piped]
    assert [s["parcels_alive"] for s in sync] == [s["parcels_alive"] for s in piped]
    assert bits_equal(a.get_field(abi.FIELD_VEL_V), b.get_field(abi.FIELD_VEL_V))
    with pytest.raises(DropFluidError):
        b.step_result(3)  # nothing pending there
    b.step_async(0)
    with pytest.raises(DropFluidError):
        b.step_async(0)  # still pending
    b.step_result(0)
    a.close()
    b.close()


# ---- light volume and brick occupancy (lighting.ts:19-240) -------------------------------------
@pytest.mark.parametrize("prec,variant", [(0, "studio"), (0, "dark_camera"), (2, "studio")])
def test_light_volume_bit_exact(both, prec, variant):
    """The light volume (binary16 key light, back light, multiple scattering,
    filtered total) and both brick maps equal the oracle bit for bit, from a
    seeded dye and wave field with two drops above the surface; the dark
    variant also moves the camera (the back light's heading)."""
    abi = _abi()
    cfg = ref_config(prec=prec)
    g, o = both(cfg)
    st = ref_state(cfg, seed=12)
    # a sparser dye than the stage tests' (most voxels under the empty-water
    # threshold, marches that run their 9 samples)
    conc = st[abi.FIELD_CONC]
    conc *= (conc[..., :1] > 0.35).astype(np.float32) * 0.05
    if prec == abi.DOB_PREC_REFERENCE_FP16:
        # the device stores the loaded dye as binary16; give the oracle the same values
        st[abi.FIELD_CONC] = conc.astype(np.float16).astype(np.float32)
    blk = ref_block()
    if variant == "dark_camera":
        blk[51] = 1.0
        blk[8:16] = [0.3, 0.1, -0.5, 0.0, 0.1, 0.2, 0.7, 1.0]
        blk[32:35] = [0.5, 0.4, 1.8]
    for e in (g, o):
        e.set_uniforms(blk)
        load_state(e, st)
        e.light_volume()
    a, b = g.get_field(abi.FIELD_LIGHT), o.get_field(abi.FIELD_LIGHT)
    assert bits_equal(a, b), (int((a != b).any(axis=-1).sum()), float(np.abs(a - b).max()))
    assert (a[..., 0] < 1.0).any() and (a[..., 2] > 0.0).any()
    for f in (abi.FIELD_BRICKS_RAW, abi.FIELD_BRICKS):
        assert bits_equal(g.get_field(f), o.get_field(f)), f
    assert (g.get_field(abi.FIELD_BRICKS) == 1.0).any() and (g.get_field(abi.FIELD_BRICKS) == 2.0).any()


def test_lighting_flag_runs_once_per_call(gpu_lib):
    """DOB_PHYS_LIGHTING ends dob_step / dob_step_uniforms with the lighting
    passes on the last step's parameters: the same bits as an explicit
    dob_light_volume after the same steps."""
    abi = _abi()
    from dropfluid import DropFluid
    cfg = ref_config()
    cfg_l = ref_config()
    cfg_l.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_LIGHTING
    a, b = DropFluid(cfg), DropFluid(cfg_l)
    st = ref_state(cfg, seed=13)
    del st[abi.FIELD_CURL]
    blocks = np.stack([ref_block(sim_time=0.5 + k / 60.0, spawn=256, cursor=256 * k) for k in range(3)])
    for e in (a, b):
        e.set_uniforms(blocks[0])
        e.reset()
        load_state(e, st)
        e.step_uniforms(blocks)
    a.light_volume()
    assert bits_equal(a.get_field(abi.FIELD_LIGHT), b.get_field(abi.FIELD_LIGHT))
    assert bits_equal(a.get_field(abi.FIELD_BRICKS), b.get_field(abi.FIELD_BRICKS))
    r = DropFluid(box_config())
    from dropfluid import DropFluidError
    with pytest.raises(DropFluidError) as ei:
        r.light_volume()
    assert ei.value.status == abi.DOB_ESTATE
    for e in (a, b, r):
        e.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_reference_step_sparse_dye_equals_stage_launches(gpu_lib, prec):
    """Inside a step the reference-mode predictor and resolve skip clear
    water by 8x8x8 brick flags, four planes per thread; launched as single
    stages they trace every voxel.  With the dye in one corner of the grid,
    three steps (graph replays) give the same bits as the same stages
    launched one by one, in FP32 and with binary16 storage."""
    abi = _abi()
    from dropfluid import DropFluid
    cfg = ref_config(prec=prec)
    cfg.physics_flags = abi.DOB_PHYS_REFERENCE_ALL
    st = ref_state(cfg, seed=5)
    conc = st[abi.FIELD_CONC]
    keep = np.zeros(conc.shape[:3], bool)
    keep[4:28, 40:84, 6:30] = True  # (z, y, x) of the 64x96x64 dye grid
    conc[~keep] = 0.0
    blk = ref_block(spawn=0)
    a, b = DropFluid(cfg), DropFluid(cfg)
    for e in (a, b):
        e.set_uniforms(blk)
        load_state(e, st)
    order = [abi.STAGE_ADVECT_MAC, abi.STAGE_MAC_TO_CENTER, abi.STAGE_CURL, abi.STAGE_CASSON_FORCES,
             abi.STAGE_MAC_RHS, abi.STAGE_PRESSURE_SOLVE, abi.STAGE_PROJECT, abi.STAGE_MAC_TO_CENTER,
             abi.STAGE_CLEAR_SPLATS, abi.STAGE_PARCEL_EMIT, abi.STAGE_PARCEL_ADVECT, abi.STAGE_CONC_PREDICT,
             abi.STAGE_CONC_RESOLVE]
    for _ in range(3):
        a.step(1)
        for s in order:
            b.run_stage(s)
    for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W, abi.FIELD_PRESSURE, abi.FIELD_CONC,
              abi.FIELD_CONC_PRED):
        assert bits_equal(a.get_field(f), b.get_field(f)), f
    c = a.get_field(abi.FIELD_CONC)
    assert (c[..., 1] > 0).any() and (c[..., 1] == 0).mean() > 0.5
    a.close()
    b.close()


def test_mixed_steps_are_reproducible(gpu_lib):
    """The mixed mode's mean removal sums per-block partials in a fixed order
    (not FP64 atomics in completion order), so two runs of the same steps
    give the same bits; the double-float pressure's low part would
    otherwise carry the last bits of whichever order the blocks finished in."""
    abi = _abi()
    from dropfluid import DropFluid, scenes
    out = []
    for _ in range(2):
        sc = scenes.box192(abi.DOB_PREC_MIXED)
        e = DropFluid(sc.config)
        sc.release(e, 0)
        e.step(3)
        out.append({f: e.get_field(f) for f in (abi.FIELD_VEL_U, abi.FIELD_PRESSURE, abi.FIELD_CONC)})
        e.close()
    for f in out[0]:
        assert bits_equal(out[0][f], out[1][f]), f
