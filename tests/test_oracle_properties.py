"""Properties of the oracle that hold independently of the reference's
numbers (the reference pins none for the step): multigrid convergence on a
manufactured solution in both boundary modes, divergence-free projection,
exact trilinear transport of linear fields, FP32 vs FP64 agreement, the
mixed-precision defect loop and determinism."""
import numpy as np
import pytest

from dropfluid import abi, scenes
from helpers import rel_l2, smooth_field


def apply_laplacian(p, ref):
    """The reference's 7-point operator (fluid.ts:561-603, h = 1)."""
    nz, ny, nx = p.shape
    out = np.zeros_like(p, dtype=np.float64)
    q = p.astype(np.float64)
    diag = np.zeros_like(out) + (1.0 if ref else 0.0)
    sumn = np.zeros_like(out)
    sumn[:, :, 1:] += q[:, :, :-1]; diag[:, :, 1:] += 1
    sumn[:, :, :-1] += q[:, :, 1:]; diag[:, :, :-1] += 1
    sumn[:, 1:, :] += q[:, :-1, :]; diag[:, 1:, :] += 1
    sumn[:, :-1, :] += q[:, 1:, :]
    if not ref:
        diag[:, :-1, :] += 1
    sumn[1:, :, :] += q[:-1, :, :]; diag[1:, :, :] += 1
    sumn[:-1, :, :] += q[1:, :, :]; diag[:-1, :, :] += 1
    out = sumn - diag * q
    return out


@pytest.mark.parametrize("ref", [False, True])
def test_vcycle_converges_on_manufactured_solution(oracle_mod, ref):
    n = (32, 32, 32)
    c = abi.config_reference() if ref else abi.config_closed_box(*n)
    c.nx, c.ny, c.nz = n
    c.mg_levels = 4
    c.mg_pre = c.mg_post = 2
    c.mg_coarse_sweeps = 24
    c.reference_schedule = 0
    c.mg_cycles = 1
    c.parcel_capacity = 16
    s = oracle_mod.OracleSim(c, fp64=True)
    pstar = smooth_field((n[2], n[1], n[0]), 3, 1.0).astype(np.float64)
    if not ref:
        pstar -= pstar.mean()
    b = apply_laplacian(pstar, ref)
    s.set_field(abi.FIELD_RHS, b.astype(np.float32))
    s.set_field(abi.FIELD_PRESSURE, np.zeros_like(b, dtype=np.float32))
    errs = []
    for _ in range(6):
        s.run_stage(abi.STAGE_PRESSURE_SOLVE)
        p = s.get_field(abi.FIELD_PRESSURE).astype(np.float64)
        if not ref:
            p -= p.mean()
        errs.append(np.linalg.norm(p - pstar) / np.linalg.norm(pstar))
    rates = [errs[k + 1] / errs[k] for k in range(len(errs) - 1) if errs[k] > 1e-6]
    assert errs[-1] < 1e-3, errs
    assert max(rates) < 0.35, (errs, rates)


def test_projection_is_divergence_free(oracle_mod):
    c = abi.config_closed_box(32, 32, 32)
    c.mg_levels = 4
    c.mg_cycles = 12
    c.parcel_capacity = 16
    s = oracle_mod.OracleSim(c, fp64=True)
    for f, sd in ((abi.FIELD_VEL_U, 1), (abi.FIELD_VEL_V, 2), (abi.FIELD_VEL_W, 3)):
        s.set_field(f, smooth_field((32, 32, 32), sd, 1.0))
    for st in (abi.STAGE_MAC_RHS, abi.STAGE_PRESSURE_SOLVE, abi.STAGE_PROJECT):
        s.run_stage(st)
    div = s.get_field(abi.FIELD_DIVERGENCE)
    assert np.abs(div).max() < 1e-5


def test_uniform_flow_translates_linear_dye_exactly(oracle_mod):
    """Semi-Lagrangian RK2 with a uniform centre velocity moves a linear dye
    field by exactly v dt in the interior (trilinear is exact on linears)."""
    n = 24
    c = abi.config_closed_box(n, n, n)
    c.mg_levels = 3
    c.parcel_capacity = 16
    s = oracle_mod.OracleSim(c, fp64=True)
    vel = np.array([10.0, -5.0, 2.5])
    cen = np.zeros((n, n, n, 4), np.float32)
    cen[..., :3] = vel
    s.set_field(abi.FIELD_VEL_CENTER, cen)
    z, y, x = np.meshgrid(*(np.arange(n) + 0.5,) * 3, indexing="ij")
    dye = 0.01 * x + 0.02 * y + 0.03 * z
    s.set_field(abi.FIELD_CONC, dye.astype(np.float32))
    s.run_stage(abi.STAGE_CONC_PREDICT)
    pred = s.get_field(abi.FIELD_CONC_PRED).astype(np.float64)
    d = vel * c.dt
    expect = 0.01 * (x - d[0]) + 0.02 * (y - d[1]) + 0.03 * (z - d[2])
    inner = (slice(3, -3),) * 3
    assert np.abs(pred[inner] - expect[inner]).max() < 1e-5


def test_fp32_oracle_tracks_fp64_oracle(oracle_mod):
    sc = scenes.box48()
    a = oracle_mod.OracleSim(sc.config)
    b = oracle_mod.OracleSim(sc.config, fp64=True)
    for e in (a, b):
        scenes.run(sc, e, steps=6)
    for f in (abi.FIELD_VEL_V, abi.FIELD_PRESSURE, abi.FIELD_CONC):
        assert rel_l2(a.get_field(f), b.get_field(f)) < 1e-4


def test_box48_divergence_after_projection(oracle_mod):
    sc = scenes.box48()
    s = oracle_mod.OracleSim(sc.config)
    scenes.run(sc, s, steps=4)
    st = s.step(1, stats=True)
    assert st["max_div"] < 1e-5, st
    assert st["vcycles"] == sc.config.mg_cycles


@pytest.mark.parametrize("rel_tol,div_tol", [(1e-8, 0.0), (0.0, 1e-5), (1e-8, 1e-5)])
def test_mixed_defect_loop_reaches_tolerance(oracle_mod, rel_tol, div_tol):
    """The defect loop of a high-precision pressure reaches a relative
    residual of 1e-8 and/or a max-norm divergence target, below the FP32
    rounding of the pressure itself."""
    c = abi.config_closed_box(32, 32, 32)
    c.mg_levels = 4
    c.precision_mode = abi.DOB_PREC_MIXED
    c.mg_cycles = 1
    c.mg_rel_tol = rel_tol
    c.mg_div_tol = div_tol
    c.mg_max_outer = 30
    c.parcel_capacity = 16
    s = oracle_mod.OracleSim(c)
    for f, sd in ((abi.FIELD_VEL_U, 1), (abi.FIELD_VEL_V, 2), (abi.FIELD_VEL_W, 3)):
        s.set_field(f, smooth_field((32, 32, 32), sd, 40.0))
    s.run_stage(abi.STAGE_MAC_RHS)
    b = s.get_field64(abi.FIELD_RHS)
    s.run_stage(abi.STAGE_PRESSURE_SOLVE)
    p = s.get_field64(abi.FIELD_PRESSURE)
    r = b - apply_laplacian(p, False)
    if rel_tol:
        assert np.linalg.norm(r) / np.linalg.norm(b) <= rel_tol
    if div_tol:
        assert np.abs(r).max() * c.dt / c.dx <= div_tol
    # the FP32-rounded pressure alone could not get there
    r32 = b - apply_laplacian(p.astype(np.float32).astype(np.float64), False)
    if rel_tol:
        assert np.linalg.norm(r32) / np.linalg.norm(b) > 10 * rel_tol


def test_oracle_is_deterministic(oracle_mod):
    sc = scenes.box48()
    out = []
    for _ in range(2):
        s = oracle_mod.OracleSim(sc.config)
        scenes.run(sc, s, steps=3)
        out.append((s.get_field(abi.FIELD_VEL_V), s.get_parcels(), s.get_field(abi.FIELD_SPLAT_INTACT)))
    for a, b in zip(*out):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_single_parcel_splat_sum(oracle_mod):
    """Fixed-point splat: the 8 cells receive round(65536 m w_k) each
    (particles.ts:248-266) — checked against a host computation."""
    c = abi.config_closed_box(16, 16, 16)
    c.mg_levels = 2
    c.parcel_capacity = 1
    s = oracle_mod.OracleSim(c)
    pos = np.array([5.3, 7.71, 9.02], np.float32)
    m = np.float32(0.134)
    s.set_parcels(np.array([[*pos, m, 0, 0, 0, 0]], np.float32))
    s.run_stage(abi.STAGE_PARCEL_ADVECT)  # zero velocity: the parcel stays
    sp = s.get_field(abi.FIELD_SPLAT_INTACT)
    uvw = pos / np.float32(16.0)
    coord = uvw * np.float32(16.0) - np.float32(0.5)
    base = np.floor(coord).astype(int)
    f = coord - base.astype(np.float32)
    expect = 0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                wx = f[0] if dx else 1 - f[0]
                wy = f[1] if dy else 1 - f[1]
                wz = f[2] if dz else 1 - f[2]
                expect += int(np.rint(np.float32(m * np.float32(65536.0)) * wx * wy * wz))
    assert int(sp.sum()) == expect
    assert int(sp[base[2], base[1], base[0]]) > 0


@pytest.mark.parametrize("dims,h2,ref", [((2, 2, 2), 1.0, 0), ((6, 8, 6), 1024.0, 0), ((6, 8, 6), 64.0, 1),
                                         ((4, 6, 4), 1.0, 1), ((3, 4, 3), 16.0, 0), ((8, 4, 6), 4.0, 1)])
def test_separable_coarse_inverse_matches_gauss_jordan(oracle_mod, dims, h2, ref):
    """The exact coarsest solve's dense (pseudo-)inverse from the axis
    eigenpairs equals Gauss-Jordan's, closed box (minimum-norm inverse of the
    singular Neumann operator) and reference mode (Dirichlet ghost above the
    top)."""
    a = oracle_mod.coarse_inverse(dims, h2, ref, 1)
    b = oracle_mod.coarse_inverse(dims, h2, ref, 0)
    assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
    assert np.allclose(a, a.T, rtol=0, atol=1e-12 * np.abs(a).max())
