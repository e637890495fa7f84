"""The FP64 oracle's discrete adjoint against its own forward (CPU).

Linear stages (centre average, divergence with mean removal, the whole
pressure solve, projection) pass the dot-product test <A x, y> = <x, A^T y>;
nonlinear stages match central differences of the forward on smooth moving
states; a recorded drop trajectory's gradient with respect to the drop
impulse matches central differences of the loss.  Perturbed fields cross the
oracle's interface in double precision.
"""
import numpy as np
import pytest

import adjoint_cases as AC
from dropfluid import abi


@pytest.fixture(scope="module")
def orc(oracle_mod):
    cfg = AC.box_config((16, 24, 16))
    return cfg, oracle_mod.OracleSim(cfg, fp64=True), AC.stage_state(cfg, seed=3)


def _dot(a, b):
    return float(np.sum(np.asarray(a, np.float64) * np.asarray(b, np.float64)))


@pytest.mark.parametrize("stage", AC.LINEAR)
def test_linear_stage_dot_product(orc, stage):
    cfg, o, st = orc
    ins, outs, _, _ = AC.STAGES[stage]
    xs = AC.seeded_cotangents(o, ins, 10 + stage)
    ys = AC.seeded_cotangents(o, outs, 20 + stage)
    AC.load(o, st)
    for f, a in xs.items():
        o.set_field(f, a)
    o.run_stage(stage)
    lhs = sum(_dot(o.get_field(f), ys[f]) for f in outs)
    adj = AC.run_stage_adjoint(o, st, stage, ys)
    rhs = sum(_dot(xs[f], adj[f]) for f in ins)
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


# relative tolerance of <J d, y> vs central differences per nonlinear stage
# (the adjoint arrays are read back as float32)
FD_TOL = {abi.STAGE_ADVECT_MAC: 1e-5, abi.STAGE_CASSON_FORCES: 1e-5,
          abi.STAGE_CONC_PREDICT: 1e-5, abi.STAGE_CONC_RESOLVE: 1e-5}


@pytest.mark.parametrize("stage", sorted(FD_TOL))
def test_nonlinear_stage_matches_central_differences(orc, stage):
    cfg, o, st = orc
    ins, outs, _, _ = AC.STAGES[stage]
    ds = AC.seeded_cotangents(o, ins, 30 + stage)
    ys = AC.seeded_cotangents(o, outs, 40 + stage)
    eps = 1e-6  # the FP64 interface keeps the perturbation exact

    def f(sign):
        AC.load(o, st)
        for fld in ins:
            o.set_field64(fld, st[fld].astype(np.float64) + sign * eps * ds[fld])
        o.run_stage(stage)
        return sum(_dot(o.get_field64(fld), ys[fld]) for fld in outs)

    fd = (f(1) - f(-1)) / (2 * eps)
    adj = AC.run_stage_adjoint(o, st, stage, ys)
    ad = sum(_dot(ds[fld], adj[fld]) for fld in ins)
    assert abs(fd - ad) <= FD_TOL[stage] * abs(fd), (fd, ad)


def test_trajectory_impulse_gradient_matches_central_differences(oracle_mod):
    cfg, center, r = AC.drop_scene((16, 24, 16))
    o = oracle_mod.OracleSim(cfg, fp64=True)
    steps = 6
    AC.init_drop(o, center, r, 1.1)
    o.tape_forward(steps)
    target = o.get_field(abi.FIELD_CONC).astype(np.float64)

    def loss(imp):
        AC.init_drop(o, center, r, imp)
        o.tape_forward(steps)
        d = o.get_field(abi.FIELD_CONC).astype(np.float64) - target
        return float(np.sum(d * d)), d

    _, d = loss(1.0)
    o.tape_backward((2 * d).astype(np.float32))
    ad = o.sphere_impulse(center, r, [0.0, -2.0, 0.0])
    h = 1e-4
    fd = (loss(1.0 + h)[0] - loss(1.0 - h)[0]) / (2 * h)
    assert abs(fd - ad) <= 1e-3 * abs(fd), (fd, ad)
    # the initial pressure does not influence the trajectory's dye in the
    # closed box beyond its warm start; its gradient exists and is finite
    assert np.isfinite(o.gradients()["p"]).all()


def test_trajectory_random_directions_match_central_differences(oracle_mod):
    """A -1.5 cells/step drop with N(0, 0.05) face noise (the benchmark
    drops), 8 steps: <grad, d> against central differences of the FP64 loss
    for seeded random directions of the initial MAC velocity."""
    from dropfluid import scenes
    sc = scenes.box48()
    sc.drops[0].n_parcels = 0
    sc.drops[0].w_cells_per_step = -1.5
    sc.drops[0].noise_cells_per_step = 0.05
    o = oracle_mod.OracleSim(sc.config, fp64=True)
    steps = 8

    def fwd(scale=1.0, pert=None):
        o.reset()
        w0 = sc.drops[0].w_cells_per_step
        sc.drops[0].w_cells_per_step = w0 * scale
        sc.release(o, 0)
        sc.drops[0].w_cells_per_step = w0
        for f, d in (pert or {}).items():
            o.set_field64(f, o.get_field64(f) + d)
        o.tape_forward(steps)
        return o.get_field64(abi.FIELD_CONC)

    target = fwd(1.1)
    d0 = fwd() - target
    o.tape_backward((2 * d0).astype(np.float32))
    g = o.gradients()
    rng = np.random.default_rng(2)
    shape = g["u"].shape
    eps = 1e-6
    for _ in range(3):
        d = {f: rng.standard_normal(shape) for f in (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W)}
        ad = sum(float(np.sum(g[k] * d[f])) for k, f in
                 (("u", abi.FIELD_VEL_U), ("v", abi.FIELD_VEL_V), ("w", abi.FIELD_VEL_W)))
        lp = float(np.sum((fwd(pert={f: eps * a for f, a in d.items()}) - target) ** 2))
        lm = float(np.sum((fwd(pert={f: -eps * a for f, a in d.items()}) - target) ** 2))
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - ad) <= 1e-3 * abs(fd), (fd, ad)



def test_soft_drop_gradient_matches_central_differences(oracle_mod):
    """Soft-edged drop (smoothstep edge 2 cells wide): the gradient in the
    impulse scale and in the three centre coordinates against central
    differences of the FP64 loss.  The target comes from a run with 1.1x the
    impulse and a shifted centre, so every component is non-trivial."""
    cfg, center, r = AC.drop_scene((16, 24, 16))
    o = oracle_mod.OracleSim(cfg, fp64=True)
    steps = 6

    def run(c, imp):
        AC.init_soft_drop(o, c, r, imp)
        o.tape_forward(steps)
        return o.get_field64(abi.FIELD_CONC)

    target = run([center[0] + 0.3, center[1] - 0.2, center[2] + 0.25], 1.1)

    def loss(c, imp=1.0):
        d = run(c, imp) - target
        return float(np.sum(d * d)), d

    _, d = loss(center)
    o.tape_backward((2 * d).astype(np.float32))
    g_imp, g_pos = AC.soft_drop_grad(o, center, r)
    h = 1e-4
    fd_imp = (loss(center, 1.0 + h)[0] - loss(center, 1.0 - h)[0]) / (2 * h)
    assert abs(fd_imp - g_imp) <= 1e-3 * abs(fd_imp), (fd_imp, g_imp)
    eps = 1e-2
    for k in range(3):
        cp, cm = list(center), list(center)
        cp[k] = float(np.float32(center[k] + eps))
        cm[k] = float(np.float32(center[k] - eps))
        fd = (loss(cp)[0] - loss(cm)[0]) / (cp[k] - cm[k])
        assert abs(fd - g_pos[k]) <= 1e-3 * np.linalg.norm(g_pos), (k, fd, g_pos)
