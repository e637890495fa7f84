"""Shared cases of the discrete-adjoint tests: seeded closed-box states, the
stage table (which forward fields a stage reads and writes, and which
adjoint fields carry their cotangents) and small trajectory scenes.

Stage states use smooth sinusoidal fields (no white noise) with a centre
velocity of a few tenths of a cell per step, so departure points sit away
from cell centres and the dye limiter is rarely at a tie; there the stage
maps are differentiable and central differences are meaningful.
"""
from __future__ import annotations

import numpy as np

from dropfluid import abi

# stage -> (forward inputs, forward outputs, {input field: adjoint field}, {output field: adjoint field})
STAGES = {
    abi.STAGE_ADVECT_MAC: ([0, 1, 2, 3], [0, 1, 2], {0: 16, 1: 17, 2: 18, 3: 22}, {0: 19, 1: 20, 2: 21}),
    abi.STAGE_MAC_TO_CENTER: ([0, 1, 2], [3], {0: 16, 1: 17, 2: 18}, {3: 22}),
    abi.STAGE_CASSON_FORCES: ([0, 1, 2, 7], [0, 1, 2], {0: 16, 1: 17, 2: 18, 7: 23}, {0: 19, 1: 20, 2: 21}),
    abi.STAGE_MAC_RHS: ([0, 1, 2], [6], {0: 16, 1: 17, 2: 18}, {6: 27}),
    abi.STAGE_PRESSURE_SOLVE: ([5, 6], [5], {5: 26, 6: 27}, {5: 26}),
    abi.STAGE_PROJECT: ([0, 1, 2, 5], [0, 1, 2], {0: 16, 1: 17, 2: 18, 5: 26}, {0: 16, 1: 17, 2: 18}),
    abi.STAGE_CONC_PREDICT: ([7, 3], [8], {7: 23, 3: 22}, {8: 25}),
    abi.STAGE_CONC_RESOLVE: ([7, 8, 3], [7], {7: 23, 8: 25, 3: 22}, {7: 24}),
}
LINEAR = (abi.STAGE_MAC_TO_CENTER, abi.STAGE_MAC_RHS, abi.STAGE_PRESSURE_SOLVE, abi.STAGE_PROJECT)
ADJ_FIELDS = tuple(range(abi.FIELD_ADJ_VEL_U, abi.FIELD_ADJ_RHS + 1))


def sines(shape, seed, amp, modes=4):
    """Sum of low-frequency separable sinusoids, max |f| = amp."""
    rng = np.random.default_rng(seed)
    g = np.meshgrid(*[np.linspace(0, 1, n, endpoint=False) for n in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(modes):
        k = rng.integers(1, 3, size=len(shape))
        ph = rng.uniform(0, 2 * np.pi, size=len(shape))
        t = np.ones(shape)
        for d in range(len(shape)):
            t = t * np.sin(2 * np.pi * k[d] * g[d] + ph[d])
        f += rng.uniform(-1, 1) * t
    return amp * f / np.abs(f).max()


def box_config(n=(16, 24, 16), levels=3):
    c = abi.config_closed_box(*n)
    c.mg_levels = levels
    c.parcel_capacity = 64
    return c


def stage_state(cfg, seed=0, speed=20.0):
    """Forward fields of a smooth moving state (float32 arrays by field id)."""
    sh = (cfg.nz, cfg.ny, cfg.nx)
    st = {}
    for k, f in enumerate((abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W)):
        st[f] = sines(sh, seed + k, speed).astype(np.float32)
    cen = np.zeros(sh + (4,), np.float32)
    for k in range(3):
        cen[..., k] = sines(sh, seed + 10 + k, speed)
    st[abi.FIELD_VEL_CENTER] = cen
    st[abi.FIELD_PRESSURE] = sines(sh, seed + 20, 1.0).astype(np.float32)
    rhs = sines(sh, seed + 21, 1.0)
    st[abi.FIELD_RHS] = (rhs - rhs.mean()).astype(np.float32)
    st[abi.FIELD_CONC] = (0.5 + 0.4 * sines(sh, seed + 30, 1.0)).astype(np.float32)
    st[abi.FIELD_CONC_PRED] = (0.5 + 0.4 * sines(sh, seed + 31, 1.0)).astype(np.float32)
    return st


def load(engine, st):
    for f, a in st.items():
        engine.set_field(f, a)


def zero_adjoints(engine):
    for f in ADJ_FIELDS:
        shape, _ = engine.field_shape(f) if hasattr(engine, "field_shape") else engine._field_shape(f)
        engine.set_field(f, np.zeros(shape, np.float32))


def seeded_cotangents(engine, fields, seed):
    rng = np.random.default_rng(seed)
    out = {}
    for f in fields:
        shape, _ = engine.field_shape(f) if hasattr(engine, "field_shape") else engine._field_shape(f)
        a = rng.standard_normal(shape).astype(np.float32)
        if f == abi.FIELD_VEL_CENTER:
            a[..., 3] = 0.0
        out[f] = a
    return out


def run_stage_adjoint(engine, st, stage, ybar):
    """Load the state, zero every adjoint field, set the output cotangents and
    run the stage's adjoint; returns {input field: adjoint array}."""
    ins, outs, adj_in, adj_out = STAGES[stage]
    load(engine, st)
    zero_adjoints(engine)
    for f, a in ybar.items():
        engine.set_field(adj_out[f], a)
    engine.adjoint_stage(stage)
    return {f: engine.get_field(adj_in[f]) for f in ins}


def drop_scene(n=(24, 32, 24), levels=3):
    cfg = box_config(n, levels)
    center = [n[0] / 2.0, n[1] * 0.7, n[2] / 2.0]
    return cfg, center, 4.0


def init_drop(engine, center, radius, impulse=1.0):
    engine.reset()
    engine.inject_sphere(center, radius, 1.0, [0.0, -2.0 * impulse, 0.0], 0.05, 7)


SOFT_EDGE = 2.0  # world units (cells at dx = 1)


def init_soft_drop(engine, center, radius, impulse=1.0, edge=SOFT_EDGE):
    """Rest state plus a soft-edged drop (dob_inject_sphere_soft) moving down
    at 2 cells/step times `impulse`, with N(0, 0.05) face noise."""
    engine.reset()
    engine.inject_sphere_soft(center, radius, edge, 1.0, [0.0, -2.0 * impulse, 0.0], 0.05, 7)


def soft_drop_grad(engine, center, radius, edge=SOFT_EDGE):
    """(d loss / d impulse, d loss / d centre) after tape_backward."""
    return engine.sphere_soft_grad(center, radius, edge, 1.0, [0.0, -2.0, 0.0], 0.05, 7)
