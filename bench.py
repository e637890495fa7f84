#!/usr/bin/env python3
"""Benchmark of the GB300 drop-of-blood MAC fluid step.

Workload (one "step" = one full fluid step of the scene, inputs resident in
HBM): the 192x256x192 closed-box drop scene with three r=12 drops released
at steps 0/40/80 and 393216 parcels, FP32 storage, 4 V-cycles of 2+2
red-black sweeps per step (8 on the two steps after each release) on 5
grids with an exact solve of the 12x16x12 coarsest grid
(dropfluid.scenes.box192).  The mixed-precision variant of the
same scene and the discrete adjoint are measured beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --accuracy      # FP32 and mixed vs an FP64 run at steps 50/100/200
  python bench.py --configs       # per-configuration GPU and host-core throughput

Multi-GPU: the step does not exchange data between replicas on this pool
(one GPU per box): N ranks run N independent replicas ("scaling": "weak");
rank 0 prints one JSON line with the whole-job throughput (sum over
replicas, timed as the max over ranks).

--impl reference runs the CPU restatement of the reference step (the
oracle; the reference itself is TypeScript + WGSL for a browser's WebGPU
and cannot run here) on the host cores, on the same scene, and prints the
same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "drop-of-blood_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "steps/s @192x256x192: mixed vs FP32 at div<1e-5; adjoint/forward step ratio"
WORKLOAD = ("box192: 192x256x192 closed-box MAC step, 3 drops r=12 released at steps 0/40/80, 393216 parcels, "
            "FP32 storage, 4 V-cycles of 2+2 RBGS on 5 grids with an exact 12x16x12 coarsest solve (8 V-cycles "
            "on the two steps after each release), Casson tau_y=0.005 mu_p=1e-3, dx=1 dt=0.02")


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Host-side barrier and max-reduction for replica timing (gloo, CPU)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/roofline_traffic.json), scaled to this workload."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d
    except (OSError, ValueError):
        return None


def run_scene_steps(scene, eng, start, n, timed, graph=True):
    """Advance n steps from `start`, releasing drops on schedule.  Returns
    the device milliseconds of the step segments when `timed` (releases are
    host calls between segments and are not timed).  graph=False (untimed
    only) launches the steps kernel by kernel instead of replaying a graph."""
    total = 0.0
    k = start
    end = start + n
    while k < end:
        for d in scene.releases_at(k):
            scene.release(eng, d)
        nxt = end
        for d in scene.drops:
            if k < d.release_step < nxt:
                nxt = d.release_step
        seg = nxt - k
        if timed:
            total += eng.time_steps(seg)
        else:
            eng.step(seg, graph=graph)
        k = nxt
    return total


def cpu_baseline(scene_fn, steps, threads):
    import oracle
    oracle.build()
    oracle.set_threads(threads)
    sc = scene_fn()
    sim = oracle.OracleSim(sc.config)
    for d in sc.releases_at(0):
        sc.release(sim, d)
    sim.step(1)  # warm-up
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    return steps / dt, dt


def wave_leg(peak):
    """The 512x512 wave solver (wave.ts:55-388) on a reference-mode context
    made with DOB_PHYS_WAVE, one drop at the surface: device time of one
    substep (its four kernels) over 50 launches after 5 warm-up ones, with
    88 algorithmic bytes per texel.  Errors are reported in the line, not
    raised, so the headline number never depends on this leg."""
    try:
        from dropfluid import DropFluid, abi, uniforms as U
        c = abi.config_reference()
        c.nx, c.ny, c.nz = 32, 48, 32
        c.mg_levels = 3
        c.parcel_capacity = 4096
        c.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE
        e = DropFluid(c)
        snap = U.DropSnapshot(sim_time=0.4, active_count=1)
        snap.slots[0] = U.DropSlot(active=True, center=(0.03, 0.285, -0.02), radius=0.05, vel_y=-0.3,
                                   oscillation=0.01, vol_drain_rate=0.42, seed=1.5)
        e.set_uniforms(U.SimUniformPacker().pack(drops=snap, dt=1.0 / 60.0, global_seed=1.5).copy())
        e.reset()
        e.bench_kernel(1, reps=5)
        ms, nbytes = e.bench_kernel(1, reps=50)
        gbs = nbytes / (ms * 1e-3) / 1e9
        return {"us_per_substep": ms * 1e3, "bytes_per_substep": nbytes, "achieved_gbs": gbs,
                "frac_of_measured_hbm": gbs / peak, "kernels": 4,
                "note": "2 MB complex spectrum, L2-resident; one substep per step, timed alone"}
    except Exception as ex:  # reported, never fatal
        return {"error": f"{type(ex).__name__}: {ex}"}


def impulse_step(w_cells, h, dx, dt):
    """The injected face velocity is a float32: the scales 1 +- h reach the
    fields as float32(v (1 +- h)) / v.  Returns the realised difference of
    the two scales, the denominator of the central difference."""
    import numpy as np
    v = w_cells * dx / dt
    return (float(np.float32(v * (1.0 + h))) - float(np.float32(v * (1.0 - h)))) / v


def fd64_check(sc, grads, target, d_imp, ndirs, seed=12345, h=1e-5, eps=1e-6):
    """The device gradient of the box96 loss against central differences of
    the FP64 oracle's loss (the oracle in double arithmetic, the same scene,
    V-cycles per step and target), and the FP64 oracle's own adjoint against
    the same differences: the drop impulse (scale 1 +- h, divided by the
    realised float32 difference of the injected velocities) and the same
    seeded random directions of the initial MAC velocity as the device check
    (step eps in world units against face speeds of 75: small enough that
    the FP64 trajectory crosses next to no limiter or clamp branch).  Each
    loss is 32 FP64 steps on the host cores."""
    import numpy as np
    import oracle
    from dropfluid import abi, scenes
    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    cfg = sc.config.copy()
    cfg.mg_cycles_injected = 0  # the recorded trajectory runs mg_cycles on every step
    o = oracle.OracleSim(cfg, fp64=True)
    vel = (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W)

    def loss64(scene, pert=None):
        o.reset()
        for j in scene.releases_at(0):
            scene.release(o, j)
        if pert is not None:
            for f, d in pert.items():
                o.set_field64(f, o.get_field64(f) + d)
        # the recorded trajectory's forward: centre velocity from the faces,
        # then plain steps (dob_tape_forward gives the same bits)
        o.run_stage(abi.STAGE_MAC_TO_CENTER)
        o.step(scene.steps)
        d = o.get_field64(abi.FIELD_CONC) - target
        return float(np.sum(d * d))

    fd_imp = ((loss64(scenes.box96(impulse_scale=1.0 + h)) - loss64(scenes.box96(impulse_scale=1.0 - h))) /
              impulse_step(sc.drops[0].w_cells_per_step, h, cfg.dx, cfg.dt))
    # the FP64 oracle's own discrete adjoint of its own trajectory
    o.reset()
    for j in sc.releases_at(0):
        sc.release(o, j)
    o.tape_forward(sc.steps)
    o.tape_backward((2.0 * (o.get_field64(abi.FIELD_CONC) - target)).astype(np.float32))
    g64 = {k: np.asarray(v, np.float64) for k, v in o.gradients().items()}
    d0 = sc.drops[0]
    imp64 = o.sphere_impulse(d0.center, d0.radius, (0.0, d0.w_cells_per_step * cfg.dx / cfg.dt, 0.0))
    rng = np.random.default_rng(seed)
    shape = grads["u"].shape
    errs, errs64, rows = [], [], []
    for _ in range(ndirs):
        d = {f: rng.standard_normal(shape).astype(np.float32).astype(np.float64) for f in vel}
        ad = sum(float(np.sum(grads[k].astype(np.float64) * d[f])) for k, f in zip("uvw", vel))
        ad64 = sum(float(np.sum(g64[k] * d[f])) for k, f in zip("uvw", vel))
        fd = (loss64(sc, {f: eps * a for f, a in d.items()}) - loss64(sc, {f: -eps * a for f, a in d.items()})) / (2 * eps)
        errs.append(abs(fd - ad) / max(abs(fd), 1e-30))
        errs64.append(abs(fd - ad64) / max(abs(fd), 1e-30))
        rows.append([ad, ad64, fd])
    o.close()

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
    return {"impulse_fd64": fd_imp, "impulse_rel_err": abs(d_imp - fd_imp) / abs(fd_imp),
            "impulse_adjoint64": imp64, "impulse_adjoint64_rel_err": abs(imp64 - fd_imp) / abs(fd_imp),
            "dirs": ndirs, "eps_world": eps, "h_impulse": h,
            "rel_err_max": max(errs), "rel_err_median": float(np.median(errs)),
            "adjoint64_rel_err_max": max(errs64), "adjoint64_rel_err_median": float(np.median(errs64)),
            "device_vs_adjoint64_field_rel_l2": {k: rel(np.asarray(grads[k], np.float64), g64[k]) for k in "uvw"},
            "directional": rows, "directional_columns": ["device", "FP64 adjoint", "FP64 differences"],
            "host_s": time.perf_counter() - t0,
            "reference": "FP64 oracle (double arithmetic on the host cores), same scene, target and V-cycles"}


def adjoint_leg(fd_dirs: int = 16, fd64_dirs: int = 16):
    """Forward/backward pair of the discrete adjoint.

    box96 (96x128x96, one r=8 drop with N(0, 0.05) face noise, 32 steps,
    checkpoints every 8): loss =
    ||dye - target||^2 with the target from the same scene at 1.1x the drop
    impulse; gradient w.r.t. the initial MAC velocity and the impulse, checked
    against central differences (impulse, and 16 seeded random directions of
    the initial velocity).  box192 (three soft-edged r=12 drops injected at
    step 0, 64 steps, checkpoints every 16): the full-size cost and the
    gradient in the three impulses and release positions, against central
    differences.  The ratio is the wall time per step of dob_tape_backward
    right after its dob_tape_forward (recomputation of every segment but the
    last, which the forward records) over the device time of one forward
    step of the same scene; tape_forward_ms_per_step is the wall time per
    step of that forward (checkpoints and the recorded last segment)."""
    import numpy as np
    from dropfluid import DropFluid, abi, scenes
    from dropfluid.adjoint import DropTrajectory, l2_loss

    def cost(scene, k, release_all=False):
        eng = DropFluid(scene.config)
        traj = DropTrajectory(eng, k)

        def fwd(sc, pert=None):
            eng.reset()
            for j in (range(len(sc.drops)) if release_all else sc.releases_at(0)):
                sc.release(eng, j)
            if pert is not None:
                for f, d in pert.items():
                    eng.set_field(f, eng.get_field(f) + d)
            return traj.forward(sc.steps)
        return eng, traj, fwd

    out = {}
    # ---- box96 -----------------------------------------------------------------------------------
    sc = scenes.box96()
    eng, traj, fwd = cost(sc, 8)
    target = fwd(scenes.box96(impulse_scale=1.1)).astype(np.float64)
    loss, g = l2_loss(fwd(sc), target)
    grads = traj.backward(g)  # first call captures the segment graphs
    eng.sync()
    t0 = time.perf_counter()
    fwd(sc)
    eng.sync()
    t_tape_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    grads = traj.backward(g)
    eng.sync()
    t_bwd = time.perf_counter() - t0
    d_imp = traj.drop_impulse_grad(sc, sc.drops[0])
    fwd_ms = eng.time_steps(sc.steps) / sc.steps  # state after the run: same scene, same cost
    h = 1e-3
    lp = l2_loss(fwd(scenes.box96(impulse_scale=1.0 + h)), target)[0]
    lm = l2_loss(fwd(scenes.box96(impulse_scale=1.0 - h)), target)[0]
    fd_imp = (lp - lm) / impulse_step(sc.drops[0].w_cells_per_step, h, sc.config.dx, sc.config.dt)
    rng = np.random.default_rng(12345)
    eps = 1e-3 * 75.0  # 0.1 % of the injected face speed (1.5 cells/step = 75 world units)
    errs = []
    shape = eng.field_shape(abi.FIELD_VEL_U)[0]
    for _ in range(fd_dirs):
        d = {f: rng.standard_normal(shape).astype(np.float32) for f in
             (abi.FIELD_VEL_U, abi.FIELD_VEL_V, abi.FIELD_VEL_W)}
        ad = sum(float(np.sum(grads[k].astype(np.float64) * d[f])) for k, f in
                 (("u", abi.FIELD_VEL_U), ("v", abi.FIELD_VEL_V), ("w", abi.FIELD_VEL_W)))
        lp = l2_loss(fwd(sc, {f: eps * a for f, a in d.items()}), target)[0]
        lm = l2_loss(fwd(sc, {f: -eps * a for f, a in d.items()}), target)[0]
        fd = (lp - lm) / (2 * eps)
        errs.append(abs(fd - ad) / max(abs(fd), 1e-30))
    fd64 = fd64_check(sc, grads, target, d_imp, fd_dirs) if fd64_dirs else None
    out["box96"] = {
        "fd64": fd64,
        "steps": sc.steps, "checkpoint_every": 8, "loss": loss,
        "forward_step_ms": fwd_ms, "tape_forward_ms_per_step": 1e3 * t_tape_fwd / sc.steps,
        "backward_ms_per_step": 1e3 * t_bwd / sc.steps,
        "ratio": 1e3 * t_bwd / sc.steps / fwd_ms,
        "impulse_grad": d_imp, "impulse_fd": fd_imp, "impulse_rel_err": abs(d_imp - fd_imp) / abs(fd_imp),
        "fd_dirs": fd_dirs, "fd_eps": eps, "fd_rel_err_max": max(errs), "fd_rel_err_median": float(np.median(errs)),
    }
    eng.close()
    # ---- box192, three soft-edged drops at step 0, 64 steps, checkpoints every 16 --------------
    # gradient in the three impulses and the three release positions, each
    # checked against central differences of the device loss; in FP32 and in
    # the mixed mode (whose gradients are also set against the FP32 ones)
    out["box192"] = box192_adjoint(abi.DOB_PREC_FP32)
    out["box192_mixed"] = box192_adjoint(abi.DOB_PREC_MIXED)
    fp32, mx = out["box192"], out["box192_mixed"]
    gi32, gim = np.asarray(fp32.pop("_impulse")), np.asarray(mx.pop("_impulse"))
    gp32, gpm = np.asarray(fp32.pop("_position")), np.asarray(mx.pop("_position"))
    mx["impulse_rel_diff_vs_fp32"] = float(np.max(np.abs(gim - gi32) / np.abs(gi32)))
    mx["position_rel_diff_vs_fp32"] = float(max(np.linalg.norm(gpm[k] - gp32[k]) / np.linalg.norm(gp32[k])
                                                 for k in range(len(gp32))))
    return out


def box192_adjoint(precision, checkpoint_every=64):
    """Cost and drop gradients of the 64-step box192 trajectory (three
    soft-edged drops at step 0) in one precision mode: backward / forward
    ratio, the recording forward per step, the impulse and release-position
    gradients against central differences of the device loss.  The whole
    trajectory's linearisation points stay on the tape in HBM (about 0.45
    GB per step in FP32, 29 GB for 64 steps), so the backward recomputes
    nothing; the memory-lean schedule (checkpoints every 16 steps, three of
    four segments recomputed in the backward) is timed beside it."""
    import numpy as np
    from dropfluid import DropFluid, abi, scenes
    from dropfluid.adjoint import DropTrajectory, l2_loss

    def scene(**kw):
        return scenes.box192_adjoint(precision=precision, **kw)
    sc = scene()
    eng = DropFluid(sc.config)
    traj = DropTrajectory(eng, checkpoint_every)

    def fwd192(sn):
        eng.reset()
        for j in range(len(sn.drops)):
            sn.release(eng, j)
        return traj.forward(sn.steps)
    shifts = ((0.5, -0.3, 0.2), (-0.4, 0.2, 0.3), (0.3, 0.4, -0.5))
    target = fwd192(scene(impulse_scale=(1.1, 0.9, 1.05), shift=shifts)).astype(np.float64)
    loss, g = l2_loss(fwd192(sc), target)
    traj.backward(g)  # first call captures the segment graphs
    eng.sync()
    # the timed backward follows its forward, as in a gradient step
    t0 = time.perf_counter()
    fwd192(sc)
    eng.sync()
    t_tape_fwd192 = time.perf_counter() - t0
    t0 = time.perf_counter()
    traj.backward(g)
    eng.sync()
    t_bwd = time.perf_counter() - t0
    drop_g = [traj.drop_grads(sc, k) for k in range(len(sc.drops))]
    fwd_ms = eng.time_steps(8) / 8
    h, eps = 1e-2, 5e-2
    imp_err, pos_err, fd_pos = [], [], []
    for k in range(len(sc.drops)):
        sp = [1.0] * 3
        sm = [1.0] * 3
        sp[k], sm[k] = 1.0 + h, 1.0 - h
        fd = (l2_loss(fwd192(scene(impulse_scale=sp)), target)[0] -
              l2_loss(fwd192(scene(impulse_scale=sm)), target)[0]) / (2 * h)
        imp_err.append(abs(fd - drop_g[k]["impulse"]) / abs(fd))
        fdk = []
        for j in range(3):
            shp = [[0.0] * 3 for _ in range(3)]
            shm = [[0.0] * 3 for _ in range(3)]
            shp[k][j], shm[k][j] = eps, -eps
            fd = (l2_loss(fwd192(scene(shift=shp)), target)[0] -
                  l2_loss(fwd192(scene(shift=shm)), target)[0]) / (2 * eps)
            fdk.append(fd)
        gp = drop_g[k]["position"]
        fd_pos.append(fdk)
        pos_err.append(float(np.linalg.norm(np.asarray(fdk) - gp) / np.linalg.norm(gp)))
    c = sc.config
    n, nc = c.nx * c.ny * c.nz, c.nx * c.ny * c.nz * c.dye_refine ** 3
    dye_b = 2 if precision == abi.DOB_PREC_MIXED else 4
    res = {"steps": sc.steps, "checkpoint_every": checkpoint_every,
           "tape_gb": checkpoint_every * (40 * n + 2 * dye_b * nc) / 1e9, "forward_step_ms": fwd_ms,
           "tape_forward_ms_per_step": 1e3 * t_tape_fwd192 / sc.steps,
           "backward_ms_per_step": 1e3 * t_bwd / sc.steps, "ratio": 1e3 * t_bwd / sc.steps / fwd_ms,
           "gradient_cost_ratio": 1e3 * (t_tape_fwd192 + t_bwd) / sc.steps / fwd_ms,
           "loss": loss, "drops": "three soft-edged drops (edge 2 cells) injected at step 0, 393216 parcels",
           "target": "same drops with impulses x(1.1, 0.9, 1.05) and centres shifted by up to 0.5 cells",
           "impulse_grad": [d["impulse"] for d in drop_g],
           "position_grad": [d["position"].tolist() for d in drop_g],
           "position_fd": fd_pos,
           "impulse_fd_rel_err_max": max(imp_err),
           "position_fd_rel_err_max": max(pos_err),
           "fd_steps": {"impulse": h, "position_world": eps},
           "_impulse": [d["impulse"] for d in drop_g], "_position": [d["position"] for d in drop_g]}
    if precision == abi.DOB_PREC_MIXED:
        res["precision"] = ("mixed: binary16 dye, pressure pair to max |div| dt/dx <= 1e-5; the adjoint reads the "
                            "binary16 linearisation points and solves the pressure adjoint with the mixed solver "
                            "to a relative residual of 1e-6")
    if checkpoint_every != 16:
        # the memory-lean schedule on the same trajectory and loss gradient
        t16 = DropTrajectory(eng, 16)

        def fwd16():
            eng.reset()
            for j in range(len(sc.drops)):
                sc.release(eng, j)
            t16.forward(sc.steps)
        fwd16()
        t16.backward(g)  # captures the segment graphs
        eng.sync()
        t0 = time.perf_counter()
        fwd16()
        eng.sync()
        tf16 = time.perf_counter() - t0
        t0 = time.perf_counter()
        t16.backward(g)
        eng.sync()
        tb16 = time.perf_counter() - t0
        res["checkpoint_every_16"] = {
            "tape_gb": 16 * (40 * n + 2 * dye_b * nc) / 1e9,
            "tape_forward_ms_per_step": 1e3 * tf16 / sc.steps, "backward_ms_per_step": 1e3 * tb16 / sc.steps,
            "ratio": 1e3 * tb16 / sc.steps / fwd_ms, "gradient_cost_ratio": 1e3 * (tf16 + tb16) / sc.steps / fwd_ms}
    eng.close()
    return res


ACC_STEPS = (50, 100, 200)
ACC_FIELDS = ("u", "v", "w", "p", "dye")


def accuracy_run():
    """FP32 and mixed-precision (||b - Ap|| / ||b|| <= 1e-8) runs of the
    box192 scene on the GPU against an FP64 run of the same seed: the oracle
    in double arithmetic with 12 V-cycles per step (a pressure solve
    converged to the FP64 floor: the V-cycle contracts 0.1 per cycle), on the
    host cores.  Relative L2 errors of u, v, w, p and dye at steps 50, 100
    and 200."""
    import numpy as np
    import oracle
    from dropfluid import DropFluid, abi, scenes
    F = {"u": abi.FIELD_VEL_U, "v": abi.FIELD_VEL_V, "w": abi.FIELD_VEL_W, "p": abi.FIELD_PRESSURE,
         "dye": abi.FIELD_CONC}

    def trajectory(scene, eng):
        snaps, k = {}, 0
        for s in ACC_STEPS:
            run_scene_steps(scene, eng, k, s - k, timed=False)
            k = s
            get = getattr(eng, "get_field64", eng.get_field)  # the oracle's double fields unrounded
            snaps[s] = {n: np.asarray(get(f), np.float64) for n, f in F.items()}
        return snaps

    t0 = time.perf_counter()
    runs = {}
    for name, sc in (("fp32", scenes.box192()), ("mixed_rel_1e-8", scenes.box192_mixed_1e8())):
        with DropFluid(sc.config) as eng:
            runs[name] = trajectory(sc, eng)
    t_gpu = time.perf_counter() - t0
    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    ref_sc = scenes.box192()
    ref_sc.config.mg_cycles = 12
    t0 = time.perf_counter()
    ref = trajectory(ref_sc, oracle.OracleSim(ref_sc.config, fp64=True))
    t_cpu = time.perf_counter() - t0

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
    out = {name: {str(s): {n: rel(r[s][n], ref[s][n]) for n in ACC_FIELDS} for s in ACC_STEPS}
           for name, r in runs.items()}
    return {"accuracy_vs_fp64": out, "steps": list(ACC_STEPS),
            "reference": "FP64 oracle (CPU, double arithmetic), same scene and seed, 12 V-cycles per step",
            "metric": "relative L2 error vs the FP64 run; pressure mean-free (closed box)",
            "gpu_s": t_gpu, "fp64_cpu_s": t_cpu}


def reference_sequence(warm_substeps=56):
    """The reference setup's host input from the drop-lifecycle restatement
    (dropfluid.sequencer, BloodDropEngine.ts:1682-1844): the reset block and
    the blocks of the first `warm_substeps` fixed 1/60 s substeps, whose last
    ones cover the first drop's impact on the meniscus (0.92 s, substep 56)
    and the start of its drainage and parcel emission."""
    from dropfluid.sequencer import SubstepSequencer
    seq = SubstepSequencer(seed=1.0)
    reset = seq.reset_simulation(1.0)
    blocks = [seq.advance_substep()[0] for _ in range(warm_substeps)]
    return seq, reset, blocks


# Algorithmic bytes of one reference-mode substep, per stage: every array a
# stage reads read once and every array it writes written once, at the
# storage widths of the precision mode (vs: velocity / centre / curl
# element, ds: dye element; V velocity cells, C = 8 V dye voxels).
def reference_stage_bytes(cfg, high_water):
    from dropfluid import abi
    V = cfg.nx * cfg.ny * cfg.nz
    C = V * cfg.dye_refine ** 3
    vs = 2 if cfg.precision_mode == abi.DOB_PREC_REFERENCE_FP16 else 4
    ds = 2 if cfg.precision_mode != abi.DOB_PREC_FP32 else 4
    # V-cycle, reference schedule: level 0 one sweep before and after (12 B
    # per cell and sweep), residual + restriction and prolongation 8.5 B
    # each; levels 1-2 two and two sweeps; the 12x16x12 grid is negligible
    mg = (2 * 12 + 17) * V + (4 * 12 + 17) * (V / 8 + V / 64)
    return {
        "wave": 88 * 512 * 512 if cfg.physics_flags & abi.DOB_PHYS_WAVE else 0,
        "advect_mac": 10 * vs * V,                     # u,v,w + centre in, u,v,w out
        "mac_to_center": 2 * 7 * vs * V,               # twice: faces in, centre out
        "curl": 8 * vs * V,                            # centre in, curl out
        "casson_forces": 10 * vs * V + 4 * ds * C,     # faces + curl in, dye sampled, faces out
        "mac_rhs": (3 * vs + 4) * V,
        "pressure_solve": mg,
        "project": (6 * vs + 4) * V,
        "clear_splats": 8 * C,
        "parcel_advect": 64 * high_water,              # 32 B per parcel in and out
        "conc_predict": 5 * ds * C + 4 * vs * V,       # dye in, predictor out, centre sampled
        "conc_resolve": (9 * ds + 8) * C + 4 * vs * V,  # dye, predictor, two splats in, dye out
    }


RENDER_W, RENDER_H = 960, 540  # the reference renders its volume pass at half of a 1920x1080 canvas


def render_frame(e, block, cfg):
    """The plume render (dob_render_plume) of the live state: a submerged
    camera 0.6 m in front of the impact point, just below the meniscus,
    looking up at the drained plume, the last substep's drops, a synthetic
    stand-in for the spectral table; one render for the image (light volume
    + march, copied to the host), then 10 timed launches of the march alone
    (dob_bench_kernel 3)."""
    import numpy as np
    from dropfluid import uniforms as U
    eye, target = (0.0, 0.10, 0.60), (0.0, 0.20, 0.0)
    vp, ivp = U.camera_matrices(eye, target, 40.0, RENDER_W / RENDER_H)
    blk = np.array(block, np.float32).copy()
    blk[0:16], blk[16:32], blk[32:35] = ivp, vp, eye
    blk[36], blk[37] = RENDER_W, RENDER_H
    blk[56] = max(0.20, float(np.linalg.norm(np.subtract(target, eye))))
    e.set_uniforms(blk)
    e.set_spectral_lut(U.synthetic_spectral_lut())
    img = e.render_plume(RENDER_W, RENDER_H)
    f = img.view(np.float16).astype(np.float32)
    e.bench_kernel(3, reps=2)
    ms, _ = e.bench_kernel(3, reps=10)
    px = RENDER_W * RENDER_H
    out = {"width": RENDER_W, "height": RENDER_H, "ms_per_frame": ms, "rays_per_s": px / (ms * 1e-3),
           "frames_per_s": 1e3 / ms, "pixels_through_dye": float((f[..., 3] > 0).mean()),
           "tau_total_max": float(f[..., 3].max()),
           "note": "marchPlume (render.ts:1593-2109) from fsMain's camera ray as the submerged primary march, "
                   "one thread per pixel; synthetic spectral table; light volume not included in the time"}
    # the same frame at a quarter of the pixels by the oracle on the host
    # cores (its restatement of the march), bits compared with the device's
    try:
        import oracle
        from dropfluid import abi
        oracle.build()
        oracle.set_threads(os.cpu_count() or 1)
        w, h = RENDER_W // 2, RENDER_H // 2
        vp2, ivp2 = U.camera_matrices(eye, target, 40.0, w / h)
        blk[0:16], blk[16:32], blk[36], blk[37] = ivp2, vp2, w, h
        e.set_uniforms(blk)
        dev = e.render_plume(w, h)
        o = oracle.OracleSim(cfg)
        o.set_uniforms(blk)
        for fld in (abi.FIELD_CONC, abi.FIELD_WAVE):
            o.set_field(fld, e.get_field(fld))
        t0 = time.perf_counter()
        host = o.render_plume(w, h, U.synthetic_spectral_lut())
        t = time.perf_counter() - t0
        o.close()
        out["cpu_reference"] = {"width": w, "height": h, "seconds": t, "rays_per_s": w * h / t,
                                "cores": os.cpu_count(), "bits_equal_device": bool(np.array_equal(dev, host)),
                                "kind": "port (oracle restatement, light volume included)"}
    except Exception as ex:  # reported in the line, not raised
        out["cpu_reference"] = {"error": str(ex)[:200]}
    return out


def reference_mode_leg(peak, substeps=60):
    """The reference's own setup (dob_config_reference: 96x128x96 velocity,
    192x256x192 four-channel dye, reference V-cycle schedule, 393216
    parcels, the wave solver each substep), driven by the host
    drop-lifecycle sequence.  After 50 untimed substeps, `substeps` more
    (the first drop's impact, drainage and parcel emission) run through
    dob_step_uniforms with a block copy per substep (wall clock, host
    included); the device time of 20 graph-replayed substeps on the last
    block; per-stage device times (stage by stage, events) against the
    stage byte model.  Errors are reported in the line, not raised."""
    try:
        import numpy as np
        from dropfluid import DropFluid, abi
        cfg = abi.config_reference()
        cfg.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE
        out = {}
        for name, prec in (("fp32", abi.DOB_PREC_FP32), ("fp16_storage", abi.DOB_PREC_REFERENCE_FP16)):
            cfg.precision_mode = prec
            seq, reset, warm = reference_sequence(50)
            e = DropFluid(cfg)
            e.set_uniforms(reset)
            e.reset()
            e.step_uniforms(np.stack(warm))
            blocks = [seq.advance_substep() for _ in range(substeps)]
            e.sync()
            t0 = time.perf_counter()
            e.step_uniforms(np.stack([b[0] for b in blocks]))
            e.sync()
            wall = time.perf_counter() - t0
            ms = e.time_steps(20) / 20.0
            tst = e.step(2, timing=True)
            stage_ms = {k: v / 2.0 for k, v in tst["stage_ms"].items() if v > 0}
            sb = reference_stage_bytes(cfg, seq.high_water)
            total = sum(sb.values())
            stages = {}
            for key, v in stage_ms.items():  # stage names as in abi.STAGE_NAMES
                b = sb.get(key)
                stages[key] = {"ms": v, "bytes": b,
                               "gbs": (b / (v * 1e-3) / 1e9) if b else None,
                               "frac": (b / (v * 1e-3) / 1e9 / peak) if b else None}
            dom = max(stages.items(), key=lambda kv: kv[1]["ms"])
            e.bench_kernel(2, reps=3)
            lk_ms, lk_bytes = e.bench_kernel(2, reps=20)
            light = {"us_per_launch": lk_ms * 1e3, "bytes_per_launch": lk_bytes,
                     "achieved_gbs": lk_bytes / (lk_ms * 1e-3) / 1e9,
                     "frac_of_measured_hbm": lk_bytes / (lk_ms * 1e-3) / 1e9 / peak,
                     "kernels": 2, "note": "light volume + brick dilation (lighting.ts:19-240), once per frame; "
                                           "20 launches on the live state, CUDA events"}
            render = render_frame(e, blocks[-1][0], cfg)
            out[name] = {
                "steps_per_s_e2e": substeps / wall, "e2e_path": "dob_step_uniforms, one 512-byte block per substep",
                "steps_per_s_device": 1e3 / ms, "ms_per_step_device": ms,
                "bytes_per_step": total, "achieved_gbs": total / (ms * 1e-3) / 1e9,
                "frac_of_measured_hbm": total / (ms * 1e-3) / 1e9 / peak,
                "spawned_parcels": int(sum(b[1] for b in blocks)), "high_water": seq.high_water,
                "stages": stages, "dominant_stage": dom[0], "light_volume": light, "plume_render": render,
                "launches_per_step": e.launches_per_step(),
            }
            e.close()
        out["workload"] = ("reference setup: 96x128x96 velocity, 192x256x192 dye, Dirichlet free-surface top, "
                           "reference V-cycle (L0 1+1, L1-L2 2+2, L3 6 sweeps), 393216-parcel ring, wave solver "
                           "each substep; uniforms from the drop-lifecycle sequence (seed 1), substeps 51-110")
        return out
    except Exception as ex:  # reported, never fatal
        return {"error": f"{type(ex).__name__}: {ex}"}


def configs_report():
    """Per configuration: GPU steps/s (graph replays, device time) and the
    oracle on the host cores (FP32 on all cores and on one, FP64 on all),
    each the median of 3 runs after 2 warm-up steps; cell-updates/s counts
    velocity cells."""
    import oracle
    from dropfluid import DropFluid, abi, scenes
    oracle.build()
    ncores = os.cpu_count() or 1

    def reference96():
        cfg = abi.config_reference()  # 96x128x96 velocity, 192x256x192 dye, 393216 parcels
        # the block of the drop-lifecycle sequence right after the first
        # drop's impact (draining, parcels spawned every substep)
        _, reset, blocks = reference_sequence(60)

        def setup(e):
            e.set_uniforms(reset)
            e.reset()
            e.set_uniforms(blocks[-1])
        return cfg, setup

    def scene_setup(sc):
        def setup(e):
            for d in sc.releases_at(0):
                sc.release(e, d)
        return sc.config, setup

    cases = [("cfg0 box48 (48x64x48, FP32)", scene_setup(scenes.box48()), 20, (20, 20, 20)),
             ("cfg1 box192 (192x256x192, FP32)", scene_setup(scenes.box192()), 20, (3, 1, 3)),
             ("cfg3 box96 (96x128x96, FP32)", scene_setup(scenes.box96()), 32, (8, 2, 8)),
             ("reference mode (96x128x96 velocity, 192x256x192 dye, free-surface top, first drop draining)",
              reference96(), 20,
              (2, 1, 2))]
    out = []
    for name, (cfg, setup), gsteps, (n32, n1, n64) in cases:
        cells = cfg.nx * cfg.ny * cfg.nz
        with DropFluid(cfg) as e:
            setup(e)
            e.step(3)
            ms = e.time_steps(gsteps)
        gpu = gsteps / (ms / 1e3)

        def cpu(fp64, threads, n):
            oracle.set_threads(threads)
            o = oracle.OracleSim(cfg, fp64=fp64)
            setup(o)
            o.step(2)
            runs = []
            for _ in range(3):
                t0 = time.perf_counter()
                o.step(n)
                runs.append(n / (time.perf_counter() - t0))
            o.close()
            v = statistics.median(runs)
            return {"steps_per_s": v, "cell_updates_per_s": v * cells, "threads": threads,
                    "sample": f"median of 3 runs of {n} steps"}
        out.append({"config": name, "cells": cells,
                    "gpu": {"steps_per_s": gpu, "cell_updates_per_s": gpu * cells, "steps": gsteps},
                    "cpu_fp32": cpu(False, ncores, n32), "cpu_fp32_1thread": cpu(False, 1, n1),
                    "cpu_fp64": cpu(True, ncores, n64)})
        print(json.dumps(out[-1]), flush=True)
    return {"configs": out, "host_cores": ncores}


# Algorithmic bytes of one closed-box step per velocity cell (every array a
# stage reads read once, every array it writes written once): the stages
# outside the pressure solve, and one V-cycle of 2+2 red-black sweeps (12 B
# per cell and sweep) with its transfers (8.5 B each) on every level, levels
# summed as L0 (1 + 1/8 + 1/64 + ...).  FP32 storage: advection 24, Casson 28,
# divergence 16, projection 28, dye advection 20, parcels 2.7 (393216 x 64 B
# over 192x256x192).  Mixed: FP16 dye (Casson 26, dye 16), BF16 levels >= 2
# (half the bytes there), and per round the error-free residual (p, plo, b in,
# r out: 16 B) and the update (e, p, plo in, p, plo out: 20 B); the tested
# cycle cut short after its pre-smoothing and restriction adds 32.5 B.
def step_bytes_per_cell(cycles, mixed=False, rounds=0, cut_short=0.0):
    lev = [1.0, 1 / 8, 1 / 64, 1 / 512, 1 / 4096]
    per_level = 4 * 12 + 8.5 + 8.5
    if not mixed:
        return 118.4 + cycles * per_level * sum(lev)
    cyc = per_level * (lev[0] + lev[1]) + 0.5 * per_level * sum(lev[2:])
    return 112.7 + cycles * cyc + rounds * (16 + 20) + cut_short * 32.5


def headline_step_roofline(scene, start, n, steps_per_s):
    """Step-level roofline of the FP32 window: V-cycles per step from the
    release rule (mg_cycles_injected on the two steps after a release)."""
    c = scene.config
    cyc = []
    for k in range(start, start + n):
        after = any(0 <= k - d.release_step < 2 for d in scene.drops)
        cyc.append(c.mg_cycles_injected if after else c.mg_cycles)
    mean_c = sum(cyc) / len(cyc)
    b = step_bytes_per_cell(mean_c) * c.nx * c.ny * c.nz
    peak, src = measured_peaks()
    gbs = b * steps_per_s / 1e9
    return {"bytes_per_step": b, "vcycles_per_step": mean_c, "achieved_gbs": gbs, "frac": gbs / peak,
            "peak_source": src, "model": "stage byte model per velocity cell (bench.step_bytes_per_cell); it "
                                         "counts the dye predictor and resolve over every voxel, while the step "
                                         "skips clear water there, so the fraction is the step's rate against "
                                         "the dense algorithm's bytes"}


def release_note(scene, start, n):
    """Which drop releases (and their extra-cycle steps) a timed window holds."""
    rel = [d.release_step for d in scene.drops if start <= d.release_step < start + n]
    if not rel:
        return f"steps {start}-{start + n - 1}: no drop release in the window"
    return f"steps {start}-{start + n - 1}: drop releases at steps {rel} (8 V-cycles on the two steps after each)"


def run_reference(args, rank, world):
    """The reference arm: the oracle (the CPU restatement of the reference
    step; the reference's own WGSL step needs a browser WebGPU stack) on all
    host cores, over the same window of the same scene as the GPU arm: W
    untimed steps from the first release, then K timed steps with the
    releases that fall inside them."""
    if rank != 0:
        return 0
    import oracle
    from dropfluid import scenes
    threads = os.cpu_count() or 1
    warmup = max(3, args.warmup)
    steps = max(1, min(args.steps, 200))
    oracle.build()
    oracle.set_threads(threads)
    sc = scenes.box192()
    sim = oracle.OracleSim(sc.config)
    t_start = time.perf_counter()
    run_scene_steps(sc, sim, 0, warmup, timed=False)
    t0 = time.perf_counter()
    run_scene_steps(sc, sim, warmup, steps, timed=False)
    secs = time.perf_counter() - t0
    value = steps / secs
    window = release_note(sc, warmup, steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [192, 256, 192], "parallelism": "replicas",
                   "timed": f"host wall clock of K oracle steps; {window}"},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} steps of box192 ({window}) after {warmup} warm-up steps, FP32 oracle "
                                   f"with OpenMP on {threads} threads: {secs:.1f} s; the reference's own WGSL step "
                                   f"needs a browser WebGPU stack, unavailable on this box"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t_start,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)  # the box192 configuration's run
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-reference-mode", action="store_true")
    ap.add_argument("--accuracy", action="store_true",
                    help="error of the FP32 and mixed runs against an FP64 run at steps 50/100/200, then exit")
    ap.add_argument("--configs", action="store_true",
                    help="per-configuration GPU and host-core throughput (FP32, FP32 1 thread, FP64), then exit")
    ap.add_argument("--profile-reference", action="store_true",
                    help="run only the reference setup on the drop-lifecycle sequence (50 substeps, then --steps "
                         "substeps, the light volume after each, untimed) and exit: the command the "
                         "reference-mode ncu captures are taken with")
    ap.add_argument("--profile-run", action="store_true",
                    help="run only the FP32 scene (warm-up + steps, untimed) and exit: the command "
                         "the ncu launch lists and kernel captures are taken with")
    ap.add_argument("--profile-scene", choices=["box192", "box96", "box192_mixed"], default="box192",
                    help="scene of --profile-run: box192 (the headline workload), box96 (96x128x96, "
                         "the small case for full-metric kernel captures) or box192_mixed (box192 with "
                         "FP16 dye and the mixed pressure solve)")
    ap.add_argument("--profile-no-graph", action="store_true",
                    help="with --profile-run: launch the steps kernel by kernel, not as graph replays (ncu "
                         "profiles no kernel of a graph that holds conditional nodes, as the mixed step's does)")
    args = ap.parse_args()
    rank, world, local = rank_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    args.warmup = max(3, args.warmup)

    from dropfluid import DropFluid, abi, build, scenes
    build.build()
    if args.accuracy:
        if rank == 0:
            print(json.dumps(accuracy_run()), flush=True)
        return 0
    if args.configs:
        if rank == 0:
            print(json.dumps(configs_report()), flush=True)
        return 0
    if args.profile_reference:
        import numpy as np
        cfg = abi.config_reference()
        cfg.physics_flags = abi.DOB_PHYS_REFERENCE_ALL | abi.DOB_PHYS_WAVE | abi.DOB_PHYS_LIGHTING
        seq, reset, warm = reference_sequence(50)
        with DropFluid(cfg) as e:
            e.set_uniforms(reset)
            e.reset()
            e.step_uniforms(np.stack(warm))
            for _ in range(args.steps):
                e.step_uniforms(seq.advance_substep()[0][None])
            e.sync()
        return 0
    dist = Dist(world)

    # ---- FP32 drop-in step (the headline) ----------------------------------------------------
    if args.profile_run and args.profile_scene == "box96":
        sc = scenes.box96()
    elif args.profile_run and args.profile_scene == "box192_mixed":
        sc = scenes.box192(abi.DOB_PREC_MIXED)
    else:
        sc = scenes.box192()
    eng = DropFluid(sc.config)
    graph = not (args.profile_run and args.profile_no_graph)
    run_scene_steps(sc, eng, 0, args.warmup, timed=False, graph=graph)
    eng.sync()
    if args.profile_run:
        run_scene_steps(sc, eng, args.warmup, args.steps, timed=False, graph=graph)
        eng.sync()
        return 0
    clocks = ClockSampler()
    clocks.start()
    dist.barrier()
    eng.sync()
    ms = run_scene_steps(sc, eng, args.warmup, args.steps, timed=True)
    eng.sync()
    dist.barrier()
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = world * args.steps / (ms_max / 1000.0)
    st = eng.step(1, stats=True)
    nstep = args.warmup + args.steps + 1
    launches = eng.launches_per_step()
    # per-stage device time (stage-by-stage launches with events)
    tst = eng.step(2, timing=True)
    stage_ms = {k: v / 2.0 for k, v in tst["stage_ms"].items() if v > 0}
    # dominant kernel: the level-0 smoother pass, timed alone on the live state
    k_ms, k_bytes = eng.bench_kernel(0, reps=20)
    peak, peak_src = measured_peaks()
    achieved = k_bytes / (k_ms * 1e-3) / 1e9
    traffic = None
    tr = ncu_traffic()
    if tr and "bytes_per_cell" in tr:
        traffic = tr["bytes_per_cell"] * sc.config.nx * sc.config.ny * sc.config.nz
    h2d, d2h = eng.io_bytes()

    # ---- end to end: public API, host parameter upload + statistics readback every step -------
    # dob_step_async / dob_step_result with two steps in flight: each step's
    # parameters go host->device from pinned memory and its statistics come
    # back device->host; the host reads step k's result while step k+1 runs.
    # The headline reads the statistics the step forms without an extra pass
    # (max |div| from the projection, ||b|| from the mean removal); a second
    # window adds the error-free residual norm and the live-parcel count.
    def pipelined(mask):
        eng.set_step_stats(mask)
        eng.sync()
        dist.barrier()
        t0 = time.perf_counter()
        stats = eng.run_pipelined(args.steps, depth=2)
        dt_s = dist.max(time.perf_counter() - t0)
        assert len(stats) == args.steps
        return world * args.steps / dt_s, stats
    e2e_value, e2e_stats = pipelined(0)
    e2e_all_value, e2e_all_stats = pipelined(abi.STATS_ALL)

    # ---- projection accuracy per step, and the mixed-precision solve ---------------------------
    # The timed window is replayed from a snapshot with statistics on, so the
    # divergence of every timed step is known.  The mixed solve iterates each
    # step until max |div| dt/dx <= 1e-5 (and, for mixed_rel_1e-8, until
    # ||b - Ap|| / ||b|| <= 1e-8, below the FP32 pressure's rounding floor).
    eng.close()
    mixed = None
    if not args.no_mixed:
        def window(scene, timed_value=None):
            e = DropFluid(scene.config)
            run_scene_steps(scene, e, 0, args.warmup, timed=False)
            e.save_state(0)
            e.sync()
            dist.barrier()
            ms_w = dist.max(run_scene_steps(scene, e, args.warmup, args.steps, timed=True))
            e.load_state(0)
            divs, iters, cycs = [], [], []
            for k in range(args.warmup, args.warmup + args.steps):
                for d in scene.releases_at(k):
                    scene.release(e, d)
                stw = e.step(1, stats=True)
                divs.append(stw["max_div"])
                iters.append(stw["outer_iters"])
                cycs.append(stw["vcycles"])
            e.close()
            v = world * args.steps / (ms_w / 1000.0)
            return {"value": v, "unit": "steps/s", "ms_per_step": ms_w / args.steps,
                    "max_div_max": max(divs), "max_div_median": statistics.median(divs),
                    "steps_div_le_1e-5": sum(1 for dv in divs if dv <= 1e-5), "steps": len(divs),
                    "outer_iters_mean": statistics.mean(iters), "vcycles_mean": statistics.mean(cycs)}
        # FP32 with a fixed number of V-cycles per step: the fewest cycles
        # that keep max |div| dt/dx <= 1e-5 on every step of the run (the
        # steps right after a drop release need more than the others) is the
        # FP32 path "at div < 1e-5" the mixed loop is compared with
        fp32 = {}
        for cyc in (4, 5, 6, 8):
            scc = scenes.box192()
            scc.config.mg_cycles = cyc
            fp32[cyc] = window(scc)
        fp32_w, fp32_8 = fp32[4], fp32[8]
        ok = [c for c in sorted(fp32) if fp32[c]["steps_div_le_1e-5"] == fp32[c]["steps"]]
        at_div = ok[0] if ok else None
        # V-cycles run in the first round before its first convergence test
        mixes = {}
        for cyc in (0, 2, 3):
            scm = scenes.box192(abi.DOB_PREC_MIXED)
            scm.config.mg_cycles = cyc
            mixes[cyc] = window(scm)
        ok_m = [c for c in sorted(mixes) if mixes[c]["steps_div_le_1e-5"] == mixes[c]["steps"]]
        best = max(ok_m, key=lambda c: mixes[c]["value"]) if ok_m else 0
        mx = mixes[best]
        m8 = window(scenes.box192_mixed_1e8())
        mixed = dict(mx)
        peak_w = measured_peaks()[0]
        cells = 192 * 256 * 192

        def step_roof(w, mixed_mode, cycles):
            b = step_bytes_per_cell(cycles, mixed_mode, w.get("outer_iters_mean", 0),
                                    1.0 if mixed_mode else 0.0) * cells
            gbs = b * w["value"] / 1e9
            return {"bytes_per_step": b, "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak_w,
                    "vcycles_per_step": cycles}
        mixed.update({
            "step_roofline": step_roof(mx, True, mx["vcycles_mean"]),
            "fp32_step_roofline": step_roof(fp32_w, False, 4),
            "untested_cycles": best,
            "by_untested_cycles": {str(c): {k: mixes[c][k] for k in ("value", "vcycles_mean", "max_div_max",
                                                                     "steps_div_le_1e-5")} for c in mixes},
            "fp32_cycles_at_div_1e-5": at_div,
            "speedup_vs_fp32_at_div_1e-5": mx["value"] / fp32[at_div]["value"] if at_div else None,
            "speedup_vs_fp32": mx["value"] / fp32_w["value"],
            "speedup_vs_fp32_8cycles": mx["value"] / fp32_8["value"],
            "precision": "FP16 dye; pressure as an FP32 pair (double-float); per round one error-free residual, "
                         "then V-cycles on the correction (BF16 levels >= 2), untested_cycles of them untested, "
                         "then tested on the restriction's residual until max |div| dt/dx <= 1e-5; "
                         "outer_iters = rounds, vcycles = V-cycles",
            "fp32_4cycles": fp32_w, "fp32_5cycles": fp32[5], "fp32_6cycles": fp32[6], "fp32_8cycles": fp32_8,
            "mixed_rel_1e-8": m8,
        })

    # ---- discrete adjoint (forward/backward pair) ---------------------------------------------------
    adj = None
    if not args.no_adjoint:
        adj = adjoint_leg()

    # ---- CPU baseline (rank 0, N=1 only) ----------------------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cval, csecs = cpu_baseline(scenes.box192, 3, threads)
        cpu = {"value": cval, "unit": "steps/s", "cores": threads, "kind": "port",
               "sample": f"3 steps of box192 (FP32 oracle, OpenMP on {threads} threads) after drop 0 "
                         f"and 1 warm-up step: {csecs:.1f} s"}

    wave = wave_leg(measured_peaks()[0]) if rank == 0 else None
    refmode = reference_mode_leg(measured_peaks()[0]) if rank == 0 and not args.no_reference_mode else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "grid": [192, 256, 192], "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (>=12 fields x 37.7 MB per step), no flush",
                       "timed": "device time of K graph-replayed steps (CUDA events on the library stream); "
                                "drop releases between segments untimed; "
                                + release_note(sc, args.warmup, args.steps)},
            "cell_updates_per_s": value * 192 * 256 * 192,
            "step_roofline": headline_step_roofline(sc, args.warmup, args.steps, value),
            "max_div": st["max_div"], "residual_l2": st["residual_l2"], "rhs_l2": st["rhs_l2"],
            "mixed": mixed,
            "adjoint_forward_ratio": adj["box96"]["ratio"] if adj else None,
            "adjoint": adj,
            "wave": wave,
            "reference_mode": refmode,
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "DropFluid.run_pipelined (dob_step_async + dob_step_result, 2 steps in flight): "
                            "params host->device from pinned memory, step graph with statistics (max |div| and "
                            "||b||, formed by the projection and the mean removal), statistics device->host into "
                            "pinned memory, host waits for every step's result",
                    "max_div_max": max(x["max_div"] for x in e2e_stats),
                    "all_statistics": {"value": e2e_all_value,
                                       "adds": "the error-free residual norm ||b - A p|| and the live-parcel count "
                                               "every step (dob_set_step_stats(DOB_STATS_ALL))",
                                       "residual_l2_max": max(x["residual_l2"] for x in e2e_all_stats),
                                       "max_div_max": max(x["max_div"] for x in e2e_all_stats)}},
            "gpu_launches": launches * args.steps,
            "launches_per_step": launches,
            "stage_ms": stage_ms,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "level-0 RBGS smoother pass (red + black sweep of p), timed alone on the live "
                                   "state with CUDA events, 20 launches",
                         "algorithmic_bytes_per_launch": k_bytes, "avg_launch_ms": k_ms, "peak_source": peak_src},
            "clocks": clk,
            "cpu_baseline": cpu,
            "steps_total": nstep,
        }
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
