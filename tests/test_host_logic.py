"""Host-side logic: the seeded scene generator, the scene runner's release
schedule, and the replica timing reduction used by bench.py under
torchrun (gloo, world size 2, CPU)."""
import os
import socket
import sys

import numpy as np
import pytest

from dropfluid import abi, scenes


def test_splitmix64_known_answer():
    """Published SplitMix64 outputs for seed 1234567."""
    out = scenes.SplitMix64(1234567).next_u64(5)
    assert list(map(int, out)) == [6457827717110365317, 3203168211198807973, 9817491932198370423,
                                   4593380528125082431, 16408922859458223821]


def test_stream_is_sequential():
    a = scenes.SplitMix64(99)
    x = np.concatenate([a.next_u64(3), a.next_u64(4)])
    assert np.array_equal(x, scenes.SplitMix64(99).next_u64(7))


def test_parcels_uniform_in_sphere():
    p = scenes.parcels_in_sphere((10.0, 20.0, 30.0), 4.0, 20000, 0)
    d = np.linalg.norm(p[:, :3] - np.array([10.0, 20.0, 30.0]), axis=1)
    assert d.max() <= 4.0 + 1e-5
    # uniform in volume: a quarter of the volume lies within r/4^(1/3)
    frac = (d < 4.0 * 0.25 ** (1 / 3)).mean()
    assert abs(frac - 0.25) < 0.02
    assert np.all(p[:, 3] == np.float32(0.134))
    assert np.array_equal(p, scenes.parcels_in_sphere((10.0, 20.0, 30.0), 4.0, 20000, 0))


def test_box192_scene_matches_configuration():
    sc = scenes.box192()
    c = sc.config
    assert (c.nx, c.ny, c.nz) == (192, 256, 192)
    assert [d.release_step for d in sc.drops] == [0, 40, 80]
    assert sum(d.n_parcels for d in sc.drops) == 393216 == c.parcel_capacity
    for d in sc.drops:
        x, y, z = d.center
        assert d.radius == 12.0
        assert 0.8 * c.ny <= y <= c.ny - d.radius
        assert d.radius < x < c.nx - d.radius and d.radius < z < c.nz - d.radius
        assert d.w_cells_per_step == -1.5 and d.noise_cells_per_step == 0.05
    # 2+2 RBGS V-cycles, 4 per step, on a hierarchy deepened to a 12x16x12
    # coarsest grid that is solved exactly
    assert c.mg_pre == c.mg_post == 2 and c.mg_cycles == 4
    assert c.mg_levels == 5 and c.mg_coarse_sweeps == -1
    assert scenes.box192(abi.DOB_PREC_MIXED).config.precision_mode == abi.DOB_PREC_MIXED


def test_box48_scene_matches_configuration():
    sc = scenes.box48()
    c = sc.config
    assert (c.nx, c.ny, c.nz) == (48, 64, 48)
    assert c.dx == 1.0 and abs(c.dt - 0.02) < 1e-9
    assert abs(c.casson_tau_y - 0.005) < 1e-9 and abs(c.casson_mu_p - 1e-3) < 1e-9
    d = sc.drops[0]
    assert d.center == (24.0, 56.0, 24.0) and d.radius == 4.0 and d.w_cells_per_step == -2.0
    assert d.n_parcels == 8192 and sc.steps == 20


class _Recorder:
    def __init__(self):
        self.calls = []

    def inject_sphere(self, *a):
        self.calls.append(("inject",) + a[:2])

    def set_parcels(self, p, off):
        self.calls.append(("parcels", len(p), off))

    def step(self, n=1, **kw):
        self.calls.append(("step", n))


def test_runner_releases_on_schedule():
    sc = scenes.box192()
    for d in sc.drops:
        d.n_parcels = 10
    r = _Recorder()
    scenes.run(sc, r, steps=85)
    kinds = [c[0] for c in r.calls]
    assert kinds.count("inject") == 3
    assert r.calls[0][0] == "inject"
    idx = [i for i, c in enumerate(r.calls) if c[0] == "inject"]
    steps_before = [sum(1 for c in r.calls[:i] if c[0] == "step") for i in idx]
    assert steps_before == [0, 40, 80]
    offs = [c[2] for c in r.calls if c[0] == "parcels"]
    assert offs == [0, 10, 20]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    d = bench.Dist(world)
    d.barrier()
    m = d.max(10.0 + rank)
    d.close()
    q.put((rank, m))


def test_replica_timing_max_over_ranks_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res == {0: 11.0, 1: 11.0}
