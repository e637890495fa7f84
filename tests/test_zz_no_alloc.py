"""dob_pressure_solve_noalloc: the pressure solve for callers that cannot
allocate device memory (hosts whose own allocator owns the GPU, plugins
inside them, frame loops that must not call cudaMalloc).  It works in a
fixed device array inside the library and takes the caller's buffers.

The GPU tests call it through the C ABI on device buffers the test owns and
compare it with the context path (dob_set_field + DOB_STAGE_PRESSURE_SOLVE +
dob_get_field) on two calls in a row, so the second call also shows that
what the first left in the shared array does not leak into its result.  The
file is named to be collected last, after every other test has used the
device; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2, smooth_field

STAGE_TOL = 2e-5  # same bar as the context's stage parity: FP32, relative L2


def _abi():
    from dropfluid import abi
    return abi


def _config(mode, dims):
    """Closed box: the library's default hierarchy for the grid (exact
    coarsest solve); reference mode: 4 grids with 6 coarse sweeps."""
    abi = _abi()
    if mode == "box":
        c = abi.config_closed_box(*dims)
        c.parcel_capacity = 1024
    else:
        c = abi.config_reference()
        c.nx, c.ny, c.nz = dims
        c.parcel_capacity = 1024
        c.mg_levels = 4
    return c


def _rhs(cfg, seed):
    shape = (cfg.nz, cfg.ny, cfg.nx)
    b = smooth_field(shape, seed, 1.0).astype(np.float64)
    if cfg.bc_mode == _abi().DOB_BC_CLOSED_BOX:
        b -= b.mean()  # compatible right-hand side of the pure-Neumann problem
    return b.astype(np.float32)


def _context_solve(cfg, rhs, p0):
    """The existing entry point: a context, its field I/O and its stage."""
    from dropfluid import DropFluid
    abi = _abi()
    with DropFluid(cfg) as sim:
        sim.set_field(abi.FIELD_RHS, rhs)
        sim.set_field(abi.FIELD_PRESSURE, p0)
        sim.run_stage(abi.STAGE_PRESSURE_SOLVE)
        return sim.get_field(abi.FIELD_PRESSURE)


def _noalloc_solve(lib, torch, cfg, rhs, p0):
    """The no-allocation entry point on caller-owned device buffers."""
    from dropfluid._lib import check
    d_rhs = torch.from_numpy(rhs.ravel()).to("cuda:0")
    d_p = torch.from_numpy(p0.ravel()).to("cuda:0")
    stream = torch.cuda.current_stream()
    rc = lib.dob_pressure_solve_noalloc(C.byref(cfg), C.c_void_p(d_rhs.data_ptr()), C.c_void_p(d_p.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
    check(rc, "dob_pressure_solve_noalloc")
    stream.synchronize()
    return d_p.cpu().numpy().reshape(rhs.shape)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,dims", [("box", (64, 48, 32)), ("ref", (96, 128, 96))])
def test_noalloc_matches_context_solve_twice(gpu_lib, mode, dims):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = _config(mode, dims)
    shape = (cfg.nz, cfg.ny, cfg.nx)
    # call 1: zero initial guess; call 2: new right-hand side, warm start
    cases = [(_rhs(cfg, 11), np.zeros(shape, np.float32)),
             (_rhs(cfg, 12), smooth_field(shape, 13, 0.05))]
    for rhs, p0 in cases:
        want = _context_solve(cfg, rhs, p0)
        got = _noalloc_solve(gpu_lib, torch, cfg, rhs, p0)
        assert np.isfinite(got).all()
        err = rel_l2(got, want)
        assert err < STAGE_TOL, (mode, err)
        # the solve did work: the pressure moved away from the initial guess
        assert rel_l2(got, p0) > 1e-2


@pytest.mark.gpu
def test_noalloc_smaller_grid_after_larger(gpu_lib):
    """A smaller grid after a larger one reuses the front of the array; its
    result must not depend on what the larger call left behind."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    big = _config("box", (128, 128, 64))
    small = _config("box", (32, 32, 32))
    _noalloc_solve(gpu_lib, torch, big, _rhs(big, 21), np.zeros((64, 128, 128), np.float32))
    for seed in (22, 23):
        rhs = _rhs(small, seed)
        p0 = np.zeros(rhs.shape, np.float32)
        assert rel_l2(_noalloc_solve(gpu_lib, torch, small, rhs, p0), _context_solve(small, rhs, p0)) < STAGE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("order", [((96, 128, 96), (48, 64, 48)), ((48, 64, 48), (96, 128, 96))])
def test_noalloc_same_coarsest_grid_other_spacing(gpu_lib, order):
    """48x64x48 with 3 grids and 96x128x96 with 4 both end at a 12x16x12
    coarsest grid, solved exactly with a dense inverse scaled by the level's
    h^2 (16 and 64).  Called one after the other, in either order, each call
    must use the inverse of its own hierarchy, not the one the previous call
    left in the shared array."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for k, dims in enumerate(order * 2):
        cfg = _config("box", dims)
        assert cfg.mg_coarse_sweeps == -1
        assert [d >> (cfg.mg_levels - 1) for d in dims] == [12, 16, 12]
        rhs = _rhs(cfg, 31 + k)
        p0 = np.zeros(rhs.shape, np.float32)
        err = rel_l2(_noalloc_solve(gpu_lib, torch, cfg, rhs, p0), _context_solve(cfg, rhs, p0))
        assert err < STAGE_TOL, (dims, err)


def test_noalloc_rejects_bad_sizes_before_device_use(gpu_lib):
    """Grids beyond the fixed array's 2^21 cells and malformed requests are
    refused with DOB_EINVAL before any device call (no GPU needed)."""
    abi = _abi()
    fake = C.c_void_p(4096)  # never dereferenced: every case fails validation first
    for dims, levels in [((256, 128, 128), 4), ((130, 128, 128), 2), ((6, 8, 8), 3)]:
        cfg = _config("box", dims)
        cfg.mg_levels = levels
        rc = gpu_lib.dob_pressure_solve_noalloc(C.byref(cfg), fake, fake, None)
        assert rc == abi.DOB_EINVAL, dims
    msg = gpu_lib.dob_last_error(None).decode()
    assert "dob_pressure_solve_noalloc" in msg
    cfg = _config("box", (64, 64, 64))
    cfg.precision_mode = abi.DOB_PREC_MIXED
    assert gpu_lib.dob_pressure_solve_noalloc(C.byref(cfg), fake, fake, None) == abi.DOB_EINVAL
    cfg = _config("box", (64, 64, 64))
    assert gpu_lib.dob_pressure_solve_noalloc(C.byref(cfg), None, fake, None) == abi.DOB_EINVAL
    rc = gpu_lib.dob_pressure_solve_noalloc(C.byref(cfg), C.c_void_p(4098), fake, None)
    assert rc == abi.DOB_EINVAL
