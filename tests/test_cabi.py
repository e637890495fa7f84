"""The C-ABI library as a CPU-only artefact: it loads, exports every entry
point include/dropfluid.h declares, its structs have the header's layout,
and argument validation happens before any device call."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dropfluid.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dob_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib(gpu_lib):
    return gpu_lib


def test_exports_every_declared_symbol(lib):
    from dropfluid import _lib
    fns = header_functions()
    assert len(fns) >= 20
    for name in fns:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name
    assert set(_lib.SIGNATURES) <= set(fns)


def test_struct_layout_matches_header():
    from dropfluid import abi
    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "dropfluid.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(dob_config), sizeof(dob_step_stats),
         offsetof(dob_config, mg_rel_tol), offsetof(dob_config, dye_sharpness),
         offsetof(dob_step_stats, stage_ms), offsetof(dob_config, mg_div_tol),
         offsetof(dob_config, mg_cycles_injected));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sz_cfg, sz_st, off_tol, off_sharp, off_ms, off_div, off_inj = map(int, out)
    assert C.sizeof(abi.DobConfig) == sz_cfg
    assert C.sizeof(abi.DobStepStats) == sz_st
    assert abi.DobConfig.mg_rel_tol.offset == off_tol
    assert abi.DobConfig.dye_sharpness.offset == off_sharp
    assert abi.DobStepStats.stage_ms.offset == off_ms
    assert abi.DobConfig.mg_div_tol.offset == off_div
    assert abi.DobConfig.mg_cycles_injected.offset == off_inj


def test_config_builders_match_python(lib):
    from dropfluid import abi
    c = abi.DobConfig()
    assert lib.dob_config_reference(C.byref(c)) == 0
    assert c.as_dict() == abi.config_reference().as_dict()
    for dims in ((48, 64, 48), (192, 256, 192)):
        c = abi.DobConfig()
        assert lib.dob_config_closed_box(C.byref(c), *dims) == 0
        assert c.as_dict() == abi.config_closed_box(*dims).as_dict()


@pytest.mark.parametrize("mutate", [
    lambda c: setattr(c, "struct_size", 4),
    lambda c: setattr(c, "nx", 30),
    lambda c: setattr(c, "mg_levels", 0),
    lambda c: setattr(c, "mg_levels", 6),  # 32 / 2^5 = 1: odd coarse grid
    lambda c: setattr(c, "dye_refine", 3),
    lambda c: setattr(c, "bc_mode", 7),
    lambda c: setattr(c, "dt", float("nan")),
    lambda c: setattr(c, "parcel_capacity", 0),
])
def test_invalid_config_is_rejected_before_device_use(lib, mutate):
    from dropfluid import abi
    c = abi.config_closed_box(32, 32, 32)
    mutate(c)
    h = C.c_void_p()
    assert lib.dob_create(C.byref(c), C.byref(h)) == abi.DOB_EINVAL
    assert not h.value
    assert lib.dob_last_error(None)


def test_null_arguments(lib):
    from dropfluid import abi
    assert lib.dob_create(None, None) == abi.DOB_EINVAL
    assert lib.dob_reset(None) == abi.DOB_EINVAL
    assert lib.dob_step(None, 1, 0, None) == abi.DOB_EINVAL
    assert lib.dob_set_step_stats(None, abi.STATS_ALL) == abi.DOB_EINVAL
    lib.dob_destroy(None)
    assert lib.dob_abi_version() == abi.DOB_ABI_VERSION
