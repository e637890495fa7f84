"""In-tree build of libdropfluid.so for sm_103a (nvcc only, no cmake).

Each kernel family is one translation unit, compiled in parallel; the
parcel/injection unit (k_exact.cu), the wave solver (k_wave.cu) and the
light volume (k_light.cu) are compiled without multiply-add contraction so their arithmetic can be
reproduced bit for bit on the host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libdropfluid.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-Xptxas", "-O3"]
UNITS = {
    "dob_api.cu": [],
    "k_fluid.cu": [],
    "k_box.cu": [],
    "k_mg.cu": [],
    "k_exact.cu": ["-fmad=false"],
    "k_wave.cu": ["-fmad=false"],
    "k_light.cu": ["-fmad=false"],
    "k_render.cu": ["-fmad=false"],
    "dob_noalloc.cu": [],
    "dob_tape.cu": [],
    "k_adjoint.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(os.path.dirname(ROOT), "include", "dropfluid.h")]


def _stale(out: str, inputs) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs)


def build(verbose: bool = False, force: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    cc = nvcc()
    objs = []

    def compile_one(name):
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, list(UNITS)))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
