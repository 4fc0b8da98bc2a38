"""Build the CUDA library (brams_gb300/_lib/libgb_rrtmg_lw.so) with nvcc for sm_103a.

Translation units are compiled in parallel and linked into one shared
library exporting the C ABI of include/gb_rrtmg_lw.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libgb_rrtmg_lw.so")
UNITS = ["lw_solver.cu", "lw_mcica.cu", "lw_capi.cu", "lw_tables.cpp", "lw_mlp.cu", "lw_mlp_capi.cu", "lw_mlp_tc.cu",
         "lw_cldprop.cu", "lw_pack.cu", "lw_ozone.cpp", "lw_shard.cpp",
         "sw_solver.cu", "sw_solver_f32.cu", "sw_capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The column kernel is compiled without multiply-add contraction: every fused
# multiply-add in it is an explicit fmaf, so that its results are fixed by the
# source and every launch shape and kernel flavour (full, learned-only,
# hand-over list) gives the same bits for a column.  cldprop likewise, so
# that its fp64 results follow the reference's operations one by one.
UNIT_FLAGS = {"lw_solver.cu": ["-fmad=false"], "sw_solver.cu": ["-fmad=false"], "lw_cldprop.cu": ["-fmad=false"], "lw_pack.cu": ["-fmad=false"],
              "lw_ozone.cpp": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "gb_rrtmg_lw.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
    objs = []

    def comp(u):
        obj = os.path.join(OUT, u.rsplit(".", 1)[0] + ".o")
        cmd = [cc] + common + UNIT_FLAGS.get(u, []) + ["-c", os.path.join(SRC, u), "-o", obj]
        if u.endswith(".cpp"):
            cmd = [cc] + common + UNIT_FLAGS.get(u, []) + ["-x", "cu", "-c", os.path.join(SRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(comp, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
