"""Builds libimpulse_gpu.so in-tree: one nvcc job per translation unit, in parallel.

Usage: python -m impulse_gb300.build   (or impulse_gb300.build.build() from Python)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libimpulse_gpu.so")
UNITS = ["ig_engine.cu", "ig_inst_f32.cu", "ig_inst_df.cu", "ig_inst_f64.cu", "ig_inst_f32_e8.cu",
         "ig_inst_f32_e16.cu", "ig_inst_df_e8.cu", "ig_inst_df_e16.cu", "ig_inst_f64_e8.cu", "ig_inst_f64_e16.cu",
         "ig_inst_f32_e16db.cu", "ig_inst_df_e16db.cu", "ig_inst_f64_e16db.cu",
         "ig_line_f32_e8.cu", "ig_line_f32_e16.cu", "ig_line_f32_e16db.cu", "ig_line_df_e8.cu", "ig_line_df_e16.cu",
         "ig_line_df_e16db.cu", "ig_pair_f32.cu", "ig_copy.cu", "ig_wide_df.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "impulse_gpu.h"))
    objs, jobs = [], []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB):
        # -z defs: an unresolved symbol is a link error, not a load-time failure
        cmd = [nvcc, *ARCH, "-shared", "-Xlinker", "-z,defs", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
