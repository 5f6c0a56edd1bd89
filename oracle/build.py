"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle/mavi_oracle.c into oracle/_build/libmavi_oracle.so with -O3,
-ffp-contract=off (no fused multiply-add, like Julia without @fastmath) and
OpenMP (the Threaded force mode and the CPU baseline). No -march=native and no
-ffast-math: the same source must give the same FP64 results on every host
it is built on (x86-64 here, Arm on the GPU machines). The reference itself is
Julia and cannot be compiled here, so there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libmavi_oracle.so"
SRC = [HERE / "mavi_oracle.c"]
DEPS = SRC + [HERE / "mavi_oracle.h", HERE.parent / "include" / "mavi_cuda.h"]


def build(force: bool = False) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime > max(p.stat().st_mtime for p in DEPS):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), *map(str, SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
