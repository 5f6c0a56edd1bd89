"""In-tree build of libmavi_cuda.so for sm_103a (GB300).

The translation units (host runtime + C ABI, FP64 passes, mixed passes, the
mixed multi-lane passes, the FMA peak probe, the allocation-free chunk lists,
invasion detection) compile
in parallel, then link into ``lib/libmavi_cuda.so``. No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = PKG / "_build"
SOURCES = ["mavi_api.cu", "mavi_steps_fp64.cu", "mavi_steps_mixed.cu", "mavi_steps_lanes.cu", "mavi_steps_split.cu", "mavi_steps_cols.cu", "mavi_peak.cu",
           "mavi_noalloc.cu", "mavi_invasions.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and pathlib.Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> pathlib.Path:
    out = OBJ / (pathlib.Path(src).stem + ".o")
    extra = os.environ.get("MAVI_NVCC_FLAGS", "").split()   # tuning defines, e.g. -DMAVI_PASS_BLOCKS_MIXED=6
    cmd = [nvcc(), *FLAGS, *extra, *ARCH, "-c", str(CSRC / src), "-o", str(out)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
    if verbose:
        (OBJ / (pathlib.Path(src).stem + ".ptxas.txt")).write_text(r.stderr)
    return out


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    """Compile libmavi_cuda.so; returns its path. Skips the build when the
    library is newer than every source file unless ``force``."""
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    target = LIB / "libmavi_cuda.so"
    inputs = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "mavi_cuda.h"]
    if (not force and target.exists()
            and target.stat().st_mtime > max(p.stat().st_mtime for p in inputs)):
        return target
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = target.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, target)
    return target


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
