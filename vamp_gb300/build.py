"""Build libvamp_gb300.so for sm_103a (in tree, under vamp_gb300/_lib).

Each robot's kernels live in their own translation unit so that they compile in parallel.
Usage: python -m vamp_gb300.build [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
BUILD = PKG / "_build"
LIB = OUT / "libvamp_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    # explicit __fmaf_rn/__fmul_rn/__fadd_rn everywhere that rounding matters; forbid any other
    # contraction so the kernels round exactly like the CPU oracle
    "-fmad=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-O2",
]

# ptxas optimisation level for the translation units where it was measured to matter.  The
# Panda's same-edge edge kernel is bound by instruction fetch; built with ptxas -O1 it checked the
# 65,536-edge workload in 2.665 ms against 2.748 ms at the default -O3 (two builds each, same box).
# The other robots' kernels were as fast or faster at -O3, so they keep it.
PTXAS_LEVEL = {"robot_panda.cu": 1}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _defines() -> list[str]:
    # VG_MIN_BLOCKS: resident 128-thread blocks per SM the kernels are compiled for.
    # VG_FORM_COMPACT=1: pass frames to the fine checks in registers instead of staging them in
    # shared memory; VG_SELF_UNROLLED=1: one block of code per self-collision link pair instead
    # of a loop over a table; VG_STAGED_ALL=1: the staged form for the robots whose default is the
    # table-driven form (all schedule forms give identical results).
    out = []
    mb = os.environ.get("VG_MIN_BLOCKS")
    if mb:
        out.append(f"-DVG_MIN_BLOCKS={int(mb)}")
    if os.environ.get("VG_FORM_COMPACT") == "1":
        out.append("-DVG_FORM_COMPACT")
    if os.environ.get("VG_SELF_UNROLLED") == "1":
        out.append("-DVG_SELF_UNROLLED")
    if os.environ.get("VG_STAGED_ALL") == "1":
        out.append("-DVG_STAGED_ALL")
    # VG_CAPT_SHARED_WEIGHT=w: the pointcloud query scans one lane's list with the whole warp
    # when 4 x the longest list exceeds w x the warp's shared steps
    # VG_DEFAULT_LOOPED_ENV=1: the default edge kernel runs the environment section as loops
    if os.environ.get("VG_DEFAULT_LOOPED_ENV") == "1":
        out.append("-DVG_DEFAULT_LOOPED_ENV=1")
    w = os.environ.get("VG_CAPT_SHARED_WEIGHT")
    if w:
        out.append(f"-DVG_CAPT_SHARED_WEIGHT={int(w)}")
    return out


def _compile(src: Path, verbose: bool) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    level = ["-Xptxas", f"-O{PTXAS_LEVEL[src.name]}"] if src.name in PTXAS_LEVEL else []
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *level, *_defines(), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, *CSRC.glob("*.cuh"), *CSRC.glob("*.h"), *CSRC.glob("*.inc"), *(CSRC / "robots").glob("*.cuh"),
            PKG.parent / "include" / "vamp_gb300.h", Path(__file__)]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    stamp = BUILD / "defines.txt"
    defs = " ".join(_defines())
    if not stamp.exists() or stamp.read_text() != defs:
        force = True
        stamp.write_text(defs)
    todo = [s for s in srcs if force or _stale(BUILD / (s.stem + ".o"), s)]
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for obj, log in ex.map(lambda s: _compile(s, verbose), todo):
                logs[obj.name] = log
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    if todo or not LIB.exists():
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        for k, v in logs.items():
            print(f"== {k}\n{v}", file=sys.stderr)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.verbose, a.force))


if __name__ == "__main__":
    main()
