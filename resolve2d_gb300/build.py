"""Build recipe for the in-tree CUDA library (and, for the test harness, the
CPU oracle).  Compiles for sm_103a only, with the floating-point flags the
bit-exact parity depends on:

* ``--fmad=false`` / ``-ffp-contract=off``: no fused multiply-add, so every
  f32 operation rounds exactly as the reference's (Zig's default float mode
  is strict);
* IEEE division and square root (nvcc's defaults; no ``--use_fast_math``).
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libr2d_gb300.so"
INCLUDE = REPO / "include"

SOURCES = ["r2d_world_kernel.cu", "r2d_large.cu", "r2d_capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libr2d_gb300.so")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


TIMERS_LIB = BUILD / "libr2d_timers.so"


def build_library(force: bool = False, verbose: bool = False, timers: bool = False,
                  defines: dict | None = None, name: str | None = None) -> Path:
    """Compile the translation units in parallel and link libr2d_gb300.so.
    timers=True builds libr2d_timers.so instead: the same library with the
    fused kernel's per-phase cycle counters (R2D_PHASE_TIMERS), for
    resolve2d_gb300.phase_timers.  `defines` (e.g. {"R2D_REG_TARGET": 80})
    with `name` builds a tuning variant as lib<name>.so beside it."""
    BUILD.mkdir(exist_ok=True)
    deps = _deps()
    lib = TIMERS_LIB if timers else LIB
    tag = "_timers" if timers else ""
    if name:
        lib = BUILD / f"lib{name}.so"
        tag = "_" + name
    if not force and not _stale(lib, deps):
        return lib
    cc = nvcc()
    procs = []
    objs = []
    extra = ["-DR2D_PHASE_TIMERS"] if timers else []
    extra += [f"-D{k}={v}" for k, v in (defines or {}).items()]
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + tag + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{out}")
    tmp = BUILD / (lib.name + ".tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for o in objs], "-lcudart"]
    out = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"link failed ({' '.join(cmd)}):\n{out.stdout}")
    os.replace(tmp, lib)
    return lib


def build_oracle(force: bool = False) -> Path:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    odir = REPO / "oracle"
    args = ["make", "-s", "-C", str(odir)]
    if force:
        args.insert(1, "-B")
    out = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}")
    return odir / "_build" / "libr2d_oracle.so"


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_oracle())
