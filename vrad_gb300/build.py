"""Builds libvradgpu.so in-tree for sm_103a with nvcc (no cmake, no torch).

Kernels on the bit-exact path (trace, direct light, transfers) compile with
FMA contraction off; host C++ compiles with -ffp-contract=off so its float32
expressions (intersection records, kd-tree costs, light parameters) round
once per operation on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libvradgpu.so"
PROBE = OUT / "libvrgprobe.so"  # bench-only L2 bandwidth probe
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_EXACT = ["trace.cu", "direct.cu", "transfer.cu", "batch.cu", "relight.cu", "lightmap.cu", "coverage.cu"]
CU_FAST = ["bounce.cu", "kdbuild_gpu.cu"]
CPP = ["capi.cpp", "environment.cpp", "kdbuild.cpp", "lights.cpp", "patches.cpp", "tune.cpp", "bsp.cpp", "bsp_file.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libvradgpu.so")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _sources():
    return [CSRC / s for s in CU_EXACT + CU_FAST + CPP + ["probe.cu"]]


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "vradgpu.h"]


def up_to_date() -> bool:
    if not LIB.exists() or not PROBE.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() + _headers() + [Path(__file__)])


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    inc = ["-I", str(CSRC), "-I", str(PKG.parent / "include")]
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr", *ARCH, *inc]
    OUT.mkdir(parents=True, exist_ok=True)
    jobs = []
    for s in CU_EXACT:
        jobs.append([nvcc, *common, "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-c",
                     str(CSRC / s), "-o", str(OUT / (s + ".o"))])
    for s in CU_FAST:
        jobs.append([nvcc, *common, "-c", str(CSRC / s), "-o", str(OUT / (s + ".o"))])
    cuda_inc = str(_cuda_home(nvcc) / "include")
    for s in CPP:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-Wall", "-I", cuda_inc, *inc, "-c", str(CSRC / s), "-o",
                     str(OUT / (s + ".o"))])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    tmp = OUT / f"libvradgpu.{os.getpid()}.so"
    objs = [str(OUT / (s + ".o")) for s in CU_EXACT + CU_FAST + CPP]
    run([nvcc, "-shared", *ARCH, "-o", str(tmp), *objs, "-lpthread"])
    os.replace(tmp, LIB)
    ptmp = OUT / f"libvrgprobe.{os.getpid()}.so"
    run([nvcc, *common, "-shared", str(CSRC / "probe.cu"), "-o", str(ptmp)])
    os.replace(ptmp, PROBE)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
