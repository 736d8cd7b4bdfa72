"""Builds libstocha_gpu.so in-tree (stocha_gb300/libstocha_gpu.so).

Kernels: nvcc for sm_103a only.  Host C-ABI: g++ with -ffp-contract=off (the
host prepares the constants every kernel starts from with the reference's
FP64 expression order; an FMA contraction would change their last bits).
The FP64 kernel translation units use --fmad=false for the same reason.
Translation units compile in parallel; unchanged ones are skipped.

Usage: python -m stocha_gb300.build [--force] [--verbose-ptxas]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstocha_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags
CUDA_UNITS = {
    "paths_f64.cu": ["--fmad=false"],
    "paths_f32.cu": [],
    "rng.cu": ["--fmad=false"],
    "lsmc.cu": [],
    "exotics.cu": ["--fmad=false"],
    "risk.cu": [],
    "copula_t.cu": ["--fmad=false"],
    "greeks.cu": [],
    "batch.cu": [],
    "peaks.cu": [],
    "noalloc.cu": [],
}
HOST_UNITS = ["api.cpp", "rng_host.cpp", "lsmc_host.cpp", "greeks_host.cpp", "batch_host.cpp", "serve.cpp",
              "hostcopy.cpp", "exotics_host.cpp", "risk_host.cpp"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    jobs = []
    objs = []
    for unit, extra in CUDA_UNITS.items():
        src = os.path.join(CSRC, unit)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if force or verbose_ptxas or _newer(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
                   "-ffp-contract=off", *extra, "-c", src, "-o", obj]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for unit in HOST_UNITS:
        src = os.path.join(CSRC, unit)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
                         "-Wall", "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, p in ex.map(run, jobs):
            out = (p.stdout + p.stderr).strip()
            if p.returncode != 0:
                failed.append((cmd, out))
            elif out and (verbose_ptxas or not quiet):
                print(out, file=sys.stderr)
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("stocha_gb300 build failed:\n" + msg)
    if force or jobs or _newer(LIB, objs):
        link = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lpthread"]
        p = subprocess.run(link, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("stocha_gb300 link failed:\n" + p.stdout + p.stderr)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="--verbose-ptxas" in sys.argv, quiet=False)
    print(LIB)
