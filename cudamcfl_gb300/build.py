"""Builds libmcfl.so and the mcfl_run command for sm_103a, in-tree.

    python -m cudamcfl_gb300.build        (or cudamcfl_gb300.build.build())

CUDA translation units are compiled by nvcc for compute_103a/sm_103a only;
host translation units by g++.  Floating-point contraction is disabled
wherever a result must be reproducible bit for bit (the exact-math transport
kernel, the FP64 helper kernels, host code that derives weights).  Objects are
rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libmcfl.so")
CLI = os.path.join(OUT, "mcfl_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE]
EXACT = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
FAST = ["--use_fast_math"]

CUDA_UNITS = {
    "transport_exact.cu": EXACT,
    "transport_fast.cu": FAST,
    "transport_f64.cu": [],
    "engine_kernels.cu": EXACT,
    "noalloc.cu": EXACT,
}
HOST_UNITS = ["engine.cpp", "run.cpp", "mci.cpp", "safeprimes.cpp", "server.cpp", "tune.cpp"]
HEADERS = ["engine_types.h", "portable_math.h", "mcfl_internal.h", "transport.cuh"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles what is out of date and returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    hdr = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mcfl.h")]
    steps = []
    objs = []
    for src, flags in CUDA_UNITS.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdr):
            steps.append(["nvcc", *ARCH, *NVCC_COMMON, *flags, "-c", s, "-o", o])
    for src in HOST_UNITS:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdr):
            steps.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                          "-I" + CSRC, "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        for f in [ex.submit(_run, c) for c in steps]:
            f.result()
    if steps or not os.path.exists(LIB):
        _run(["nvcc", *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", LIB, *objs, "-lpthread"])
    cli_src = os.path.join(CSRC, "mcfl_run_main.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB, os.path.join(INCLUDE, "mcfl.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + OUT, "-lmcfl",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
