"""Build libgpmood.so (CUDA kernels for sm_103a + the C ABI) in-tree.

Every CUDA source is compiled with ``-gencode arch=compute_103a,code=sm_103a``;
stage_kernels.cu is compiled twice: once with ``--fmad=false`` (namespace
gpm_exact, the reference's rounding) and once with FMA contraction (gpm_fast).
Objects go to ``_build/`` next to this file; the library lands next to it too.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libgpmood.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgpmood")


def _jobs() -> list[tuple[list[str], Path]]:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(CSRC),
                     "-I", str(INCLUDE), "--expt-relaxed-constexpr"]
    jobs = []
    for name, flags in (("stage_exact", ["-DGPM_EXACT=1", "--fmad=false"]),
                        ("stage_fast", ["-DGPM_EXACT=0", "--fmad=true"])):
        obj = BUILD / f"{name}.o"
        jobs.append(([nvcc, *common, *flags, "-c", str(CSRC / "stage_kernels.cu"), "-o", str(obj)], obj))
    for src in ("nn_gate.cu", "nn_ref.cu", "probe.cu", "noalloc.cu", "adjoint.cu"):
        obj = BUILD / (Path(src).stem + ".o")
        jobs.append(([nvcc, *common, "-c", str(CSRC / src), "-o", str(obj)], obj))
    gxx = shutil.which("g++") or "g++"
    for src in ("gp_weights.cpp", "gpmood_capi.cpp", "batch_capi.cpp"):
        obj = BUILD / (Path(src).stem + ".o")
        jobs.append(([gxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(cuda / "include"),
                      "-I", str(CSRC), "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)], obj))
    return jobs


def build(verbose: bool = False) -> Path:
    """Compile every translation unit in parallel and link libgpmood.so."""
    BUILD.mkdir(exist_ok=True)
    jobs = _jobs()

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(run, [cmd for cmd, _ in jobs]))
    cuda = _cuda_home()
    tmp = LIB.with_suffix(".so.tmp")
    link = [str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs],
            "-cudart", "static", "-lm"]
    run(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
