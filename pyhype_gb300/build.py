"""Build libeuler2d.so in-tree for sm_103a with nvcc (no torch extension machinery).

Translation units compile in parallel; the FP64 parity kernels build with
``-fmad=false`` so no multiply-add is contracted.  Run ``python -m pyhype_gb300.build``
or call :func:`build`.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libeuler2d.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", os.path.join(HERE, "..", "include")]
# object name -> (source, extra flags).  The reconstruction launchers of each
# (arithmetic type, limiter) pair are one object each (e2d_recon_unit.cu), so the
# largest kernels compile in parallel.
UNITS = {
    "e2d_fp64": ("e2d_fp64.cu", ["-fmad=false"]),
    # the FP32 form's multiply-adds are explicit (fmaT in e2d_device.cuh): contraction off
    # everywhere, so every kernel form evaluates the same operations
    "e2d_fp32": ("e2d_fp32.cu", ["-fmad=false"]),
    "e2d_api": ("e2d_api.cu", ["-fmad=false"]),
    "e2d_bench": ("e2d_bench.cu", []),
    "e2d_noalloc": ("e2d_noalloc.cu", ["-fmad=false"]),
    "e2d_adjoint": ("e2d_adjoint.cu", ["-fmad=false"]),
}
for _lim in range(4):
    UNITS[f"e2d_recon_f64_l{_lim}"] = ("e2d_recon_unit.cu", ["-fmad=false", "-DE2D_T=double", f"-DE2D_LIM={_lim}"])
    UNITS[f"e2d_recon_f32_l{_lim}"] = ("e2d_recon_unit.cu", ["-fmad=false", "-DE2D_T=float", f"-DE2D_LIM={_lim}"])


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libeuler2d.so")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "euler2d.h"), __file__]
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()

    def compile_unit(name):
        obj = os.path.join(OBJ, name + ".o")
        src, flags = UNITS[name]
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
