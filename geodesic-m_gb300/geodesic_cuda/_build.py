"""Builds the native parts of the CUDA backend in-tree.

* `_build/libgeodesic_cuda.so` — the CUDA kernels and the C-ABI (nvcc,
  sm_103a only, -lineinfo);
* `_build/libgmsynth.so` — the synthetic-system generator (gcc).

Translation units compile in parallel; nothing is rebuilt when outputs are
newer than every source and header.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(PKG, "_build")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
CUDA_LIB = os.path.join(OUT, "libgeodesic_cuda.so")
SYNTH_LIB = os.path.join(OUT, "libgmsynth.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build_synth(force=False):
    src = os.path.join(PKG, "synth", "gmsynth.c")
    if force or _stale(SYNTH_LIB, [src]):
        os.makedirs(OUT, exist_ok=True)
        tmp = SYNTH_LIB + f".tmp{os.getpid()}"
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-Wall", "-pthread", "-o", tmp, src, "-lm"])
        os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


def build_cuda(force=False, verbose=False):
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                     glob.glob(os.path.join(INCLUDE, "*.h")))
    if not sources:
        return None
    if not (force or _stale(CUDA_LIB, sources + headers)):
        return CUDA_LIB
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-lineinfo"]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if not force and not _stale(obj, [src] + headers):
            return obj, ""
        cmd = [NVCC, *ARCH, *common, "-c", src, "-o", obj]
        if verbose:
            cmd[1:1] = ["-Xptxas", "-v"]
        if src.endswith("_exact.cu"):
            # FP64 integrator/constraint arithmetic rounds like the reference:
            # no fused multiply-add anywhere in that translation unit
            cmd[1:1] = ["--fmad=false"]
        log = _run(cmd)
        return obj, log

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, sources))
    objs = [o for o, _ in results]
    tmp = CUDA_LIB + f".tmp{os.getpid()}"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, CUDA_LIB)
    if verbose:
        for _, log in results:
            if log:
                print(log)
    return CUDA_LIB


def build_all(force=False):
    return build_synth(force), build_cuda(force)


if __name__ == "__main__":
    import sys
    print(build_synth("-f" in sys.argv), build_cuda("-f" in sys.argv, "-v" in sys.argv))
