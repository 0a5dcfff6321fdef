"""Build librfgpu.so (the C-ABI CUDA library) in-tree for sm_103a.

nvcc only, no cmake: each .cu compiles to an object in parallel, then one
link.  --fmad=false plus explicit __f*_rn intrinsics keep every f32
operation singly rounded, as the reference (Rust) computes them.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librfgpu.so")
SRCS = ["rf_kernels.cu", "rf_sort.cu", "rf_api.cu", "rf_noalloc.cu", "rf_server.cu", "rf_obj.cu", "rf_lines.cu", "rf_raster_tw8.cu", "rf_raster_tw16.cu",
        "rf_raster_tw32.cu", "rf_raster_tw64.cu"]
HDRS = ["rf_exact.cuh", "rf_internal.cuh", "rf_kernels.cuh", "rf_device.cuh", "rf_raster.cuh",
        "rf_ctx_internal.h"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
         "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I" + os.path.join(HERE, "..", "include")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    mt = os.path.getmtime(out)
    return any(os.path.getmtime(d) > mt for d in deps)


def build(force=False, verbose=False):
    """Compile retrofire_gb300/_build/librfgpu.so if stale; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HDRS] + [
        os.path.join(HERE, "..", "include", "rfgpu.h"), __file__]
    objs, jobs = [], []
    for src in SRCS:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [sp] + hdrs):
            jobs.append([NVCC] + FLAGS + ["-c", sp, "-o", obj] + (["-Xptxas", "-v"] if verbose else []))
    with ThreadPoolExecutor(max_workers=len(SRCS)) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(r.args))
            if verbose:
                sys.stderr.write(r.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
                               "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
