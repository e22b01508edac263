"""Build recipe of the native parts of stencil3d_gb300.

Compiles the CUDA sources under ``csrc/`` for sm_103a (GB300) into
``_build/libst3d.so`` and the hstencil3d-compatible command line driver
``_build/gstencil3d`` (host C++ over the C ABI; ``_build/gstencil3d_f64`` is
the same driver built with USE_DOUBLE, the reference's double build).  Translation units compile in
parallel; nothing here needs a GPU.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libst3d.so")
CLI = os.path.join(OUT, "gstencil3d")
CLI_F64 = os.path.join(OUT, "gstencil3d_f64")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I", os.path.join(REPO, "include"), "-I", CSRC]

CU_SOURCES = ["st3d_api.cu", "st3d_kernels_simple.cu", "st3d_kernels_tma.cu",
              "st3d_kernels_tma16.cu", "st3d_kernels_delta16.cu", "st3d_kernels_mma16.cu",
              "st3d_kernels_tb.cu",
              "st3d_kernels_aux.cu", "st3d_kernels_copy.cu", "st3d_noalloc.cu", "st3d_batch.cu",
              "st3d_stream.cu"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("command failed: " + " ".join(cmd))
    if verbose and (r.stdout or r.stderr):
        sys.stdout.write(r.stdout + r.stderr)
    return r


def build(verbose=False, force=False, ptxas_info=False):
    """Compile libst3d.so and gstencil3d; returns the library path."""
    if not os.path.exists(NVCC) and shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found (CUDA_HOME=%s)" % CUDA_HOME)
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(lambda c: _run(c, verbose or ptxas_info), jobs):
            pass
    if force or jobs or _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"], verbose)
    host_src = [os.path.join(HOST, f) for f in ("gstencil3d.cpp", "st3d_compat.cpp")]
    if all(os.path.exists(p) for p in host_src):
        host_hdr = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".h", ".hpp"))]
        for exe, defs in ((CLI, []), (CLI_F64, ["-DUSE_DOUBLE"])):
            if force or _newer(exe, host_src + host_hdr + hdrs + [LIB]):
                _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp"] + defs +
                     ["-I", os.path.join(REPO, "include"), "-I", HOST, "-o", exe] + host_src +
                     ["-L", OUT, "-lst3d", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
