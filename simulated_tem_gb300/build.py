"""Build libstem.so, libstem_nn.so (the corrector) and the peak microbenchmark library in-tree
for sm_103a.

nvcc cross-compiles the CUDA sources for sm_103a on any host; the host-side
C++ is compiled by g++ for the machine it runs on.  Objects go to
``simulated_tem_gb300/_build/``; the libraries land beside this file.
Every host translation unit is compiled with -ffp-contract=off so the double
arithmetic that restates the reference is never fused into multiply-adds.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstem.so")
PEAKS_LIB = os.path.join(HERE, "libstem_peaks.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]

LIB_SOURCES = ["stem_ctx.cu", "k_bin.cu", "k_column.cu", "k_column_ring.cu", "k_column_f64ring.cu", "k_column_v3_np1.cu",
               "k_column_v3_np2.cu", "k_column_v3_np4.cu", "k_column_v3_np8.cu", "k_column_v3_np16.cu", "k_blur.cu", "blur_noalloc.cu", "k_output.cu",
               "k_parse.cu", "k_geom.cu", "k_tilt.cu", "host_d2bi.cpp", "host_tilt.cpp", "host_output.cpp",
               "host_input.cpp"]
NN_LIB = os.path.join(HERE, "libstem_nn.so")
NN_SOURCES = ["nn_conv.cu", "nn_ops.cu", "nn_api.cu"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libstem")


def _cuda_root(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, ptxas_info=False):
    """Compile every source (in parallel) and link the libraries; returns their paths."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    inc = os.path.join(HERE, "..", "include")
    libs = [
        (LIB, LIB_SOURCES, [os.path.join(CSRC, "internal.h"), os.path.join(CSRC, "parse_number.cuh"),
                            os.path.join(CSRC, "k_column_v3.cuh"), os.path.join(CSRC, "fp64_column.cuh"),
                            os.path.join(CSRC, "host_geom.h"),
                            os.path.join(inc, "stem.h"),
                            os.path.join(inc, "stem_host.h")]),
        (NN_LIB, NN_SOURCES, [os.path.join(CSRC, "nn.h"), os.path.join(CSRC, "tc_sm100.cuh"), os.path.join(CSRC, "nn_conv_strip.cuh"),
                              os.path.join(inc, "stem_nn.h")]),
    ]
    jobs, link = [], []
    for lib, sources, headers in libs:
        objs = []
        for src in sources:
            path = os.path.join(CSRC, src)
            obj = os.path.join(BUILD, src + ".o")
            objs.append(obj)
            if not _stale(obj, [path] + headers):
                continue
            if src.endswith(".cu"):
                cmd = [nvcc] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", path, "-o", obj]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-I", os.path.join(_cuda_root(nvcc), "include"), "-c", path, "-o", obj]
            jobs.append(cmd)
        link.append((lib, objs))
    outputs = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            outputs.append(out)
    for lib, objs in link:
        if _stale(lib, objs):
            outputs.append(_run([nvcc] + ARCH + ["-shared", "-o", lib] + objs))
    peaks_src = os.path.join(CSRC, "peaks.cu")
    if _stale(PEAKS_LIB, [peaks_src]):
        outputs.append(_run([nvcc] + NVCC_FLAGS + ["-shared", peaks_src, "-o", PEAKS_LIB]))
    if verbose:
        for o in outputs:
            if o.strip():
                print(o)
    return LIB, PEAKS_LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB, NN_LIB, PEAKS_LIB)
