"""Builds libgls_cuda.so in-tree for sm_103a (GB300).

    python -m climage_gb300.build            # or __graft_entry__.build()

Translation units compile in parallel with nvcc; the kernels are built with
--fmad=false -prec-div=true -prec-sqrt=true -ftz=false so that every float operation is
an individually rounded IEEE operation (the convention gls_clmath.h documents).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgls_cuda.so")

SOURCES = ["gls_api.cu", "k_stages.cu", "k_nlf.cu", "k_fused.cu", "k_fused_final.cu", "raw_converter.cu", "k_noalloc.cu", "k_cnn.cu", "k_awb.cu", "k_lj92.cu", "k_calib.cu", "k_tune.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo",
    "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
    "-Xptxas", "-warn-spills",
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".cu"))]
    deps.append(os.path.join(HERE, "..", "include", "gls_cuda.h"))
    if _newer(obj, deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    if not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


def build_cpp_test():
    """Compiles tests/cpp/test_cpp_layer.cpp (a C++ client of include/gls_cuda.hpp)."""
    lib = build()
    src = os.path.join(HERE, "..", "tests", "cpp", "test_cpp_layer.cpp")
    exe = os.path.join(BUILD, "test_cpp_layer")
    hdrs = [os.path.join(HERE, "..", "include", f) for f in ("gls_cuda.h", "gls_cuda.hpp")]
    if _newer(exe, [src, lib] + hdrs):
        return exe
    cmd = [nvcc(), "-std=c++20", "-O2", "-x", "cu", src, "-o", exe, "-L" + HERE, "-lgls_cuda",
           "-Xlinker", "-rpath=" + HERE] + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("C++ layer test build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return exe


if __name__ == "__main__":
    print(build(verbose=True))
