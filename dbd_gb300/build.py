"""Build recipe of libdbd and its CLI binaries (nvcc, sm_103a only).

Compiles every translation unit of dbd_gb300/csrc in parallel into
dbd_gb300/_build/, links dbd_gb300/_lib/libdbd.so, then links bin/SSpMM,
bin/compute, bin/d2h and bin/debug against it.  Objects are rebuilt only when
a source or header is newer than the object.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libdbd.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["k_analysis.cu", "k_spgemm.cu", "k_adjoint.cu", "k_batch.cu", "k_digest.cu", "k_mtx.cu", "noalloc.cu"]
CPP_SOURCES = ["engine.cpp", "csr_io.cpp", "writer.cpp"]
CLI = {"SSpMM": ["-DDBD_CLI_SCOPE=2"], "compute": ["-DDBD_CLI_SCOPE=0"],
       "d2h": ["-DDBD_CLI_SCOPE=1"], "debug": ["-DDBD_CLI_SCOPE=2", "-DDBD_CLI_DEBUG"]}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))) if os.path.exists(_nvcc()) else "/usr/local/cuda"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "dbd.h"))
    return hs


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, src):
        return obj
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + inc + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + inc + ["-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    cli = os.path.join(CSRC, "cli.cpp")
    for name, defs in CLI.items():
        out = os.path.join(BINDIR, name)
        if os.path.exists(out) and os.path.getmtime(out) > max(os.path.getmtime(cli), os.path.getmtime(LIB)):
            continue
        cmd = ["g++"] + CXX_FLAGS + defs + ["-I", os.path.join(ROOT, "include"), cli, "-o", out,
                                           "-L", LIBDIR, "-ldbd", "-Wl,-rpath,$ORIGIN/../_lib"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
