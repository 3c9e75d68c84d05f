"""Builds the reference's own CPU code into oracle/_ref/libdbdref.so.

TEST INFRASTRUCTURE ONLY.  The reference's host sources ship inside
DBD_FULL.zip (dbd/src/*); this recipe extracts the host files of the path
(SSpMM.hpp, main.cpp, distributeWorkload.cpp, computeCPU.cpp, readInput.cpp) into a temporary directory
outside the repository, compiles them with the flags of the reference's own
Makefile (ZIP:dbd/Makefile:7-9: g++ -O3 -std=c++14 -fopenmp, plus -DCOMPUTE
as its `compute` target) together with oracle/ref_harness.cpp, and writes only
the shared library into oracle/_ref/.  No reference source is copied into the
repository.  When the reference tree is absent (as on a machine that only
receives the repository), it does nothing.
"""
import os
import subprocess
import sys
import tempfile
import zipfile

HERE = os.path.dirname(os.path.abspath(__file__))


DEFAULT_REFERENCE_DIR = "/root/reference"


def reference_root():
    """The reference checkout: $DBD_REFERENCE_DIR, else the read-only checkout
    this recipe was written against; None when that directory does not
    exist (machines without the reference use the committed fixtures)."""
    root = os.environ.get("DBD_REFERENCE_DIR") or DEFAULT_REFERENCE_DIR
    return root if os.path.isdir(root) else None


def _ref_zip():
    root = reference_root()
    return os.path.join(root, "DBD_FULL.zip") if root else None


MEMBERS = ["dbd/src/SSpMM.hpp", "dbd/src/main.cpp", "dbd/src/distributeWorkload.cpp",
           "dbd/src/computeCPU.cpp", "dbd/src/readInput.cpp"]
OUT = os.path.join(HERE, "_ref", "libdbdref.so")


def build(verbose=False):
    ref_zip = _ref_zip()
    if not ref_zip or not os.path.exists(ref_zip):
        if verbose:
            print("build_ref: reference tree absent; oracle/_ref not built")
        return None
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with tempfile.TemporaryDirectory(prefix="dbdref_") as tmp:
        with zipfile.ZipFile(ref_zip) as z:
            for m in MEMBERS:
                z.extract(m, tmp)
        src = os.path.join(tmp, "dbd", "src")
        cmd = ["g++", "-O3", "-std=c++14", "-fopenmp", "-w", "-fPIC", "-shared",
               "-DCOMPUTE", "-Dmain=dbd_reference_main", "-Wno-return-type", "-I", src,
               os.path.join(src, "main.cpp"), os.path.join(src, "distributeWorkload.cpp"),
               os.path.join(src, "computeCPU.cpp"), os.path.join(src, "readInput.cpp"),
               os.path.join(HERE, "ref_harness.cpp"), "-lpthread", "-Wl,--no-undefined", "-o", OUT]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    p = build(verbose=True)
    print(p or "skipped")
    sys.exit(0)
