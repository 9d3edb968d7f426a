"""Builds the reference's own hot-path code as a shared library for the oracle's checks.

TEST INFRASTRUCTURE. Compiles the reference checkout's ``src/core/*.cpp`` and
``src/tensor/*.cpp`` where they lie (nothing is copied into this repository), with the
flags of the reference's CMake Release build (``-O3 -DNDEBUG``, C++17), against the
single-process MPI subset in ``oracle/mpi_shim`` (the reference's MPI dependency is not
available here), plus ``oracle/ref_driver.cpp`` (C entry points for ctypes). Output:
``oracle/_ref/libqtnh_ref.so`` (git-ignored; x86-64 only, as the reference checkout is
only present on the build host).

Usage: ``python oracle/ref_build.py [path of the reference checkout]``.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT_DIR, "libqtnh_ref.so")
DEFAULT_REFERENCE = "/root/reference"


def sources(ref):
    return sorted(glob.glob(os.path.join(ref, "src", "core", "*.cpp")) +
                  glob.glob(os.path.join(ref, "src", "tensor", "*.cpp")))


def build(ref=DEFAULT_REFERENCE, force=False):
    """Returns the library path, or None when the reference checkout is absent."""
    srcs = sources(ref) if os.path.isdir(ref) else []
    if not srcs:
        return None
    own = [os.path.join(HERE, "mpi_shim", "mpi_shim.cpp"), os.path.join(HERE, "ref_driver.cpp"),
           os.path.join(HERE, "mpi_shim", "mpi.h")]
    deps = srcs + own + glob.glob(os.path.join(ref, "include", "*", "*.hpp"))
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps):
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-DNDEBUG", "-fPIC", "-shared", "-w", "-I", os.path.join(HERE, "mpi_shim"),
           "-I", os.path.join(ref, "include"), "-o", LIB_PATH] + srcs + own[:2]
    subprocess.check_call(cmd)
    return LIB_PATH


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REFERENCE, force=True)
    print(path or "reference checkout not found")
