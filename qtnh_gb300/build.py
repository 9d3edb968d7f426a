"""Build the engine's shared libraries in-tree.

``libqtnh_cuda.so``  C ABI + CUDA kernels (sm_103a), from ``csrc/*.cu`` and ``csrc/*.cpp``.
``libqtnh.so``       the qtnh C++ API (``include/qtnh.hpp``), from ``cpp/*.cpp``; calls only
                     the C ABI and needs no CUDA headers.
``tests/cpp/_build/api_test``  the C++ API test driver.
``_build/api_bench``  workloads through the C++ API (drivers/api_bench.cpp), for the
                     benchmark and the drop-in tests.

Every .cu file is compiled with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` in parallel; the CUDA
runtime is linked statically so the library only needs the driver at run time.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
INCLUDE = os.path.join(ROOT, "include")
CUDA_LIB = "libqtnh_cuda.so"
API_LIB = "libqtnh.so"
CPP = os.path.join(HERE, "cpp")
TEST_SRC = os.path.join(ROOT, "tests", "cpp", "api_test.cpp")
TEST_BIN = os.path.join(ROOT, "tests", "cpp", "_build", "api_test")
DRIVER_SRC = os.path.join(HERE, "drivers", "api_bench.cpp")
DRIVER_BIN = os.path.join(BUILD, "api_bench")
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-I", INCLUDE, "-I", CPP]

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "qtnh_cuda.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _headers_mtime()):
        return obj
    cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    lib = os.path.join(LIBDIR, CUDA_LIB)
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", lib] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    api = _build_api(lib, force)
    _build_test(api, force)
    _build_driver(api, force)
    if verbose:
        print("built", lib, api, TEST_BIN)
    return lib


def _newer(target, deps):
    return os.path.exists(target) and os.path.getmtime(target) >= max(os.path.getmtime(d) for d in deps)


def _api_headers():
    hs = []
    for d, _, fs in os.walk(INCLUDE):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".hpp", ".h"))]
    hs += [os.path.join(CPP, f) for f in os.listdir(CPP) if f.endswith(".hpp")]
    return hs


def _build_api(cuda_lib, force):
    srcs = sorted(os.path.join(CPP, f) for f in os.listdir(CPP) if f.endswith(".cpp"))
    api = os.path.join(LIBDIR, API_LIB)
    if not force and _newer(api, srcs + _api_headers() + [cuda_lib]):
        return api
    cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-shared", "-o", api] + srcs + [
        "-L", LIBDIR, "-lqtnh_cuda", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("API library build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return api


def _build_test(api, force):
    os.makedirs(os.path.dirname(TEST_BIN), exist_ok=True)
    if not force and _newer(TEST_BIN, [TEST_SRC, api] + _api_headers()):
        return TEST_BIN
    cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-o", TEST_BIN, TEST_SRC, "-L", LIBDIR, "-lqtnh", "-lqtnh_cuda",
                                                        "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("API test build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return TEST_BIN


def _build_driver(api, force):
    if not force and _newer(DRIVER_BIN, [DRIVER_SRC, api] + _api_headers()):
        return DRIVER_BIN
    cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-O3", "-o", DRIVER_BIN, DRIVER_SRC, "-L", LIBDIR, "-lqtnh",
                                                        "-lqtnh_cuda", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("API driver build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return DRIVER_BIN


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
