"""In-tree build of libfastrecon_gb300.so (sm_103a) with nvcc/g++.

Each translation unit is compiled in parallel, then linked into
``fastrecon_gb300/_lib/libfastrecon_gb300.so``.  A unit is rebuilt only when
it (or a header) is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libfastrecon_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", os.path.join(CUDA_HOME, "include"),
             "-I", os.path.join(ROOT, "include")]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(src: str, obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _compile(src: str, extra=()):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [NVCC, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    else:
        cmd = ["g++", *CXX_FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    """Compile every CUDA/C++ unit for sm_103a and link the shared library."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _headers()
    srcs = sources()
    todo = [s for s in srcs if force or ptxas_v or _stale(s, os.path.join(OBJ, os.path.basename(s) + ".o"), deps)]
    extra = ("-Xptxas", "-v") if ptxas_v else ()
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            for obj, log in ex.map(lambda s: _compile(s, extra), todo):
                if verbose and log.strip():
                    print(log)
    objs = [os.path.join(OBJ, os.path.basename(s) + ".o") for s in srcs]
    if force or todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-L", os.path.join(CUDA_HOME, "lib64"), "-lcufft",
               "-Xlinker", "-rpath," + os.path.join(CUDA_HOME, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_cpp_api(force=force)
    build_cli(force=force)
    return LIB


CPP_SRC = os.path.join(PKG, "cpp")
CPP_LIB = os.path.join(LIBDIR, "libfastrecon.so")


def build_cpp_api(force: bool = False) -> str:
    """The C++ drop-in classes (ReconData, GridLut, ConvKernel, ImageFilter,
    ImageData, cuImageData, ...) as libfastrecon.so on top of the C ABI."""
    srcs = sorted(glob.glob(os.path.join(CPP_SRC, "*.cpp")))
    hdrs = glob.glob(os.path.join(ROOT, "include", "fastrecon", "*.h")) + [os.path.join(ROOT, "include",
                                                                                        "fastrecon_gb300.h")]
    if not force and os.path.exists(CPP_LIB) and \
            os.path.getmtime(CPP_LIB) >= max(os.path.getmtime(f) for f in srcs + hdrs + [LIB]):
        return CPP_LIB
    tmp = CPP_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(CUDA_HOME, "include"), *srcs, "-o", tmp, "-L", LIBDIR, "-lfastrecon_gb300",
           "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
           "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"C++ API build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CPP_LIB)
    return CPP_LIB


CLI_SRC = os.path.join(CPP_SRC, "cli", "fastrecon_main.cpp")
CLI = os.path.join(LIBDIR, "fastrecon")


def build_cli(force: bool = False) -> str:
    """The reference's command-line program (Program/Main.cpp) on the C++ API:
    fastrecon_gb300/_lib/fastrecon."""
    hdrs = glob.glob(os.path.join(ROOT, "include", "fastrecon", "*.h"))
    if not force and os.path.exists(CLI) and \
            os.path.getmtime(CLI) >= max(os.path.getmtime(f) for f in hdrs + [CLI_SRC, CPP_LIB]):
        return CLI
    tmp = CLI + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(CUDA_HOME, "include"), CLI_SRC, "-o", tmp, "-L", LIBDIR, "-lfastrecon", "-lfastrecon_gb300",
           "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
           "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def clean():
    for d in (OBJ, LIBDIR):
        if os.path.isdir(d):
            shutil.rmtree(d)


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas" in sys.argv))
