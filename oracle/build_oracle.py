"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles the plain-C restatement ``fr_oracle.c`` (and
  ``fr_oracle_ext.c``, the components with no reference counterpart) into
  ``oracle/_build/liboracle.so`` (gcc, OpenMP, ``-ffp-contract=off``).
* ``build_ref()`` compiles the reference's OWN CPU sources, where they lie in
  the reference checkout, against the stub headers in ``oracle/ref_shim``
  (Qt containers/timer, GSL I0, FFTW3f calls) into
  ``oracle/_ref/libfastrecon_ref.so``.  It only runs where the reference
  checkout exists; nothing else reads the checkout.

Flags follow the reference's Release build (CMakeLists.txt:5 Release,
CMakeLists.txt:15 ``-std=c++11``, OpenMP), plus ``-ffp-contract=off`` so no
multiply-add is fused on any host (GCC fuses by default on aarch64, never on
plain x86-64), which keeps the results identical on x86 and Arm.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
DEFAULT_REF_ROOT = "/root/reference"

REF_SOURCES = [
    "ReconData/ReconData.cpp",
    "ReconData/GridLut.cpp",
    "ReconData/ConvKernel.cpp",
    "ImageData/ImageData.cpp",
    "ImageFilter/ImageFilter.cpp",
    "ImageFilter/FFT.cpp",
]

COMMON_FLAGS = ["-O3", "-DNDEBUG", "-fopenmp", "-ffp-contract=off", "-fPIC"]


def _run(cmd):
    subprocess.run(cmd, check=True)


def oracle_lib_path() -> str:
    return os.path.join(BUILD_DIR, "liboracle.so")


def ref_lib_path() -> str:
    return os.path.join(REF_OUT, "libfastrecon_ref.so")


def build_oracle(force: bool = False) -> str:
    out = oracle_lib_path()
    srcs = [os.path.join(HERE, "fr_oracle.c"), os.path.join(HERE, "fr_oracle_ext.c")]
    hdr = os.path.join(HERE, "fr_oracle.h")
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= max(map(os.path.getmtime, srcs + [hdr]))):
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp"
    _run(["gcc", "-std=c11", *COMMON_FLAGS, "-shared", *srcs, "-o", tmp, "-lm"])
    os.replace(tmp, out)
    return out


def build_ref(ref_root: str | None = None, force: bool = False) -> str | None:
    """Compile the reference CPU path; returns the .so path or None when the
    reference checkout is absent."""
    ref_root = ref_root or os.environ.get("FASTRECON_REF_ROOT", DEFAULT_REF_ROOT)
    if not os.path.isdir(os.path.join(ref_root, "ReconData")):
        return None
    out = ref_lib_path()
    shim = os.path.join(HERE, "ref_shim")
    deps = [os.path.join(ref_root, s) for s in REF_SOURCES]
    deps += [os.path.join(shim, f) for f in os.listdir(shim) if os.path.isfile(os.path.join(shim, f))]
    deps += [os.path.join(HERE, "fr_oracle.c"), os.path.join(HERE, "fr_oracle.h")]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(map(os.path.getmtime, deps)):
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    obj = os.path.join(REF_OUT, "fr_oracle.o")
    _run(["gcc", "-std=c11", *COMMON_FLAGS, "-c", os.path.join(HERE, "fr_oracle.c"), "-o", obj])
    cmd = ["g++", "-std=c++11", *COMMON_FLAGS, "-w", "-I", shim]
    for sub in ("ImageData", "ReconData", "ImageFilter"):
        cmd += ["-I", os.path.join(ref_root, sub)]
    cmd += [os.path.join(ref_root, s) for s in REF_SOURCES]
    cmd += [os.path.join(shim, "ref_shim.cpp"), os.path.join(shim, "ref_capi.cpp"), obj]
    tmp = out + ".tmp"
    cmd += ["-shared", "-o", tmp, "-lm"]
    _run(cmd)
    os.replace(tmp, out)
    return out


def clean() -> None:
    for d in (BUILD_DIR, REF_OUT):
        if os.path.isdir(d):
            shutil.rmtree(d)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="build the CPU oracle and, where the reference checkout exists, "
                                             "the reference's own CPU sources")
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $FASTRECON_REF_ROOT, else the build machine's checkout)")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build_oracle(force=a.force))
    print(build_ref(ref_root=a.reference, force=a.force))
