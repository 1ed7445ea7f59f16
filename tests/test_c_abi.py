"""CPU: include/fastrecon_gb300.h is a C header (C99, no C++ or torch types)
and the library links into a plain C program, which calls its host-only
entry points: the boundary a cgo / JNI / N-API binding uses."""
import os
import subprocess

import numpy as np

from conftest import GOLDEN, ROOT

LIBDIR = os.path.join(ROOT, "fastrecon_gb300", "_lib")


def test_c99_program_links_and_calls_the_library(tmp_path, frlib):
    exe = str(tmp_path / "abi_consumer")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "abi_consumer.c"), "-o", exe, "-L", LIBDIR, "-lfastrecon_gb300",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    first = r.stdout.splitlines()[0].split("|")
    assert first[1] == "ok"
    # the LUT the C program got equals the reference's (golden fixture)
    ref = np.load(os.path.join(GOLDEN, "luts.npz"))["w4.0_os1.5_l512"]
    assert np.float32(first[2]) == ref[0] and np.float32(first[3]) == ref[511]
