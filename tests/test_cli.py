"""The command-line drop-in for the reference's Program/Main.cpp
(fastrecon_gb300/cpp/cli/fastrecon_main.cpp): same options and RECON.ini
keys; on the GPU it reproduces the reference's recon from raw files."""
import os
import subprocess

import numpy as np
import pytest

from conftest import load_case, rel_l2

from test_cpp_api import write_case


def cli():
    from fastrecon_gb300 import build
    build.build()
    return build.CLI


def write_ini(d, c, extra=""):
    rz = c["recon"] if c["dim"] == 3 else 1
    with open(os.path.join(d, "RECON.ini"), "w") as f:
        f.write("[General]\n"
                "traj_file=traj_*.f32\n"
                "weight_file=dcf.f32\n"
                "data_file=data_*.c64\n"
                "out_file=image.f32\n"
                f"xres={c['readout']}\n"
                f"projections={c['spokes']}\n"
                f"rcxres={c['recon']}\nrcyres={c['recon']}\nrczres={rz}\n"
                f"overgridding_factor={c['os']!r}\n" + extra)
    return os.path.join(d, "RECON.ini")


def test_cli_arguments_without_gpu(tmp_path):
    exe = cli()
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "RECON.ini" in r.stdout and "--pils" in r.stdout
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 64 and "Missing RECON.ini" in r.stderr
    r = subprocess.run([exe, "a.ini", "b.ini"], capture_output=True, text=True)
    assert r.returncode == 64 and "too many arguments" in r.stderr
    r = subprocess.run([exe, "--bogus", "a.ini"], capture_output=True, text=True)
    assert r.returncode == 64
    r = subprocess.run([exe, str(tmp_path / "missing.ini")], capture_output=True, text=True)
    assert r.returncode == 1 and "does not exist" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "radial2d_oddgrid"])
def test_cli_recon_vs_reference(tmp_path, name):
    c = load_case(name)
    assert c["L"] == 512  # Main.cpp plans with a 512-entry LUT
    exe = cli()
    d = str(tmp_path)
    write_case(c, d)
    ini = write_ini(d, c)
    r = subprocess.run([exe, "--gpu", "-w", repr(c["W"]), ini], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Gridding total time" in r.stdout
    out = np.fromfile(os.path.join(d, "image.f32"), np.float32)
    assert rel_l2(out, c["image"]) <= 1e-5


@pytest.mark.gpu
def test_cli_pils_and_option_precedence(tmp_path):
    """--pils runs the PILS branch; -g overrides the ini's overgridding_factor."""
    c = load_case("radial2d_small")
    exe = cli()
    d = str(tmp_path)
    write_case(c, d)
    ini = write_ini(d, c)
    with open(ini) as f:
        text = f.read().replace(f"overgridding_factor={c['os']!r}", "overgridding_factor=1.25")
    with open(ini, "w") as f:
        f.write(text)
    r = subprocess.run([exe, "--pils", f"-g{c['os']!r}", ini], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Recon PILS" in r.stdout
    out = np.fromfile(os.path.join(d, "image.f32"), np.float32)
    assert rel_l2(out, c["image_pils"]) <= 1e-5
