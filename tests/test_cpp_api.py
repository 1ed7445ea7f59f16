"""The C++ drop-in API (include/fastrecon/*.h, libfastrecon.so): it builds and
links on the CPU; on the GPU the Program/Main.cpp pipeline written against it
(tests/cpp/recon_main.cpp, through ReconData::loadFromFiles, GridLut,
ImageFilter) reproduces the reference's outputs, plain and PILS."""
import os
import subprocess

import numpy as np
import pytest

from conftest import CASE_NAMES, ROOT, load_case, rel_l2

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
LIBDIR = os.path.join(ROOT, "fastrecon_gb300", "_lib")


def compile_main(outdir):
    from fastrecon_gb300 import build
    build.build()
    exe = os.path.join(outdir, "recon_main")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "cpp", "recon_main.cpp"), "-o", exe, "-L", LIBDIR, "-lfastrecon",
           "-lfastrecon_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart", f"-Wl,-rpath,{LIBDIR}",
           f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_builds_and_links(tmp_path):
    exe = compile_main(str(tmp_path))
    assert os.path.exists(exe)
    nm = subprocess.run(["nm", "-DC", os.path.join(LIBDIR, "libfastrecon.so")], capture_output=True, text=True).stdout
    for sym in ["ReconData<float>::Create", "ReconData<float>::loadFromFiles", "ReconData<float>::normalizeTraj",
                "GridLut<float>::Create", "cuGridLut<float>::plan", "cuGridLut<float>::execute",
                "ConvKernel::ConvKernel", "ImageFilter<float>::Create", "ImageFilter<float>::SOS",
                "ImageFilter<float>::fftShift", "ImageFilter<float>::lowFilter", "ImageFilter<float>::normalize",
                "ImageFilter<float>::crop", "cuImageData<float>::cuGetChannelImage", "ImageData<float>::addChannelImage"]:
        assert sym in nm, sym


def write_case(c, d):
    dim = c["dim"]
    for k in range(dim):
        np.ascontiguousarray(c["traj"][:, k]).astype(np.float32).tofile(os.path.join(d, f"traj_{k}.f32"))
    c["dcf"].astype(np.float32).tofile(os.path.join(d, "dcf.f32"))
    for ch in range(c["coils"]):
        np.ascontiguousarray(c["kdata"][ch]).astype(np.complex64).tofile(os.path.join(d, f"data_{ch}.c64"))


def run_main(exe, c, d, pils=False):
    rz = c["recon"] if c["dim"] == 3 else 1
    args = [exe, d, str(c["readout"]), str(c["spokes"]), str(c["coils"]), str(c["dim"]), str(c["recon"]),
            str(c["recon"]), str(rz), repr(c["os"]), repr(c["W"]), str(c["L"])] + (["pils"] if pils else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(os.path.join(d, "out.f32"), np.float32)
    tn = np.fromfile(os.path.join(d, "traj_norm.f32"), np.float32).reshape(-1, 4)
    g0 = np.fromfile(os.path.join(d, "grid0.c64"), np.complex64)
    return out, tn, g0


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASE_NAMES)
def test_main_pipeline_vs_reference(tmp_path, name):
    c = load_case(name)
    exe = compile_main(str(tmp_path))
    write_case(c, str(tmp_path))
    out, tn, g0 = run_main(exe, c, str(tmp_path))
    assert np.array_equal(tn.view(np.uint32), c["traj_norm"].view(np.uint32))
    assert rel_l2(g0, c["grid"][0]) <= 1e-5
    err = rel_l2(out, c["image"])
    print(f"{name}: C++ API recon rel-L2 vs reference {err:.2e}")
    assert err <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "radial2d_oddgrid"])
def test_main_pipeline_pils_vs_reference(tmp_path, name):
    c = load_case(name)
    exe = compile_main(str(tmp_path))
    write_case(c, str(tmp_path))
    out, _, _ = run_main(exe, c, str(tmp_path), pils=True)
    err = rel_l2(out, c["image_pils"])
    print(f"{name}: C++ API PILS recon rel-L2 vs reference {err:.2e}")
    assert err <= 1e-5


def compile_stream(outdir):
    from fastrecon_gb300 import build
    build.build()
    exe = os.path.join(outdir, "stream_main")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "cpp", "stream_main.cpp"), "-o", exe, "-L", LIBDIR, "-lfastrecon",
           "-lfastrecon_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart", f"-Wl,-rpath,{LIBDIR}",
           f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_stream_main_builds(tmp_path):
    assert os.path.exists(compile_stream(str(tmp_path)))


def _run_stream(tmp_path, oracle, name, env=None):
    """Runs stream_main on a golden case and checks its trajectory, DCF and
    three grids against the oracle; returns its stdout."""
    c = load_case(name)
    d = str(tmp_path)
    exe = compile_stream(d)
    dim, S, A, C = c["dim"], c["readout"], c["spokes"], c["coils"]
    il = np.concatenate([c["traj"][:, :dim], c["dcf"][:, None]], axis=1).astype(np.float32)
    il.tofile(os.path.join(d, "traj_il.f32"))
    kd = np.array(c["kdata"], np.complex64)
    for ch in range(C):
        kd[ch].tofile(os.path.join(d, f"data_{ch}.c64"))
    rng = np.random.default_rng(7)
    acqs = np.array([1, A - 1, A // 2, 2, A // 2], np.int32)  # includes a repeat
    acqs.tofile(os.path.join(d, "upd_acq.i32"))
    new = (rng.standard_normal((len(acqs), C, S)) + 1j * rng.standard_normal((len(acqs), C, S))).astype(np.complex64)
    for k in range(len(acqs)):
        for ch in range(C):
            new[k, ch].tofile(os.path.join(d, f"upd_{k}_{ch}.c64"))
    args = [exe, d, str(S), str(A), str(C), str(dim), str(c["recon"]), repr(c["os"]), repr(c["W"]), str(c["L"]),
            str(len(acqs))]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300,
                       env=None if env is None else {**os.environ, **env})
    assert r.returncode == 0, r.stdout + r.stderr
    tn = np.fromfile(os.path.join(d, "traj_norm.f32"), np.float32).reshape(-1, 4)
    assert np.array_equal(tn.view(np.uint32), c["traj_norm"].view(np.uint32))
    assert np.array_equal(np.fromfile(os.path.join(d, "dcf.f32"), np.float32), c["dcf"])
    cells = c["G"] ** dim
    half = len(acqs) // 2
    for g_name, upto in (("grid0", 0), ("grid1", half), ("grid2", len(acqs))):
        k = kd.copy()
        for j in range(upto):
            k[:, acqs[j] * S:(acqs[j] + 1) * S] = new[j]
        want = oracle.grid(c["traj_norm"], c["dcf"], k, dim, c["G"], c["W"], c["lut"], threads=4)
        got = np.fromfile(os.path.join(d, g_name + ".c64"), np.complex64).reshape(C, cells)
        err = rel_l2(got, want)
        print(f"{name} {g_name}: rel-L2 vs oracle {err:.2e}")
        assert err <= 1e-5, g_name
    return r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small"])
def test_cpp_streaming_acquisitions_vs_oracle(tmp_path, oracle, name):
    """ReconData::loadTraj (interleaved trajectory + DCF) and
    updateSingleAcquisition through the C++ API: the trajectory after plan is
    the reference's bit for bit, and the grids before the updates, after a
    first round (full regrid) and after a second round (only the updated
    readouts regridded, fr_grid_update) equal the oracle's grid of the same
    k-space at 1e-5."""
    out = _run_stream(tmp_path, oracle, name)
    assert "partitions=0" in out and "incremental1=0" in out and "incremental2=1" in out, out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small"])
def test_cpp_partitions_when_the_plan_does_not_fit(tmp_path, oracle, name):
    """cuGridLut with a plan that does not fit in device memory (host-side
    fault injection: reservations of 16 bytes per sample -- the plan's
    trajectory copy -- or more fail as cudaMalloc would) grids in sample
    partitions (fr_grid_partitioned), as the reference partitions its pair
    map (cuGridLut.cu:182-220), doubling the partitions while a partition's
    plan (its split-tile partials included) still does not fit; every
    execute regrids in full, and the grids equal the oracle's."""
    n = load_case(name)["traj"].shape[0]
    out = _run_stream(tmp_path, oracle, name, env={"FR_FAIL_ALLOC_BYTES": str(16 * n)})
    parts = int(out.split("partitions=")[1].split()[0])
    assert parts >= 2, out
    assert "incremental1=0" in out and "incremental2=0" in out, out
