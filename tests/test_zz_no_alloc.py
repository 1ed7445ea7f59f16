"""fr_grid_noalloc: gridding for callers that cannot let a library allocate
device memory during their work (a real-time reconstruction loop with a
memory budget fixed at start-up, or a host framework whose caching allocator
holds the device memory).  Its buffers come from a fixed 32 MiB device
scratch array instead of cudaMalloc.

This file is collected last (test_zz_*), so a run that stops at the first
failure has run every other test before it.  It passes alone in a fresh
process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case, rel_l2

TOL = 1e-5


def test_noalloc_rejects_sizes_beyond_the_scratch(frlib):
    """A trajectory whose buffers cannot fit the 32 MiB scratch is refused
    with FR_ERR_CAPACITY before any GPU work (no device pointer is touched)."""
    lut = (C.c_float * 512)(*([1.0] * 512))
    fake = C.c_void_p(256)  # aligned, never dereferenced: the size check comes first
    n = 4_000_000           # 64 MB of trajectory alone
    st = frlib.fr_grid_noalloc(fake, n, 2, 512, 4.0, lut, 512, fake, fake, 8, fake, None)
    assert st == 9  # FR_ERR_CAPACITY
    assert b"32 MiB" in frlib.fr_last_error()
    st = frlib.fr_grid_noalloc(fake, 16, 2, 64, 4.0, (C.c_float * 2048)(), 2048, fake, fake, 1, fake, None)
    assert st == 9 and b"FR_NOALLOC_MAX_LUT" in frlib.fr_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "spiral2d_w3", "radial2d_oddgrid"])
def test_noalloc_matches_plan_and_grid(frlib, name):
    """Two calls in a row through the C ABI agree with fr_plan_* + fr_grid
    (and the second call is not disturbed by what the first left behind)."""
    import torch

    import fastrecon_gb300 as fr
    c = load_case(name)
    traj = torch.from_numpy(c["traj"]).cuda()
    dcf = torch.from_numpy(c["dcf"]).cuda()
    kd = torch.from_numpy(c["kdata"]).cuda()
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"])
    plan.set_trajectory(traj)
    want = plan.grid(kd, dcf).cpu().numpy()

    lut = np.ascontiguousarray(c["lut"], np.float32)
    lutp = lut.ctypes.data_as(C.POINTER(C.c_float))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for scale in (1.0, 2.0):
        kds = (kd * scale).contiguous()
        out = torch.full((c["coils"], c["G"] ** c["dim"]), float("nan"), dtype=torch.complex64, device="cuda")
        st = frlib.fr_grid_noalloc(C.c_void_p(traj.data_ptr()), traj.shape[0], c["dim"], c["G"], c["W"], lutp,
                                   len(lut), C.c_void_p(kds.data_ptr()), C.c_void_p(dcf.data_ptr()), c["coils"],
                                   C.c_void_p(out.data_ptr()), stream)
        assert st == 0, frlib.fr_last_error()
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy() / scale)
    for got in outs:
        assert rel_l2(got, want) <= TOL
        assert rel_l2(got, c["grid"]) <= TOL


def _noalloc(frlib, torch, traj, dim, G, W, lut, kd, dcf, coils):
    lut = np.ascontiguousarray(lut, np.float32)
    out = torch.full((coils, G ** dim), float("nan"), dtype=torch.complex64, device="cuda")
    st = frlib.fr_grid_noalloc(C.c_void_p(traj.data_ptr()), traj.shape[0], dim, G, W,
                               lut.ctypes.data_as(C.POINTER(C.c_float)), len(lut), C.c_void_p(kd.data_ptr()),
                               C.c_void_p(dcf.data_ptr()), coils, C.c_void_p(out.data_ptr()),
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, out


def _golden_call(frlib, torch, name):
    c = load_case(name)
    st, out = _noalloc(frlib, torch, torch.from_numpy(c["traj"]).cuda(), c["dim"], c["G"], c["W"], c["lut"],
                       torch.from_numpy(c["kdata"]).cuda(), torch.from_numpy(c["dcf"]).cuda(), c["coils"])
    assert st == 0, frlib.fr_last_error()
    return rel_l2(out.cpu().numpy(), c["grid"])


@pytest.mark.gpu
def test_noalloc_alternating_cases(frlib):
    """Calls with different trajectories in a row -- a larger 3D case, a
    smaller 2D one on an odd grid, the 3D one again -- each match the
    reference's grid: counters, tile tables and partial tiles left by the
    call before do not leak into the next."""
    import torch
    for name in ["koosh3d_small", "radial2d_oddgrid", "koosh3d_small", "radial2d_small", "koosh3d_odd"]:
        assert _golden_call(frlib, torch, name) <= TOL, name


@pytest.mark.gpu
def test_noalloc_capacity_found_after_planning(frlib):
    """Trajectories whose bin records (a 3D kooshball of 1 M samples on a 64^3
    grid) or split-tile partials (200,000 samples at one point of a 2D grid)
    exceed the scratch are counted by the plan's kernels and then refused
    with FR_ERR_CAPACITY; the next call with a good trajectory is correct."""
    import torch

    from fastrecon_gb300 import synth
    lut = load_case("koosh3d_small")["lut"]
    traj = synth.kooshball_3d(4000, 256)
    n = traj.shape[0]
    t = torch.from_numpy(traj).cuda()
    kd = torch.ones((1, n), dtype=torch.complex64, device="cuda")
    dcf = torch.ones(n, dtype=torch.float32, device="cuda")
    st, _ = _noalloc(frlib, torch, t, 3, 64, 4.0, lut, kd, dcf, 1)
    assert st == 9 and b"bin lists" in frlib.fr_last_error(), frlib.fr_last_error()
    assert _golden_call(frlib, torch, "koosh3d_small") <= TOL

    m = 200_000
    pts = np.zeros((m, 4), np.float32)
    pts[0, :2] = -0.5
    pts[1, :2] = 0.4999
    t = torch.from_numpy(pts).cuda()
    kd = torch.ones((8, m), dtype=torch.complex64, device="cuda")
    dcf = torch.ones(m, dtype=torch.float32, device="cuda")
    st, _ = _noalloc(frlib, torch, t, 2, 512, 4.0, load_case("radial2d_small")["lut"], kd, dcf, 8)
    assert st == 9 and b"partial tiles" in frlib.fr_last_error(), frlib.fr_last_error()
    assert _golden_call(frlib, torch, "radial2d_small") <= TOL
