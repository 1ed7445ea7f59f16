"""Streaming acquisition (fr_grid_update): ReconData::updateSingleAcquisition
(ReconData.cpp:179-189, cuReconData.cu:52-62) on the device with incremental
regridding.  After replacing readouts, the k-space buffer must equal the
updated k-space exactly and the grid must equal fr_grid of the updated
k-space (float rounding aside: the update adds with global atomics)."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case, rel_l2

TOL = 1e-5  # the project's gridding bar, on the whole grid
TOL_DELTA = 1e-3  # on the change of the grid alone (the full grids' own rounding is ~1e-7 of their norm)


def test_update_rejects_bad_arguments_without_gpu(frlib):
    assert frlib.fr_grid_update(None, None, None, 0, 4, None, 1, None, None) == 1  # FR_ERR_INVALID_ARGUMENT


def _setup(name, checkerboard):
    import torch

    import fastrecon_gb300 as fr
    c = load_case(name)
    if checkerboard and c["G"] % 2:
        pytest.skip("checkerboard plans need an even grid")
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], checkerboard=checkerboard)
    plan.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    kd = torch.from_numpy(c["kdata"]).cuda().contiguous()
    dcf = torch.from_numpy(c["dcf"]).cuda()
    return c, plan, kd, dcf


def _readout(c, seed):
    import torch
    rng = np.random.default_rng(seed)
    scale = np.abs(c["kdata"]).mean()
    v = scale * (rng.standard_normal((c["coils"], c["readout"])) + 1j * rng.standard_normal((c["coils"], c["readout"])))
    return torch.from_numpy(v.astype(np.complex64)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "spiral2d_w3"])
def test_update_vs_oracle(oracle, name):
    """After three readout replacements the incrementally updated grid equals
    the oracle's grid (the reference's FP32 algorithm) of the updated k-space
    at the project's 1e-5 bar."""
    import torch
    c, plan, kd, dcf = _setup(name, False)
    g = plan.grid(kd, dcf)
    ref = c["kdata"].copy()
    R = c["readout"]
    for k, acq in enumerate([1, c["spokes"] - 2, 1]):
        new = _readout(c, 20 + k)
        plan.update(kd, new, acq * R, dcf, g)
        ref[:, acq * R:(acq + 1) * R] = new.cpu().numpy()
    torch.cuda.synchronize()
    want = oracle.grid(c["traj_norm"], c["dcf"], ref, c["dim"], c["G"], c["W"], c["lut"], threads=4)
    err = rel_l2(g.cpu().numpy(), want)
    print(f"{name}: incrementally updated grid vs oracle rel-L2 {err:.2e}")
    assert err <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "spiral2d_w3"])
@pytest.mark.parametrize("checkerboard", [False, True])
def test_update_matches_full_regrid(name, checkerboard):
    import torch
    c, plan, kd, dcf = _setup(name, checkerboard)
    g0 = plan.grid(kd, dcf)
    g = g0.clone()
    ref = kd.clone()
    R = c["readout"]
    # two different readouts, then the first one again
    for k, acq in enumerate([3, c["spokes"] - 1, 3]):
        new = _readout(c, 10 + k)
        plan.update(kd, new, acq * R, dcf, g)
        ref[:, acq * R:(acq + 1) * R] = new
    torch.cuda.synchronize()
    assert torch.equal(kd, ref)  # the k-space itself, bit for bit
    want = plan.grid(ref, dcf)
    got, want, g0 = g.cpu().numpy(), want.cpu().numpy(), g0.cpu().numpy()
    assert rel_l2(got, want) <= TOL
    assert rel_l2(got - g0, want - g0) <= TOL_DELTA


@pytest.mark.gpu
def test_update_range_checked(frlib):
    import torch

    from fastrecon_gb300.capi import FastreconError
    c, plan, kd, dcf = _setup("radial2d_small", False)
    g = plan.grid(kd, dcf)
    new = _readout(c, 1)
    n = kd.shape[1]
    with pytest.raises(FastreconError):
        plan.update(kd, new, n - c["readout"] + 1, dcf, g)  # one sample past the end
    st = frlib.fr_grid_update(plan.h, C.c_void_p(kd.data_ptr()), C.c_void_p(new.data_ptr()), n, 0,
                              C.c_void_p(dcf.data_ptr()), c["coils"], C.c_void_p(g.data_ptr()), None)
    assert st == 0  # an empty update at the end is a no-op
    torch.cuda.synchronize()
