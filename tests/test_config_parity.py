"""GPU parity at the benchmark configurations' full sizes.

The shipped path (default tiling, records per work item chosen from the
sample count, checkerboard flush + pruned FFT in the recon) against the
oracle on the same seeded inputs:

* config 1 in full: 2D radial 256 spokes x 512, 8 coils, |k| DCF, W 4,
  os 2 (512^2 grid), 256^2 SoS;
* config 2's full trajectory: 50,000 golden-means spokes x 256 (12.8 M
  samples), |k|^2 DCF, os 1.5 (384^3 grid), 256^3 SoS, with 2 of the 16
  coils (the oracle's time grows with the coils; the trajectory, the tile
  densities and the work items -- 4,096-record items, ~75 per centre tile --
  are those of the full configuration); and the same 2 coils in a coil
  group of 16, through the benchmark's tap-lane scatter;
* config 3: three frames (the sparsest, the densest and one between) of the
  64-frame dynamic spiral batch, gridded by the persistent batch kernel with
  the autotuner's tiling, 12 coils, 384^2 grid;
* config 5: two volumes of the batched kooshball (10k-60k spokes x 256,
  320^3 grid) through the batch kernel, 2 coils.

Bars: relative L2 <= 1e-5 against the reference's FP32 algorithm (the oracle
is pinned bit for bit to the reference's own CPU build on the golden
fixtures; its band-parallel form is pinned to the sequential one).  Each test
prints the error of the GPU result and of the reference's FP32 algorithm
against the FP64 gridding oracle.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

TOL = 1e-5


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need CUDA"
    from fastrecon_gb300 import build
    build.build()
    return t


def _report(name, gpu_vs_ref, gpu_vs_f64, ref_vs_f64, what="grid"):
    print(f"{name} {what}: GPU vs reference algorithm rel-L2 {gpu_vs_ref:.2e}, GPU vs FP64 oracle "
          f"{gpu_vs_f64:.2e}, reference FP32 vs FP64 {ref_vs_f64:.2e}")


def _grid_and_image(torch, oracle, name, traj, dcf, kd, dim, recon, os_, W=4.0, L=512):
    import fastrecon_gb300 as fr
    G = fr.grid_size(recon, os_)
    lut = oracle.kb_lut(W, os_, L)
    n = traj.shape[0]
    coils = kd.shape[0]
    kd_np = kd.cpu().numpy()
    tn, _, _, _, _ = oracle.normalize_traj(traj, dim, G)

    plan = fr.GridPlan(dim, G, W, lut=lut)
    plan.set_trajectory(torch.from_numpy(traj).cuda())
    g = plan.grid(kd, torch.from_numpy(dcf).cuda()).cpu().numpy()
    ref = oracle.grid_bands(tn, dcf, kd_np, dim, G, W, lut)
    g64 = oracle.grid_f64_bands(tn, dcf, kd_np, dim, G, W, lut)
    e_ref, e64, r64 = rel_l2(g, ref), rel_l2(g, g64), rel_l2(ref, g64)
    _report(name, e_ref, e64, r64)
    assert e_ref <= TOL
    assert np.array_equal(g == 0, ref == 0)
    del g, g64

    out = (recon,) * dim + ((1,) if dim == 2 else ())
    rec = fr.Recon(dim, recon, os_, coils, kernel_width=W, lut_length=L, max_samples=n)
    img = rec.run(torch.from_numpy(traj).cuda(), torch.from_numpy(dcf).cuda(), kd).cpu().numpy()
    want = oracle.recon_bands(traj, dcf, kd_np, dim, recon, os_, W, L, out)
    e_img = rel_l2(img, want)
    print(f"{name} image: GPU recon (checkerboard flush, pruned FFT, fused crop/SoS) vs reference algorithm "
          f"rel-L2 {e_img:.2e}")
    assert e_img <= TOL
    return e_ref, e64


def test_config1_radial2d_full(torch, oracle):
    from fastrecon_gb300 import synth
    traj, dcf, kd = synth.make_case(**synth.CONFIGS["radial2d"], xp=torch, device="cuda")
    assert traj.shape[0] == 256 * 512 and kd.shape[0] == 8
    _grid_and_image(torch, oracle, "config 1 (2D radial 256x512, 8 coils, 512^2)", traj, dcf, kd, 2, 256, 2.0)


def test_config2_kooshball_full_trajectory(torch, oracle):
    from fastrecon_gb300 import synth
    cfg = dict(synth.CONFIGS["kooshball3d"])
    cfg["coils"] = 2
    traj, dcf, kd = synth.make_case(**cfg, xp=torch, device="cuda")
    assert traj.shape[0] == 50000 * 256
    _grid_and_image(torch, oracle, "config 2 (3D kooshball 50,000x256, 2 of 16 coils, 384^3)", traj, dcf, kd, 3,
                    256, 1.5)


def test_config2_kooshball_full_trajectory_tap_lanes(torch, oracle):
    """Config 2's full trajectory through the benchmark's scatter kernel: a
    coil group of 16 (rows of 32 coil floats: the tap-lane scatter, here with
    2 of its 16 coils filled), the full trajectory's tile densities and split
    tiles.  Bit-equal to the per-warp tap-list scatter on the same
    deterministic plan, and the reference's FP32 algorithm at 1e-5."""
    import os

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    cfg = dict(synth.CONFIGS["kooshball3d"])
    cfg["coils"] = 2
    traj, dcf, kd = synth.make_case(**cfg, xp=torch, device="cuda")
    G, W = fr.grid_size(256, 1.5), 4.0
    lut = oracle.kb_lut(W, 1.5, 512)
    td, dd = torch.from_numpy(traj).cuda(), torch.from_numpy(dcf).cuda()
    grids = []
    for warp_lists in (False, True):
        if warp_lists:
            os.environ["FR_SCATTER_WARP_LISTS"] = "1"
        try:
            plan = fr.GridPlan(3, G, W, lut=lut, coil_group=16, deterministic=True)
            plan.set_trajectory(td)
            assert plan.tap_words() > 0 and plan.stats()["slots"] > 0
            grids.append(plan.grid(kd, dd).cpu().numpy())
            del plan
        finally:
            os.environ.pop("FR_SCATTER_WARP_LISTS", None)
    assert np.array_equal(grids[0].view(np.uint32), grids[1].view(np.uint32))
    g = grids[0]
    del grids
    tn, _, _, _, _ = oracle.normalize_traj(traj, 3, G)
    ref = oracle.grid_bands(tn, dcf, kd.cpu().numpy(), 3, G, W, lut)
    e_ref = rel_l2(g, ref)
    print(f"config 2 full trajectory, tap-lane scatter (coil group 16): = per-warp tap lists bit for bit; "
          f"vs reference algorithm rel-L2 {e_ref:.2e}")
    assert e_ref <= TOL
    assert np.array_equal(g == 0, ref == 0)


def _batch_frames(torch, oracle, name, trajs, kds, dcfs, dim, G, W, os_, check_frames, autotune):
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import batch as fb
    lut = oracle.kb_lut(W, os_, 512)
    counts = [t.shape[0] for t in trajs]
    traj = torch.from_numpy(np.concatenate(trajs)).cuda()
    dcf = torch.from_numpy(np.concatenate(dcfs)).cuda()
    kd = torch.cat([k.reshape(-1) for k in kds])
    coils = kds[0].shape[0]
    if autotune:
        b, _ = fb.autotune(dim, G, traj, counts, kd, dcf, coils, overgrid_factor=os_, repeats=1)
    else:
        b = fb.GridBatch(dim, G, W, lut=lut)
    b.set_trajectories(traj, counts)
    out = b.grid(kd, dcf, coils)
    torch.cuda.synchronize()
    errs = []
    for f in check_frames:
        g = out[f].cpu().numpy()
        tn, _, _, _, _ = oracle.normalize_traj(trajs[f], dim, G)
        kn = kds[f].cpu().numpy()
        ref = oracle.grid_bands(tn, dcfs[f], kn, dim, G, W, lut)
        g64 = oracle.grid_f64_bands(tn, dcfs[f], kn, dim, G, W, lut)
        e_ref, e64, r64 = rel_l2(g, ref), rel_l2(g, g64), rel_l2(ref, g64)
        _report(f"{name} frame {f} ({counts[f]} samples)", e_ref, e64, r64)
        assert e_ref <= TOL
        assert np.array_equal(g == 0, ref == 0)
        errs.append(e64)
    return errs


def test_config3_spiral_batch_frames(torch, oracle):
    """Frames of the batched dynamic spiral (the bench's seeded batch)."""
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    frames, coils, recon, os_, samples, seed = 64, 12, 192, 2.0, 2048, 3
    rng = np.random.default_rng(seed)
    inter = rng.integers(4, 25, frames)
    trajs = [synth.spiral_2d(int(k), samples, rotation=float(rng.uniform(0, 2 * np.pi))) for k in inter]
    dcfs = [synth.ramp_dcf(t, 2, 1.0) for t in trajs]
    kds = [synth.kspace(t, 2, recon, coils, seed=seed + f, xp=torch, device="cuda") for f, t in enumerate(trajs)]
    G = fr.grid_size(recon, os_)
    assert G == 384
    order = np.argsort(inter, kind="stable")
    check = [int(order[0]), int(order[frames // 2]), int(order[-1])]
    _batch_frames(torch, oracle, "config 3 (spiral batch, 12 coils, 384^2)", trajs, kds, dcfs, 2, G, 4.0, os_, check,
                  autotune=True)


def test_config5_kooshball_batch_volumes(torch, oracle):
    """Two volumes of the batched 3D configuration (320^3 grid) through the
    persistent batch kernel."""
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    rng = np.random.default_rng(11)
    spokes = [int(s) for s in rng.integers(10000, 60001, 2)]
    trajs = [synth.kooshball_3d(s, 256) for s in spokes]
    dcfs = [synth.ramp_dcf(t, 3, 2.0) for t in trajs]
    kds = [synth.kspace(t, 3, 256, 2, seed=20 + v, xp=torch, device="cuda") for v, t in enumerate(trajs)]
    G = fr.grid_size(256, 1.25)
    assert G == 320
    _batch_frames(torch, oracle, "config 5 (kooshball batch, 2 coils, 320^3)", trajs, kds, dcfs, 3, G, 4.0, 1.25,
                  [0, 1], autotune=False)
