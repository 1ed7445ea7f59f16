"""Batched gridding (no counterpart in the reference): many frames with
uneven sample counts in one persistent launch, CUDA-graph capture and
replay, and the autotuner.  Each frame must equal the single-trajectory
path (fr_plan_* + fr_grid) on the same frame, which the parity tests pin to
the reference."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2
from fastrecon_gb300 import synth

TOL = 1e-5  # the project's gridding bar: batches may chunk bins differently from the single path


def test_batch_rejects_bad_arguments_without_gpu(frlib):
    assert frlib.fr_batch_replay(None, None) == 1
    off = (C.c_size_t * 3)(0, 5, 3)
    assert frlib.fr_batch_set_trajectories(None, None, off, 2, None) == 1
    assert frlib.fr_batch_grid(None, None, None, 1, None, None) == 1


def _frames_2d(counts_il, samples=512, seed=0):
    trajs = [synth.spiral_2d(k, samples, turns=8.0) if i % 2 == 0 else synth.golden_angle_2d(k, samples)
             for i, k in enumerate(counts_il)]
    return trajs


def _kdata(counts, coils, seed):
    rng = np.random.default_rng(seed)
    return [(rng.standard_normal((coils, n)) + 1j * rng.standard_normal((coils, n))).astype(np.complex64)
            for n in counts]


def _flat(kds):
    return np.concatenate([k.ravel() for k in kds])


def _check_against_single(batch_out, trajs, kds, dcfs, dim, G, W, lut, torch, fr):
    for f, (t, k, d) in enumerate(zip(trajs, kds, dcfs)):
        plan = fr.GridPlan(dim, G, W, lut=lut)
        plan.set_trajectory(torch.from_numpy(t).cuda())
        want = plan.grid(torch.from_numpy(k).cuda(), torch.from_numpy(d).cuda()).cpu().numpy()
        assert rel_l2(batch_out[f], want) <= TOL, f


@pytest.mark.gpu
@pytest.mark.parametrize("coils", [1, 5, 12])
def test_batch_2d_matches_single_frames(coils):
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300.batch import GridBatch
    G, W = 96, 4.0
    lut = fr.kb_lut(W, 2.0, 512)
    trajs = _frames_2d([2, 5, 1, 8, 3, 4, 6])
    counts = [t.shape[0] for t in trajs]
    kds = _kdata(counts, coils, 1)
    dcfs = [synth.ramp_dcf(t, 2, 1.0) for t in trajs]
    b = GridBatch(2, G, W, lut=lut, chunk=1024)
    b.set_trajectories(torch.from_numpy(np.concatenate(trajs)).cuda(), counts)
    st = b.stats()
    assert st["frames"] == 7 and st["samples"] == sum(counts) and st["ctas"] > 0
    out = b.grid(torch.from_numpy(_flat(kds)).cuda(), torch.from_numpy(np.concatenate(dcfs)).cuda(), coils)
    _check_against_single(out.cpu().numpy(), trajs, kds, dcfs, 2, G, W, lut, torch, fr)


@pytest.mark.gpu
def test_batch_3d_uneven_volumes():
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300.batch import GridBatch
    G, W = 40, 4.0
    lut = fr.kb_lut(W, 1.25, 512)
    trajs = [synth.kooshball_3d(s, 32) for s in (120, 300, 60)]
    counts = [t.shape[0] for t in trajs]
    kds = _kdata(counts, 6, 2)
    dcfs = [synth.ramp_dcf(t, 3, 2.0) for t in trajs]
    b = GridBatch(3, G, W, lut=lut, chunk=2048)
    b.set_trajectories(torch.from_numpy(np.concatenate(trajs)).cuda(), counts)
    out = b.grid(torch.from_numpy(_flat(kds)).cuda(), torch.from_numpy(np.concatenate(dcfs)).cuda(), 6)
    _check_against_single(out.cpu().numpy(), trajs, kds, dcfs, 3, G, W, lut, torch, fr)


@pytest.mark.gpu
def test_batch_empty_frame_is_zero():
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300.batch import GridBatch
    G = 64
    trajs = [synth.radial_2d(16, 64), synth.radial_2d(24, 64)]
    counts = [trajs[0].shape[0], 0, trajs[1].shape[0]]
    kds = _kdata([counts[0], counts[2]], 3, 3)
    flat = np.concatenate([kds[0].ravel(), kds[1].ravel()])
    dcf = np.concatenate([synth.ramp_dcf(t, 2) for t in trajs])
    b = GridBatch(2, G, 4.0)
    b.set_trajectories(torch.from_numpy(np.concatenate(trajs)).cuda(), counts)
    out = b.grid(torch.from_numpy(flat).cuda(), torch.from_numpy(dcf).cuda(), 3).cpu().numpy()
    assert not np.any(out[1])
    _check_against_single(out[[0, 2]], trajs, kds, [synth.ramp_dcf(t, 2) for t in trajs], 2, G, 4.0,
                          fr.kb_lut(4.0, 2.0, 512), torch, fr)


@pytest.mark.gpu
def test_batch_graph_replay_reads_current_buffers():
    import torch

    from fastrecon_gb300.batch import GridBatch
    G = 96
    trajs = _frames_2d([3, 7, 2, 5])
    counts = [t.shape[0] for t in trajs]
    kd = torch.from_numpy(_flat(_kdata(counts, 4, 4))).cuda()
    dcf = torch.from_numpy(np.concatenate([synth.ramp_dcf(t, 2) for t in trajs])).cuda()
    b = GridBatch(2, G, 4.0)
    b.set_trajectories(torch.from_numpy(np.concatenate(trajs)).cuda(), counts)
    direct = b.grid(kd, dcf, 4).cpu().numpy()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        out = b.capture(kd, dcf, 4, stream=s)
        b.replay(stream=s)
    s.synchronize()
    assert rel_l2(out.cpu().numpy(), direct) <= TOL
    kd.mul_(2.0)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        b.replay(stream=s)
        b.replay(stream=s)
    s.synchronize()
    assert rel_l2(out.cpu().numpy(), 2 * direct) <= TOL


@pytest.mark.gpu
def test_autotune_picks_a_valid_configuration():
    import torch

    from fastrecon_gb300 import batch as fb
    G = 128
    trajs = _frames_2d([4, 9, 2, 6, 3], samples=1024)
    counts = [t.shape[0] for t in trajs]
    kd = torch.from_numpy(_flat(_kdata(counts, 12, 5))).cuda()
    dcf = torch.from_numpy(np.concatenate([synth.ramp_dcf(t, 2) for t in trajs])).cuda()
    traj = torch.from_numpy(np.concatenate(trajs)).cuda()
    tuned, ms = fb.autotune(2, G, traj, counts, kd, dcf, 12, repeats=2)
    assert ms > 0
    tuned.set_trajectories(traj, counts)
    ref = fb.GridBatch(2, G, 4.0)
    ref.set_trajectories(traj, counts)
    assert rel_l2(tuned.grid(kd, dcf, 12).cpu().numpy(), ref.grid(kd, dcf, 12).cpu().numpy()) <= TOL
