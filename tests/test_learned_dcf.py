"""Learned DCF (no counterpart in the reference): density features, the
network's forward/backward/Adam kernels, and what the trained network gains
over the plain method.  The oracle is the FP64 CPU restatement in
oracle/fr_oracle_ext.c; its gradient is pinned by finite differences."""
import numpy as np
import pytest

from conftest import CASE_NAMES, load_case
from fastrecon_gb300 import synth

RADII = [1, 2, 4, 8]
TOL_FWD = 1e-5    # FP32 network vs FP64 oracle on the same BF16-valued parameters
TOL_GRAD = 1e-4   # FP32 batch-reduced gradient vs FP64 oracle (rel-L2)


def _params(seed=0, scale=0.3):
    from fastrecon_gb300.learned_dcf import N_PARAMS
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(N_PARAMS) * scale).astype(np.float32)


def _bf16_round(a):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


# ---------------------------------------------------------------- oracle (CPU)

def test_oracle_mlp_gradient_finite_differences(oracle):
    p = _params(1, 0.2)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((9, 5)).astype(np.float32)
    t = rng.standard_normal(9).astype(np.float32)
    _, g = oracle.mlp_backward(p, x, t)
    for i in [0, 7, 319, 320, 383, 384, 2000, 4479, 4480, 4543, 4544, 4607, 4608]:
        def loss(v):
            q = p.copy()
            q[i] = v
            return np.mean((oracle.mlp_forward(q, x) - t) ** 2)
        hi, lo = np.float32(p[i] + 1e-2), np.float32(p[i] - 1e-2)
        fd = (loss(hi) - loss(lo)) / (float(hi) - float(lo))
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_oracle_features_formula(oracle):
    t = synth.spiral_2d(4, 256)
    G = 64
    tn = oracle.normalize_traj(t, 2, G)[0]
    cnt = oracle.density_counts(tn, 2, G, RADII)
    kmax = np.float32(np.sqrt((t[:, :2].astype(np.float32) ** 2).sum(1)).max())
    f = oracle.dcf_features(cnt, t, 2, RADII, kmax)
    vol = (2 * np.array(RADII, np.float32) + 1) ** 2
    assert np.allclose(f[:, :4], np.log(cnt / vol), rtol=1e-6, atol=1e-6)
    assert np.allclose(f[:, 4], np.log(np.hypot(t[:, 0], t[:, 1]) / kmax + 1 / 1024), rtol=1e-5, atol=1e-6)


# ---------------------------------------------------------------- GPU kernels

def _plan_for(fr, torch, t, dim, G, W=4.0, os_=2.0):
    from oracle.pyoracle import Oracle  # noqa: F401  (oracle fixture covers the build)
    plan = fr.GridPlan(dim, G, W, overgrid_factor=os_)
    td = torch.from_numpy(np.ascontiguousarray(t)).cuda()
    plan.set_trajectory(td)
    return plan, td


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASE_NAMES)
def test_gpu_density_counts_bit_exact(oracle, name):
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import learned_dcf as ld
    c = load_case(name)
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"])
    plan.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    got = ld.density_counts(plan, RADII).cpu().numpy()
    want = oracle.density_counts(c["traj_norm"].astype(np.float32), c["dim"], c["G"], RADII)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_gpu_features_match_oracle(oracle):
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import learned_dcf as ld
    for t, dim, G in ((synth.spiral_2d(6, 512), 2, 96), (synth.kooshball_3d(300, 48), 3, 48)):
        plan, td = _plan_for(fr, torch, t, dim, G)
        cnt = ld.density_counts(plan, RADII)
        got = ld.dcf_features(plan, td, counts=cnt).cpu().numpy()
        q = (t[:, :dim] * t[:, :dim]).astype(np.float32)
        kq = q[:, 0]
        for d in range(1, dim):
            kq = (kq + q[:, d]).astype(np.float32)
        kmax = np.sqrt(kq).astype(np.float32).max()
        want = oracle.dcf_features(cnt.cpu().numpy(), t, dim, RADII, kmax)
        # logf on the device and on the host may differ in the last place
        assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))


@pytest.mark.gpu
def test_gpu_mlp_forward_matches_oracle(oracle):
    import torch

    from fastrecon_gb300 import learned_dcf as ld
    net = ld.DCFNet(_params(3))
    pf = net.params_bf16_as_float()
    assert np.array_equal(pf, _bf16_round(net.master.cpu().numpy()))
    rng = np.random.default_rng(4)
    x = rng.standard_normal((3000, 5)).astype(np.float32)
    got = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    want = oracle.mlp_forward(pf, x)
    assert np.linalg.norm(got - want) <= TOL_FWD * np.linalg.norm(want)
    gexp = net.forward(torch.from_numpy(x).cuda(), exp=True, scale=0.25).cpu().numpy()
    assert np.allclose(gexp, 0.25 * np.exp(want), rtol=1e-4)
    net.residual = True
    got_r = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    want_r = oracle.mlp_forward(pf, x, residual=True)
    assert np.linalg.norm(got_r - want_r) <= TOL_FWD * np.linalg.norm(want_r)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 15, 16, 17, 1000, 70001])
def test_gpu_mlp_forward_tensor_cores_vs_fp32_path(oracle, n):
    """The inference forward (hidden layer on the tensor cores, mma.sync with
    BF16 operand terms and FP32 accumulation) against the FP32 CUDA-core
    forward (FR_MLP_SIMT=1) and the FP64 oracle, for sample counts around
    its 16-sample tiles."""
    import os

    import torch

    from fastrecon_gb300 import learned_dcf as ld
    net = ld.DCFNet(_params(5))
    pf = net.params_bf16_as_float()
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, 5)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    got = net.forward(xt).cpu().numpy()
    os.environ["FR_MLP_SIMT"] = "1"
    try:
        simt = net.forward(xt).cpu().numpy()
    finally:
        os.environ.pop("FR_MLP_SIMT")
    want = oracle.mlp_forward(pf, x)
    e_tc, e_simt = np.linalg.norm(got - want) / np.linalg.norm(want), np.linalg.norm(simt - want) / np.linalg.norm(want)
    print(f"n={n}: tensor-core forward vs FP64 {e_tc:.2e}, FP32 CUDA-core forward vs FP64 {e_simt:.2e}")
    assert e_tc <= TOL_FWD and e_simt <= TOL_FWD
    assert np.linalg.norm(got - simt) <= 2 * TOL_FWD * np.linalg.norm(want)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 37, 256, 5000])
@pytest.mark.parametrize("weighted", [False, True])
def test_gpu_mlp_gradient_matches_oracle(oracle, n, weighted):
    """The hand-written backward pass against the FP64 oracle's gradient."""
    import torch

    from fastrecon_gb300 import learned_dcf as ld
    net = ld.DCFNet(_params(5))
    pf = net.params_bf16_as_float()
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, 5)).astype(np.float32)
    t = rng.standard_normal(n).astype(np.float32)
    c = rng.uniform(0.1, 3.0, n).astype(np.float32) if weighted else None
    loss = net.loss_grad(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda(),
                         None if c is None else torch.from_numpy(c).cuda()).item()
    g = net.grad.cpu().numpy()
    lw, gw = oracle.mlp_backward(pf, x, t, c)
    assert abs(loss - lw) <= 1e-5 * abs(lw)
    assert np.linalg.norm(g - gw) <= TOL_GRAD * np.linalg.norm(gw)


@pytest.mark.gpu
def test_gpu_adam_step():
    import torch

    from fastrecon_gb300 import learned_dcf as ld
    p = _params(6)
    net = ld.DCFNet(p)
    rng = np.random.default_rng(7)
    g1 = rng.standard_normal(ld.N_PARAMS).astype(np.float32)
    g2 = rng.standard_normal(ld.N_PARAMS).astype(np.float32)
    m = np.zeros(ld.N_PARAMS)
    v = np.zeros(ld.N_PARAMS)
    w = p.astype(np.float64)
    for step, g in enumerate((g1, g2), 1):
        net.grad.copy_(torch.from_numpy(g))
        net.adam(lr=1e-2)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g.astype(np.float64) ** 2
        w = w - 1e-2 * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
    assert np.allclose(net.master.cpu().numpy(), w, rtol=1e-5, atol=1e-6)
    assert np.array_equal(net.params_bf16_as_float(), _bf16_round(net.master.cpu().numpy()))


def _nrmse(a, ref):
    """Relative RMS error after the best scalar scaling of a onto ref."""
    a = np.asarray(a, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    c = np.dot(a, ref) / np.dot(a, a)
    return np.linalg.norm(c * a - ref) / np.linalg.norm(ref)


@pytest.mark.gpu
def test_gpu_learned_dcf_beats_plain_method():
    """Train the network on Pipe-Menon DCFs of a few 2D trajectories (on the
    GPU, with the project's kernels) and reconstruct held-out trajectories:
    the learned-DCF image is closer to the Pipe-DCF image than the plain
    method's (analytic |k| DCF) image is."""
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import learned_dcf as ld
    recon, os_, W = 64, 2.0, 4.0
    G = fr.grid_size(recon, os_)
    train_trajs = [synth.radial_2d(96, 128), synth.golden_angle_2d(144, 128), synth.spiral_2d(8, 1024),
                   synth.spiral_2d(12, 768), synth.radial_2d(160, 96), synth.golden_angle_2d(80, 160)]
    feats, targets, weights = [], [], []
    for i, t in enumerate(train_trajs):
        plan, td = _plan_for(fr, torch, t, 2, G, W, os_)
        w = plan.dcf_pipe(20)
        feats.append(ld.dcf_features(plan, td))
        targets.append(torch.log(w) + ld.target_offset(plan.lut, plan.W, 2))
        weights.append(ld.energy_weight(t, 2, recon, w, seed=50 + i))
    X = torch.cat(feats)
    Y = torch.cat(targets)
    mean, std = X.mean(0), X.std(0) + 1e-6
    net = ld.DCFNet(seed=0)
    ld.train(net, (X - mean) / std, Y, torch.cat(weights), steps=3000, batch=8192, lr=3e-3)
    net.fold_input_scaling(mean.cpu().numpy(), std.cpu().numpy())

    rec = fr.Recon(2, recon, os_, 4)
    for t in (synth.golden_angle_2d(120, 128), synth.spiral_2d(10, 900)):
        plan, td = _plan_for(fr, torch, t, 2, G, W, os_)
        kd = torch.from_numpy(synth.kspace(t, 2, recon, 4, seed=11)).cuda()
        w_pipe = plan.dcf_pipe(20)
        w_net = ld.learned_dcf(plan, td, net)
        w_plain = fr.dcf_analytic(td, 2, 1.0)
        img_pipe = rec.run(td, w_pipe, kd).cpu().numpy()
        img_net = rec.run(td, w_net, kd).cpu().numpy()
        img_plain = rec.run(td, w_plain, kd).cpu().numpy()
        e_net, e_plain = _nrmse(img_net, img_pipe), _nrmse(img_plain, img_pipe)
        assert e_net < e_plain, (e_net, e_plain)
        assert e_net < 0.05, e_net
        # three Pipe-Menon iterations from the learned start come close to twenty from ones
        w_ref = ld.learned_dcf(plan, td, net, refine=3)
        w3 = plan.dcf_pipe(3)
        e_ref = _nrmse(rec.run(td, w_ref, kd).cpu().numpy(), img_pipe)
        e3 = _nrmse(rec.run(td, w3, kd).cpu().numpy(), img_pipe)
        assert e_ref < 0.02 and e_ref < e3, (e_ref, e3)


def test_kernel_mass_of_a_flat_kernel():
    from fastrecon_gb300 import learned_dcf as ld
    flat = np.ones(512, np.float32)
    assert abs(ld.kernel_mass(flat, 4.0, 2) - np.pi * 4.0) < 1e-6
    assert abs(ld.kernel_mass(flat, 4.0, 3) - 4.0 / 3.0 * np.pi * 8.0) < 1e-6
