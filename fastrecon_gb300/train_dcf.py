"""Train the learned-DCF network on the GPU (no counterpart in the reference).

    python -m fastrecon_gb300.train_dcf --dim 3 --trajectories 1000 \\
        --out fastrecon_gb300/models/dcf_mlp_3d.npz

Training data: seeded trajectories of the radial, golden-angle radial and
variable-density spiral families (2D) or golden-means 3D radial (3D), 10 k
to 2 M samples each, on grids of oversampling 1.25-2.  Targets: log of the
Pipe-Menon DCF (20 grid/degrid iterations, FP32, fr_dcf_pipe), each sample's
squared error weighted by (w^2 E)^(1/4) (learned_dcf.energy_weight).  Inputs:
density counts at radii 1, 2, 4, 8 cells and |k| (fr_dcf_features).  The
forward/backward/Adam steps are the library's kernels (fr_mlp_*).
Evaluation on held-out trajectories reports the image NRMSE of the learned-
DCF recon and of the plain |k|^p DCF recon against the Pipe-DCF recon.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import gridding as G_
from . import learned_dcf as ld
from . import synth

HERE = os.path.dirname(os.path.abspath(__file__))
MODELS = os.path.join(HERE, "models")
PIPE_ITERS = 20
REFINE = 3  # Pipe-Menon iterations started from the learned DCF


def model_path(dim: int) -> str:
    return os.path.join(MODELS, f"dcf_mlp_{dim}d.npz")


def draw_trajectory(dim: int, rng, n_min=10_000, n_max=2_000_000):
    """(raw trajectory, recon size, oversampling, family name) drawn from the families."""
    n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
    os_ = float(rng.choice([1.25, 1.5, 2.0]))
    if dim == 3:
        # matrix sizes independent of the readout, so that the sample density
        # per grid cell spans sparse to dense (up to ~10 samples per cell)
        readout = int(rng.choice([64, 96, 128, 192, 256]))
        recon = int(rng.choice([48, 64, 96, 128, 160, 192]))
        spokes = max(n // readout, 16)
        return synth.kooshball_3d(spokes, readout), recon, os_, "koosh3d"
    fam = rng.integers(0, 3)
    readout = int(rng.choice([128, 192, 256, 384, 512, 768, 1024]))
    spokes = max(n // readout, 8)
    recon = int(min(max(readout // 2, 32), 384))
    if fam == 0:
        return synth.radial_2d(spokes, readout), recon, os_, "radial2d"
    if fam == 1:
        return synth.golden_angle_2d(spokes, readout), recon, os_, "golden2d"
    samples = readout * 4
    inter = max(n // samples, 2)
    dens = float(rng.uniform(1.0, 2.5))
    turns = float(rng.uniform(4.0, 24.0))
    return synth.spiral_2d(inter, samples, density=dens, turns=turns), recon, os_, "spiral2d"


def pipe_and_features(t, dim, recon, os_, W=4.0):
    torch = G_._torch()
    Gs = G_.grid_size(recon, os_)
    plan = G_.GridPlan(dim, Gs, W, overgrid_factor=os_)
    td = torch.from_numpy(t).cuda()
    plan.set_trajectory(td)
    w = plan.dcf_pipe(PIPE_ITERS)
    x = ld.dcf_features(plan, td)
    return plan, td, w, x


def nrmse(a, ref):
    """Relative RMS difference after the best scalar scaling of a onto ref."""
    a = a.double().flatten()
    ref = ref.double().flatten()
    c = (a @ ref) / (a @ a)
    return float((c * a - ref).norm() / ref.norm())


def evaluate(net, dim, trajs, coils=4, seed=100):
    torch = G_._torch()
    out = []
    for i, (t, recon, os_, fam) in enumerate(trajs):
        plan, td, w_pipe, x = pipe_and_features(t, dim, recon, os_)
        w_net = net.forward(x, exp=True, scale=math.exp(-ld.target_offset(plan.lut, plan.W, dim)))
        w_ref = plan.dcf_pipe(REFINE, w0=w_net)
        w_plain = G_.dcf_analytic(td, dim, 1.0 if dim == 2 else 2.0)
        kd = synth.kspace(t, dim, recon, coils, seed=seed + i, xp=torch, device="cuda")
        rec = G_.Recon(dim, recon, os_, coils)
        img_pipe = rec.run(td, w_pipe, kd)
        e_net = nrmse(rec.run(td, w_net, kd), img_pipe)
        e_ref = nrmse(rec.run(td, w_ref, kd), img_pipe)
        e_plain = nrmse(rec.run(td, w_plain, kd), img_pipe)
        out.append(dict(family=fam, samples=int(t.shape[0]), recon=recon, os=os_, nrmse_learned=e_net,
                        nrmse_learned_refined=e_ref, nrmse_plain=e_plain))
        del rec
    return out


def build_dataset(dim, n_traj, seed, per_traj=20000, residual=False):
    torch = G_._torch()
    rng = np.random.default_rng(seed)
    X, Y, C = [], [], []
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    for i in range(n_traj):
        t, recon, os_, _fam = draw_trajectory(dim, rng)
        plan, _, w, x = pipe_and_features(t, dim, recon, os_)
        c = ld.energy_weight(t, dim, recon, w, seed=seed * 100003 + i)
        n = t.shape[0]
        idx = torch.randint(0, n, (min(per_traj, n),), device="cuda", generator=g)
        X.append(x[idx])
        Y.append(torch.log(w[idx]) + ld.target_offset(plan.lut, plan.W, dim) + (x[idx, 1] if residual else 0))
        C.append(c[idx])
    return torch.cat(X), torch.cat(Y), torch.cat(C)


def summarise(ev):
    """Median and 10/90th percentiles of each NRMSE column, per family and overall."""
    out = {}
    fams = sorted({e["family"] for e in ev})
    for key in ("nrmse_learned", "nrmse_learned_refined", "nrmse_plain"):
        v = np.array([e[key] for e in ev])
        out[key] = dict(median=float(np.median(v)), p10=float(np.percentile(v, 10)), p90=float(np.percentile(v, 90)),
                        below_1pct=int((v <= 0.01).sum()))
        for f in fams:
            vf = np.array([e[key] for e in ev if e["family"] == f])
            out[key][f] = dict(n=int(vf.size), median=float(np.median(vf)))
    out["learned_beats_plain"] = int(sum(e["nrmse_learned"] < e["nrmse_plain"] for e in ev))
    out["trajectories"] = len(ev)
    return out


def eval_saved(a):
    """Held-out evaluation of the saved network (the draw continues the
    training run's held-out sequence: its first trajectories are the ones the
    training report used)."""
    path = a.out or model_path(a.dim)
    net = ld.DCFNet.load(path)
    rng = np.random.default_rng(a.seed + 12345)
    held = [draw_trajectory(a.dim, rng, n_max=a.max_samples) for _ in range(a.held_out)]
    ev = evaluate(net, a.dim, held)
    rep_path = os.path.splitext(path)[0] + ".json"
    rep = json.load(open(rep_path)) if os.path.exists(rep_path) else {}
    rep["held_out_eval"] = dict(trajectories=len(ev), summary=summarise(ev), cases=ev)
    with open(rep_path, "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep["held_out_eval"]["summary"]))
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--dim", type=int, default=2, choices=(2, 3))
    ap.add_argument("--trajectories", type=int, default=1000)
    ap.add_argument("--held-out", type=int, default=12)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--max-samples", type=int, default=2_000_000)
    ap.add_argument("--out", default=None)
    ap.add_argument("--residual", action="store_true",
                    help="train on log-DCF + log density (radius 2): nearly density-independent targets")
    ap.add_argument("--eval-only", action="store_true",
                    help="evaluate the saved model on --held-out trajectories and add the result to its report")
    a = ap.parse_args(argv)
    torch = G_._torch()
    if a.eval_only:
        return eval_saved(a)
    t0 = time.time()
    X, Y, Cw = build_dataset(a.dim, a.trajectories, a.seed, residual=a.residual)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    mean, std = X.mean(0), X.std(0) + 1e-6
    net = ld.DCFNet(seed=a.seed, residual=a.residual)
    t1 = time.time()
    losses = ld.train(net, (X - mean) / std, Y, Cw, steps=a.steps, batch=a.batch, lr=a.lr, seed=a.seed,
                      log_every=max(a.steps // 10, 1))
    torch.cuda.synchronize()
    t_train = time.time() - t1
    net.fold_input_scaling(mean.cpu().numpy(), std.cpu().numpy())
    rng = np.random.default_rng(a.seed + 12345)
    held = [draw_trajectory(a.dim, rng, n_max=a.max_samples) for _ in range(a.held_out)]
    ev = evaluate(net, a.dim, held)
    out = a.out or model_path(a.dim)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    net.save(out)
    rep = dict(dim=a.dim, residual=a.residual, trajectories=a.trajectories, samples=int(X.shape[0]), dataset_s=round(t_data, 1),
               train_s=round(t_train, 1), steps=a.steps, batch=a.batch, losses=losses,
               held_out=ev, median_nrmse_learned=float(np.median([e["nrmse_learned"] for e in ev])),
               median_nrmse_learned_refined=float(np.median([e["nrmse_learned_refined"] for e in ev])),
               median_nrmse_plain=float(np.median([e["nrmse_plain"] for e in ev])), model=out)
    print(json.dumps(rep))
    return rep


if __name__ == "__main__":
    main()
