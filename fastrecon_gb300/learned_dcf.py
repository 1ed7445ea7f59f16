"""Learned density compensation on the device (no counterpart in the reference).

A 5 -> 64 -> 64 -> 1 tanh network maps sample-density features to log-DCF.
The features are the sample counts in boxes of radius 1, 2, 4 and 8 cells
around each sample (from the per-cell bin counts of the plan's normalised
trajectory) and log(|k| / max|k| + 1/1024).  Training weights each sample's
squared log-DCF error by (w^2 E)^(1/4), w its Pipe-Menon weight and E the
mean k-space energy of a synthetic object there, so that the fit is best
where DCF errors reach the image; the target is normalised by the kernel
mass (target_offset) so that grids of different oversampling agree.  The network is trained on Pipe-Menon weights
computed on the GPU (``GridPlan.dcf_pipe``); those weights remain its
fallback and the reference its images are compared with.

Every step runs in libfastrecon_gb300.so: fr_density_counts,
fr_dcf_features, fr_mlp_forward / fr_mlp_backward / fr_mlp_adam.  PyTorch
only holds device memory and draws mini-batch indices.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check
from .gridding import GridPlan, _ptr, _stream, _torch

RADII = (1, 2, 4, 8)
N_IN = 5
HIDDEN = 64
N_PARAMS = HIDDEN * N_IN + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1
OFF_W1, OFF_B1 = 0, HIDDEN * N_IN
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN * HIDDEN
OFF_W3 = OFF_B2 + HIDDEN
OFF_B3 = OFF_W3 + HIDDEN
FR_MLP_EXP = 1
FR_MLP_RESIDUAL = 2


def _radii_arg(radii):
    r = (C.c_int * len(radii))(*[int(v) for v in radii])
    return r, len(radii)


def density_counts(plan: GridPlan, radii=RADII, stream=None, out=None):
    """(n, len(radii)) int32: samples in the (2r+1)^d box around each sample's cell."""
    torch = _torch()
    if out is None:
        out = torch.empty((plan.n, len(radii)), dtype=torch.int32, device="cuda")
    r, nr = _radii_arg(radii)
    check(capi.load().fr_density_counts(plan.h, r, nr, _ptr(out), C.c_void_p(_stream(stream))), "fr_density_counts")
    return out


def dcf_features(plan: GridPlan, raw_traj, counts=None, radii=RADII, kmax: float = 0.0, stream=None, out=None):
    """(n, len(radii) + 1) float32 network inputs for the plan's trajectory."""
    torch = _torch()
    if counts is None:
        counts = density_counts(plan, radii, stream)
    raw_traj = raw_traj.contiguous()
    if out is None:
        out = torch.empty((plan.n, len(radii) + 1), dtype=torch.float32, device="cuda")
    r, nr = _radii_arg(radii)
    check(capi.load().fr_dcf_features(plan.h, _ptr(counts), _ptr(raw_traj), r, nr, float(kmax), _ptr(out),
                                      C.c_void_p(_stream(stream))), "fr_dcf_features")
    return out


class DCFNet:
    """The network's parameters (FP32 master + BF16 copy) and Adam state on the device."""

    def __init__(self, params=None, seed: int = 0, residual: bool = False):
        torch = _torch()
        self.lib = capi.load()
        # residual: the network is trained on log-DCF + feature 1 (log density
        # at radius 2), so that its output is nearly density-independent
        self.residual = bool(residual)
        if params is None:
            params = self.init_params(seed)
        self.master = torch.as_tensor(np.asarray(params, np.float32)).cuda().contiguous()
        self.bf16 = torch.empty(N_PARAMS, dtype=torch.bfloat16, device="cuda")
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.grad = torch.zeros_like(self.master)
        self.loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        self.step = 0
        self._ws = None
        self.refresh()

    @staticmethod
    def init_params(seed: int = 0) -> np.ndarray:
        rng = np.random.default_rng(seed)
        p = np.zeros(N_PARAMS, np.float32)
        p[OFF_W1:OFF_B1] = rng.standard_normal(HIDDEN * N_IN) * np.sqrt(1.0 / N_IN)
        p[OFF_W2:OFF_B2] = rng.standard_normal(HIDDEN * HIDDEN) * np.sqrt(1.0 / HIDDEN)
        p[OFF_W3:OFF_B3] = rng.standard_normal(HIDDEN) * np.sqrt(1.0 / HIDDEN)
        return p

    def refresh(self):
        check(self.lib.fr_mlp_to_bf16(_ptr(self.master), _ptr(self.bf16), N_PARAMS, None), "fr_mlp_to_bf16")

    def params_bf16_as_float(self) -> np.ndarray:
        return self.bf16.float().cpu().numpy()

    def forward(self, features, exp: bool = False, scale: float = 1.0, out=None, stream=None):
        """Network output per sample, or scale * exp(output) with exp=True."""
        torch = _torch()
        features = features.contiguous()
        n = features.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device="cuda")
        flags = (FR_MLP_EXP if exp else 0) | (FR_MLP_RESIDUAL if self.residual else 0)
        check(self.lib.fr_mlp_forward(_ptr(self.bf16), _ptr(features), n, flags, float(scale),
                                      _ptr(out), C.c_void_p(_stream(stream))), "fr_mlp_forward")
        return out

    def loss_grad(self, features, target, weight=None, stream=None):
        """(Weighted) mean squared error on the batch; the gradient lands in ``self.grad``."""
        torch = _torch()
        features = features.contiguous()
        target = target.contiguous()
        if weight is not None:
            weight = weight.contiguous()
        n = features.shape[0]
        need = int(self.lib.fr_mlp_workspace_bytes(n))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device="cuda")
        check(self.lib.fr_mlp_backward(_ptr(self.bf16), _ptr(features), _ptr(target),
                                       None if weight is None else _ptr(weight), n, _ptr(self._ws),
                                       _ptr(self.grad), _ptr(self.loss), C.c_void_p(_stream(stream))),
              "fr_mlp_backward")
        return self.loss

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, stream=None):
        self.step += 1
        check(self.lib.fr_mlp_adam(_ptr(self.master), _ptr(self.bf16), _ptr(self.grad), _ptr(self.m), _ptr(self.v),
                                   N_PARAMS, lr, beta1, beta2, eps, self.step, C.c_void_p(_stream(stream))),
              "fr_mlp_adam")

    def fold_input_scaling(self, mean, std):
        """Fold x -> (x - mean) / std into the first layer, so the network
        takes raw features."""
        p = self.master.cpu().numpy().astype(np.float64)
        w1 = p[OFF_W1:OFF_B1].reshape(HIDDEN, N_IN)
        b1 = p[OFF_B1:OFF_W2]
        mean = np.asarray(mean, np.float64)
        std = np.asarray(std, np.float64)
        w1n = w1 / std[None, :]
        b1n = b1 - w1n @ mean
        p[OFF_W1:OFF_B1] = w1n.ravel()
        p[OFF_B1:OFF_W2] = b1n
        self.master.copy_(_torch().from_numpy(p.astype(np.float32)))
        self.refresh()

    def save(self, path: str):
        np.savez(path, params=self.master.cpu().numpy(), residual=np.int32(self.residual))

    @classmethod
    def load(cls, path: str):
        z = np.load(path)
        return cls(z["params"], residual=bool(int(z["residual"])) if "residual" in z.files else False)


def energy_weight(traj, dim, recon, w_pipe, seed=0, power=0.25):
    """Loss weights (w^2 E)^power normalised to mean 1, with E the mean k-space
    energy over coils of a synthetic object (noise-free) at each sample."""
    from . import synth
    torch = _torch()
    kd = synth.kspace(traj, dim, recon, 4, seed=seed, noise=0.0, xp=torch, device="cuda")
    e = kd.abs().pow(2).mean(0)
    c = (w_pipe.double() ** 2 * e.double()).pow(power)
    return (c / c.mean()).float()


def kernel_mass(lut, kernel_width: float, dim: int, steps: int = 100000) -> float:
    """Integral of the radial LUT kernel over the plane (2D) or space (3D),
    with the gridding's LUT index rule: M = int K(|x|) d^d x."""
    lut = np.asarray(lut, np.float64)
    hw = kernel_width / 2
    r = (np.arange(steps) + 0.5) * (hw / steps)
    k = lut[np.minimum(np.rint(r / hw * (len(lut) - 1)).astype(np.int64), len(lut) - 1)]
    shell = 2 * np.pi * r if dim == 2 else 4 * np.pi * r * r
    return float(np.sum(k * shell) * (hw / steps))


def target_offset(lut, kernel_width: float, dim: int) -> float:
    """Pipe-Menon weights at density rho approach 1 / (rho M^2) (M the kernel
    mass), so log w + 2 log M depends on the samples' density alone: the
    network learns that normalised target and the DCF is exp(net) / M^2."""
    return 2.0 * float(np.log(kernel_mass(lut, kernel_width, dim)))


def learned_dcf(plan: GridPlan, raw_traj, net: DCFNet, kmax: float = 0.0, refine: int = 0, stream=None):
    """DCF of the plan's trajectory from the network; with refine > 0 the
    network's weights start that many Pipe-Menon iterations (the iterated DCF
    stays the reference: a few iterations from the learned start reach what
    20 from uniform weights do)."""
    feats = dcf_features(plan, raw_traj, kmax=kmax, stream=stream)
    scale = float(np.exp(-target_offset(plan.lut, plan.W, plan.dim)))
    w = net.forward(feats, exp=True, scale=scale, stream=stream)
    if refine > 0:
        check(capi.load().fr_dcf_pipe(plan.h, int(refine), _ptr(w), C.c_void_p(_stream(stream))), "fr_dcf_pipe")
    return w


def train(net: DCFNet, features, log_target, weight=None, steps: int = 2000, batch: int = 16384, lr: float = 3e-3,
          seed: int = 0, log_every: int = 0):
    """Adam with a cosine learning-rate schedule on mini-batches drawn from
    (features, log_target[, per-sample loss weight]) already on the device."""
    torch = _torch()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = features.shape[0]
    losses = []
    for it in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), device="cuda", generator=g)
        net.loss_grad(features[idx], log_target[idx], None if weight is None else weight[idx])
        step_lr = lr * 0.5 * (1 + np.cos(np.pi * it / steps))
        net.adam(lr=step_lr)
        if log_every and (it % log_every == 0 or it == steps - 1):
            losses.append((it, float(net.loss.item())))
    return losses
