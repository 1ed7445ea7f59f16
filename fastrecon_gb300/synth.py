"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (no scanner data ships with the reference).

Trajectories are sample-major ``Point<float>{x[4]}`` arrays (N, 4) in raw
k-space units, k in [-0.5, 0.5).  k-space data is the exact continuous
Fourier transform of a phantom made of Gaussian-profile ellipses
(ellipsoids in 3D) multiplied by smooth Gaussian coil sensitivities: the
product of Gaussians is a Gaussian, so the non-uniform DFT is analytic and
exact at any sample count.  Noise is complex Gaussian with standard
deviation ``noise`` times the RMS of the coil's noiseless data.

Everything works on numpy (CPU) or torch (any device) through ``xp``.
"""
from __future__ import annotations

import math

import numpy as np

GOLDEN_MEANS_3D = (0.4656, 0.6823)  # Chan et al., MRM 2009 multidimensional golden means


def radial_2d(spokes: int, readout: int) -> np.ndarray:
    """Uniform-angle radial: spoke j at theta = pi j / spokes, k_i = (i - R/2)/R."""
    th = np.pi * np.arange(spokes) / spokes
    k = (np.arange(readout) - readout / 2) / readout
    t = np.zeros((spokes * readout, 4), np.float32)
    t[:, 0] = (np.cos(th)[:, None] * k[None, :]).ravel()
    t[:, 1] = (np.sin(th)[:, None] * k[None, :]).ravel()
    return t


def golden_angle_2d(spokes: int, readout: int) -> np.ndarray:
    ga = np.pi * (np.sqrt(5) - 1) / 2
    th = (np.arange(spokes) * ga) % np.pi
    k = (np.arange(readout) - readout / 2) / readout
    t = np.zeros((spokes * readout, 4), np.float32)
    t[:, 0] = (np.cos(th)[:, None] * k[None, :]).ravel()
    t[:, 1] = (np.sin(th)[:, None] * k[None, :]).ravel()
    return t


def kooshball_3d(spokes: int, readout: int) -> np.ndarray:
    """3D radial with golden-means spoke directions: cos(polar) = (m phi1) mod 1,
    azimuth = 2 pi ((m phi2) mod 1); full-echo spokes k_i = (i - R/2)/R."""
    m = np.arange(spokes, dtype=np.float64)
    cz = (m * GOLDEN_MEANS_3D[0]) % 1.0
    az = 2 * np.pi * ((m * GOLDEN_MEANS_3D[1]) % 1.0)
    sz = np.sqrt(np.maximum(0.0, 1 - cz * cz))
    d = np.stack([sz * np.cos(az), sz * np.sin(az), cz], 1)
    k = (np.arange(readout) - readout / 2) / readout
    t = np.zeros((spokes * readout, 4), np.float32)
    t[:, :3] = (d[:, None, :] * k[None, :, None]).reshape(-1, 3)
    return t


def spiral_2d(interleaves: int, samples: int, density: float = 1.5, turns: float = 16.0,
              rotation: float = 0.0) -> np.ndarray:
    """Variable-density Archimedean-like spiral: r(t) = 0.5 t^density,
    theta(t) = 2 pi turns t, interleaves rotated uniformly."""
    tt = np.arange(samples) / samples
    r = 0.5 * tt ** density
    th0 = 2 * np.pi * turns * tt
    out = np.zeros((interleaves * samples, 4), np.float32)
    for i in range(interleaves):
        a = th0 + rotation + 2 * np.pi * i / interleaves
        out[i * samples:(i + 1) * samples, 0] = r * np.cos(a)
        out[i * samples:(i + 1) * samples, 1] = r * np.sin(a)
    return np.clip(out, -0.5, 0.4999999)


def ramp_dcf(traj: np.ndarray, dim: int, power: float = 1.0) -> np.ndarray:
    """|k|^power from the raw coordinates (|k| for 2D radial, |k|^2 for 3D)."""
    k = np.sqrt((traj[:, :dim].astype(np.float64) ** 2).sum(1))
    return (k ** power).astype(np.float32)


def phantom(dim: int, size: int, n_blobs: int = 10, seed: int = 0):
    """Random Gaussian-profile ellipse phantom.  Returns (amp, mu, cov) with
    mu/cov in pixel units of a size^dim field of view centred at 0."""
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.2, 1.0, n_blobs)
    mu = rng.uniform(-0.3, 0.3, (n_blobs, dim)) * size
    cov = np.zeros((n_blobs, dim, dim))
    for e in range(n_blobs):
        ax = rng.uniform(0.03, 0.18, dim) * size
        q, _ = np.linalg.qr(rng.standard_normal((dim, dim)))
        cov[e] = q @ np.diag(ax ** 2) @ q.T
    return amp, mu, cov


def coil_maps(dim: int, size: int, coils: int, seed: int = 0):
    """Smooth Gaussian-bump coil sensitivities around the field of view."""
    rng = np.random.default_rng(seed + 1000)
    centers = np.zeros((coils, dim))
    for c in range(coils):
        v = rng.standard_normal(dim)
        centers[c] = v / np.linalg.norm(v) * 0.6 * size
    sigma = np.full(coils, 0.5 * size)
    phase = rng.uniform(0, 2 * np.pi, coils)
    return centers, sigma, phase


def _gauss_products(amp, mu, cov, rho, sigma):
    """Each (ellipse x coil-bump) product as (A', mu', Sigma')."""
    out = []
    dim = mu.shape[1]
    eye = np.eye(dim)
    for a, m, S in zip(amp, mu, cov):
        P0 = np.linalg.inv(S)
        P = P0 + eye / sigma ** 2
        Sp = np.linalg.inv(P)
        mp = Sp @ (P0 @ m + rho / sigma ** 2)
        expo = -0.5 * (m @ P0 @ m + rho @ rho / sigma ** 2 - mp @ P @ mp)
        Ap = a * math.exp(expo) * (2 * math.pi) ** (dim / 2) * math.sqrt(np.linalg.det(Sp))
        out.append((Ap, mp, Sp))
    return out


def kspace(traj, dim: int, size: int, coils: int, seed: int = 0, noise: float = 0.01, xp=None, device=None,
           chunk: int = 1 << 22):
    """Exact k-space of the Gaussian-ellipse phantom times Gaussian coil maps at
    the trajectory points.  Returns (coils, N) complex64 (numpy, or torch on
    ``device`` when xp is torch)."""
    amp, mu, cov = phantom(dim, size, seed=seed)
    centers, sigma, phase = coil_maps(dim, size, coils, seed=seed)
    n = traj.shape[0]
    if xp is None:
        k = traj[:, :dim].astype(np.float64)
        out = np.zeros((coils, n), np.complex64)
        rng = np.random.default_rng(seed + 7)
        for c in range(coils):
            acc = np.zeros(n, np.complex128)
            for Ap, mp, Sp in _gauss_products(amp, mu, cov, centers[c], sigma[c]):
                quad = np.einsum("ni,ij,nj->n", k, Sp, k)
                acc += Ap * np.exp(-2 * math.pi ** 2 * quad - 2j * math.pi * (k @ mp))
            acc *= np.exp(1j * phase[c])
            if noise > 0:
                s = noise * np.sqrt(np.mean(np.abs(acc) ** 2)) / math.sqrt(2)
                acc += s * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
            out[c] = acc.astype(np.complex64)
        return out
    torch = xp
    kt = torch.as_tensor(np.ascontiguousarray(traj[:, :dim]), device=device).double()
    out = torch.empty((coils, n), dtype=torch.complex64, device=device)
    g = torch.Generator(device=device)
    g.manual_seed(seed + 7)
    for c in range(coils):
        prods = _gauss_products(amp, mu, cov, centers[c], sigma[c])
        for s0 in range(0, n, chunk):
            kk = kt[s0:s0 + chunk]
            acc = torch.zeros(kk.shape[0], dtype=torch.complex128, device=device)
            for Ap, mp, Sp in prods:
                Spt = torch.as_tensor(Sp, device=device)
                mpt = torch.as_tensor(mp, device=device)
                quad = ((kk @ Spt) * kk).sum(1)
                ph = -2 * math.pi * (kk @ mpt)
                acc += Ap * torch.exp(-2 * math.pi ** 2 * quad) * torch.polar(torch.ones_like(ph), ph)
            acc *= complex(math.cos(phase[c]), math.sin(phase[c]))
            out[c, s0:s0 + chunk] = acc.to(torch.complex64)
        if noise > 0:
            rms = out[c].abs().pow(2).mean().sqrt().item()
            s = noise * rms / math.sqrt(2)
            nr = torch.randn(n, generator=g, device=device) * s
            ni = torch.randn(n, generator=g, device=device) * s
            out[c] += torch.complex(nr, ni)
    return out


# --------------------------------------------------------------------------
# The benchmark configurations (sizes as the reference's use cases quote them)
# --------------------------------------------------------------------------
CONFIGS = {
    "radial2d": dict(dim=2, spokes=256, readout=512, coils=8, recon=256, os=2.0, width=4.0, dcf_power=1.0),
    "kooshball3d": dict(dim=3, spokes=50000, readout=256, coils=16, recon=256, os=1.5, width=4.0, dcf_power=2.0),
}


def make_case(dim: int, spokes: int, readout: int, coils: int, recon: int, os: float, width: float,
              dcf_power: float, seed: int = 0, xp=None, device=None, noise: float = 0.01):
    traj = radial_2d(spokes, readout) if dim == 2 else kooshball_3d(spokes, readout)
    dcf = ramp_dcf(traj, dim, dcf_power)
    data = kspace(traj, dim, recon, coils, seed=seed, noise=noise, xp=xp, device=device)
    return traj, dcf, data
