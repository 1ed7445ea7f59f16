"""Generate the golden fixtures in tests/golden/ from the reference's own CPU
code (pengwg/fastrecon ReconData/GridLut/ConvKernel/ImageFilter sources,
compiled unmodified against stub headers into oracle/_ref/libfastrecon_ref.so
by oracle/build_oracle.py).

Run where the reference checkout exists:  python tests/golden/make_golden.py
Each case stores the seeded inputs and the reference outputs:
  traj (N,4) raw, dcf (N,), kdata (C,N) complex64,
  traj_norm (N,4)   ReconData::getTraj() after GridLut::plan
  grid (C,G^d)      GridLut::execute() channel images
  image (R^d,)      |ImageFilter::SOS| after fftExecute + fftShift
  lut (L,)          ConvKernel data
"""
from __future__ import annotations

import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fastrecon_gb300 import synth  # noqa: E402
from oracle import build_oracle  # noqa: E402
from oracle.pyoracle import RefLib  # noqa: E402

CASES = {
    # name: dim, traj kind, spokes/interleaves, readout, coils, recon, os, W, L, dcf power
    "radial2d_small": (2, "radial", 32, 64, 3, 32, 2.0, 4.0, 512, 1.0),
    "radial2d_oddgrid": (2, "radial", 24, 48, 2, 21, 1.5, 4.0, 512, 1.0),  # G = 31
    "aniso2d_w5": (2, "aniso", 20, 40, 2, 24, 1.5, 5.0, 32, 1.0),          # y beyond x range, W=5
    "spiral2d_w3": (2, "spiral", 6, 256, 3, 32, 2.0, 3.0, 64, 1.0),
    "koosh3d_small": (3, "koosh", 200, 32, 2, 20, 1.5, 4.0, 512, 2.0),     # G = 30
    "koosh3d_odd": (3, "koosh", 120, 24, 2, 14, 1.5, 4.0, 256, 2.0),       # G = 21
}
LUTS = [(4.0, 2.0, 512), (4.0, 1.5, 512), (4.0, 1.25, 512), (5.0, 2.0, 32), (3.0, 1.3, 64), (6.0, 2.0, 1024)]


def make_traj(kind, dim, a, b):
    if kind == "radial":
        return synth.radial_2d(a, b)
    if kind == "aniso":
        t = synth.golden_angle_2d(a, b)
        t[:, 0] *= 0.5
        return t
    if kind == "spiral":
        return synth.spiral_2d(a, b)
    return synth.kooshball_3d(a, b)


def main():
    build_oracle.build_oracle()
    if build_oracle.build_ref() is None:
        raise SystemExit("reference checkout not found; fixtures need the reference build")
    ref = RefLib()
    for name, (dim, kind, a, b, C, recon, os_, W, L, pw) in CASES.items():
        traj = make_traj(kind, dim, a, b)
        dcf = synth.ramp_dcf(traj, dim, pw)
        kd = synth.kspace(traj, dim, recon, C, seed=zlib.crc32(name.encode()) % 1000)
        grid, tn = ref.grid(traj, dcf, kd, b, a, dim, recon, os_, W, L, threads=2)
        rec = (recon, recon, recon if dim == 3 else 1)
        img = ref.recon(traj, dcf, kd, b, a, dim, recon, os_, W, L, rec, threads=2)
        img_pils = ref.recon_pils(traj, dcf, kd, b, a, dim, recon, os_, W, L, rec, threads=2)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), traj=traj, dcf=dcf, kdata=kd, traj_norm=tn,
                            grid=grid, image=img, image_pils=img_pils, lut=ref.kb_lut(W, os_, L),
                            params=np.array([dim, a, b, C, recon, os_, W, L, pw], np.float64))
        print(name, traj.shape, grid.shape, img.shape)
    luts = {f"w{w}_os{o}_l{l}": ref.kb_lut(w, o, l) for (w, o, l) in LUTS}
    np.savez_compressed(os.path.join(HERE, "luts.npz"), **luts)
    # PILS image operations (ImageFilter::lowFilter / normalize / SOS(map)) on random images
    rng = np.random.default_rng(7)
    pils = {}
    for dim, G in [(2, 40), (3, 12), (2, 31)]:
        x = (rng.standard_normal((3, G ** dim)) + 1j * rng.standard_normal((3, G ** dim))).astype(np.complex64)
        m = (rng.standard_normal((3, G ** dim)) + 1j * rng.standard_normal((3, G ** dim))).astype(np.complex64)
        rec = (G // 2, G // 2, G // 2 if dim == 3 else 1)
        key = f"d{dim}_g{G}"
        pils[key + "_in"] = x
        pils[key + "_map"] = m
        pils[key + "_low22"] = ref.pils_op(0, x, dim, G, 22)
        pils[key + "_low5"] = ref.pils_op(0, x, dim, G, 5)
        pils[key + "_norm"] = ref.pils_op(1, x, dim, G)
        pils[key + "_sosmap"] = ref.pils_op(2, x, dim, G, maps=m, recon=rec)
    np.savez_compressed(os.path.join(HERE, "pils_ops.npz"), **pils)


if __name__ == "__main__":
    main()
