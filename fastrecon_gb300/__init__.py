"""fastrecon_gb300: GB300 (sm_103a) non-Cartesian gridding / recon path behind
fastrecon's API.  Compute runs in libfastrecon_gb300.so (hand-written CUDA
kernels + cuFFT) through the C ABI in include/fastrecon_gb300.h."""
from .capi import FastreconError, load  # noqa: F401
from .gridding import (FFT, GridPlan, Recon, crop, dcf_analytic, fft_shift, grid_partitioned, grid_size,  # noqa: F401
                       kb_lut, kernel_launches, sos)

__all__ = ["FFT", "GridPlan", "Recon", "crop", "dcf_analytic", "fft_shift", "grid_partitioned", "grid_size", "kb_lut", "kernel_launches", "sos", "load",
           "FastreconError"]
