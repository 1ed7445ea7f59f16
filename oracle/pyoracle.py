"""ctypes bindings to the CPU oracle (test infrastructure only).

``Oracle`` wraps ``oracle/_build/liboracle.so`` (the plain-C restatement of
the reference CPU path); ``RefLib`` wraps ``oracle/_ref/libfastrecon_ref.so``
(the reference's own CPU sources compiled against stub headers), present
only where the reference checkout was available at build time.

Only tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline leg use
this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle as _b

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def cells_of(dim: int, G: int) -> int:
    return G ** 3 if dim == 3 else G ** 2


class Oracle:
    """The plain-C restatement (fr_oracle.c)."""

    def __init__(self, path: str | None = None):
        path = path or _b.build_oracle()
        lib = C.CDLL(path)
        self.lib = lib
        lib.orc_bessel_i0.restype = C.c_double
        lib.orc_bessel_i0.argtypes = [C.c_double]
        lib.orc_kb_lut.argtypes = [C.c_float, C.c_float, C.c_int, _f32p]
        lib.orc_comp_bounds.argtypes = [_f32p, C.c_size_t, C.c_int, _f32p, _f32p]
        lib.orc_normalize_traj.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, _f32p, _f32p,
                                           C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_sample_range.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, C.c_float, _i32p, _i32p]
        lib.orc_tap_lut_index.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]
        lib.orc_lut_index_of_s.argtypes = [_f32p, C.c_size_t, C.c_float, C.c_int, _i32p]
        lib.orc_grid_channel.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_uint,
                                         C.c_float, _f32p, C.c_int, _f32p]
        lib.orc_grid.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_int, C.c_uint,
                                 C.c_float, _f32p, C.c_int, _f32p, C.c_int]
        lib.orc_grid_channel_f64.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_uint,
                                             C.c_float, _f32p, C.c_int, _f64p]
        lib.orc_grid_bands.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_int, C.c_uint,
                                       C.c_float, _f32p, C.c_int, _f32p, C.c_int]
        lib.orc_grid_f64_bands.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_int, C.c_uint,
                                           C.c_float, _f32p, C.c_int, _f64p, C.c_int]
        lib.orc_sample_mass.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, C.c_float, _f32p, C.c_int, _f64p,
                                        C.c_int]
        lib.orc_sample_tiles.argtypes = [_i32p, _i32p, C.c_size_t, C.c_int, _i32p, _i32p, _i32p]
        lib.orc_fft.argtypes = [_f32p, C.c_int, _u32p, C.c_int, C.c_int, C.c_int]
        lib.orc_fft_shift.argtypes = [_f32p, C.c_int, _u32p]
        lib.orc_sos.argtypes = [_f32p, C.c_int, C.c_int, _u32p, _u32p, _f32p]
        lib.orc_low_filter.argtypes = [_f32p, C.c_int, C.c_int, _u32p, C.c_int]
        lib.orc_normalize_channels.argtypes = [_f32p, C.c_int, C.c_int, _u32p]
        lib.orc_sos_map.argtypes = [_f32p, _f32p, C.c_int, C.c_int, _u32p, _u32p, _f32p]
        lib.orc_recon.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, C.c_int, C.c_int, C.c_uint,
                                  C.c_float, C.c_float, C.c_int, _u32p, _f32p, C.c_int]

    # -- ConvKernel --------------------------------------------------------
    def kb_lut(self, W: float, os_: float, L: int) -> np.ndarray:
        out = np.zeros(L, np.float32)
        assert self.lib.orc_kb_lut(W, os_, L, out) == 0
        return out

    # -- ReconData ---------------------------------------------------------
    def comp_bounds(self, traj4: np.ndarray, dim: int):
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        self.lib.orc_comp_bounds(np.ascontiguousarray(traj4, np.float32), traj4.shape[0], dim, lo, hi)
        return lo[:dim].copy(), hi[:dim].copy()

    def normalize_traj(self, traj4: np.ndarray, dim: int, G: int):
        t = np.array(traj4, np.float32, copy=True, order="C")
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        self.lib.orc_comp_bounds(t, t.shape[0], dim, lo, hi)
        tr = C.c_float()
        sc = C.c_float()
        self.lib.orc_normalize_traj(t, t.shape[0], dim, G, lo, hi, C.byref(tr), C.byref(sc))
        return t, np.float32(tr.value), np.float32(sc.value), lo[:dim].copy(), hi[:dim].copy()

    # -- GridLut -----------------------------------------------------------
    def sample_range(self, traj_norm4: np.ndarray, dim: int, G: int, kHW: float):
        n = traj_norm4.shape[0]
        s = np.zeros(n * 3, np.int32)
        e = np.zeros(n * 3, np.int32)
        self.lib.orc_sample_range(np.ascontiguousarray(traj_norm4, np.float32), n, dim, G, kHW, s, e)
        return s.reshape(n, 3), e.reshape(n, 3)

    def sample_tiles(self, start: np.ndarray, end: np.ndarray, dim: int, tile_shape):
        n = start.shape[0]
        lo = np.zeros(n * 3, np.int32)
        hi = np.zeros(n * 3, np.int32)
        ts = np.array(list(tile_shape) + [1] * (3 - len(tile_shape)), np.int32)
        self.lib.orc_sample_tiles(np.ascontiguousarray(start, np.int32).ravel(),
                                  np.ascontiguousarray(end, np.int32).ravel(), n, dim, ts, lo, hi)
        return lo.reshape(n, 3), hi.reshape(n, 3)

    def sample_mass(self, traj_norm4, dim, G, W, lut, threads=1) -> np.ndarray:
        n = traj_norm4.shape[0]
        out = np.zeros(n, np.float64)
        self.lib.orc_sample_mass(np.ascontiguousarray(traj_norm4, np.float32), n, dim, G, W,
                                 np.ascontiguousarray(lut, np.float32), len(lut), out, threads)
        return out

    def lut_index_of_s(self, s, kHW, L) -> np.ndarray:
        s = np.ascontiguousarray(s, np.float32)
        out = np.zeros(s.shape[0], np.int32)
        self.lib.orc_lut_index_of_s(s, s.shape[0], kHW, L, out)
        return out

    def grid(self, traj_norm4, dcf, kdata, dim, G, W, lut, threads=1) -> np.ndarray:
        """kdata: (C, N) complex64; returns (C, G^d) complex64."""
        kd = np.ascontiguousarray(kdata, np.complex64)
        Cn, n = kd.shape
        out = np.zeros((Cn, cells_of(dim, G)), np.complex64)
        self.lib.orc_grid(np.ascontiguousarray(traj_norm4, np.float32), np.ascontiguousarray(dcf, np.float32),
                          kd.view(np.float32).ravel(), n, Cn, dim, G, W, np.ascontiguousarray(lut, np.float32),
                          len(lut), out.view(np.float32).ravel(), threads)
        return out

    def grid_bands(self, traj_norm4, dcf, kdata, dim, G, W, lut, threads=None) -> np.ndarray:
        """``grid`` with each channel split over threads by bands of the last
        axis: bit-for-bit the same result, for full-size checks."""
        threads = threads or os.cpu_count() or 1
        kd = np.ascontiguousarray(kdata, np.complex64)
        Cn, n = kd.shape
        out = np.empty((Cn, cells_of(dim, G)), np.complex64)
        self.lib.orc_grid_bands(np.ascontiguousarray(traj_norm4, np.float32), np.ascontiguousarray(dcf, np.float32),
                                kd.view(np.float32).ravel(), n, Cn, dim, G, W, np.ascontiguousarray(lut, np.float32),
                                len(lut), out.view(np.float32).ravel(), threads)
        return out

    def grid_f64_bands(self, traj_norm4, dcf, kdata, dim, G, W, lut, threads=None) -> np.ndarray:
        """``grid_f64`` split over threads by bands (bit-for-bit the same)."""
        threads = threads or os.cpu_count() or 1
        kd = np.ascontiguousarray(kdata, np.complex64)
        Cn, n = kd.shape
        out = np.empty((Cn, cells_of(dim, G)), np.complex128)
        self.lib.orc_grid_f64_bands(np.ascontiguousarray(traj_norm4, np.float32),
                                    np.ascontiguousarray(dcf, np.float32), kd.view(np.float32).ravel(), n, Cn, dim,
                                    G, W, np.ascontiguousarray(lut, np.float32), len(lut),
                                    out.view(np.float64).ravel(), threads)
        return out

    def recon_bands(self, traj4, dcf, kdata, dim, reconSize, os_, W, L, recon, threads=None) -> np.ndarray:
        """``recon`` (Program/Main.cpp:101-181 without I/O) with the gridding
        split over threads by bands: normalise, grid, backward FFT, fftShift,
        SOS, |.|.  Bit-for-bit the same image as ``recon``."""
        threads = threads or os.cpu_count() or 1
        G = int(np.float32(reconSize) * np.float32(os_))
        tn, _, _, _, _ = self.normalize_traj(traj4, dim, G)
        lut = self.kb_lut(W, os_, L)
        g = self.grid_bands(tn, dcf, kdata, dim, G, W, lut, threads)
        g = self.fft(g, dim, G, +1, threads)
        for c in range(g.shape[0]):
            g[c] = self.fft_shift(g[c], dim, G)
        return np.abs(self.sos(g, dim, G, recon).real).astype(np.float32)

    def grid_f64(self, traj_norm4, dcf, kdata, dim, G, W, lut) -> np.ndarray:
        kd = np.ascontiguousarray(kdata, np.complex64)
        Cn, n = kd.shape
        out = np.zeros((Cn, cells_of(dim, G)), np.complex128)
        for c in range(Cn):
            o = np.zeros(cells_of(dim, G) * 2, np.float64)
            self.lib.orc_grid_channel_f64(np.ascontiguousarray(traj_norm4, np.float32),
                                          np.ascontiguousarray(dcf, np.float32),
                                          np.ascontiguousarray(kd[c]).view(np.float32), n, dim, G, W,
                                          np.ascontiguousarray(lut, np.float32), len(lut), o)
            out[c] = o.view(np.complex128)
        return out

    # -- ImageFilter -------------------------------------------------------
    def fft(self, imgs: np.ndarray, dim: int, G: int, sign: int = +1, threads: int = 1) -> np.ndarray:
        a = np.array(imgs, np.complex64, copy=True, order="C")
        batch = a.shape[0] if a.ndim > 1 else 1
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        self.lib.orc_fft(a.view(np.float32).ravel(), dim, size, batch, sign, threads)
        return a

    def fft_shift(self, img: np.ndarray, dim: int, G: int) -> np.ndarray:
        a = np.array(img, np.complex64, copy=True, order="C")
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        self.lib.orc_fft_shift(a.view(np.float32).ravel(), dim, size)
        return a

    def fft_shift_inplace(self, img: np.ndarray, dim: int, G: int) -> None:
        """``fft_shift`` on a contiguous complex64 array, in place."""
        assert img.dtype == np.complex64 and img.flags.c_contiguous
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        self.lib.orc_fft_shift(img.reshape(-1).view(np.float32), dim, size)

    def sos(self, imgs: np.ndarray, dim: int, G: int, recon) -> np.ndarray:
        a = np.ascontiguousarray(imgs, np.complex64)
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.complex64)
        self.lib.orc_sos(a.view(np.float32).ravel(), a.shape[0], dim, size, rec, out.view(np.float32))
        return out

    def low_filter(self, imgs, dim, G, res):
        a = np.array(imgs, np.complex64, copy=True, order="C")
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        self.lib.orc_low_filter(a.view(np.float32).ravel(), a.shape[0], dim, size, res)
        return a

    def normalize_channels(self, imgs, dim, G):
        a = np.array(imgs, np.complex64, copy=True, order="C")
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        self.lib.orc_normalize_channels(a.view(np.float32).ravel(), a.shape[0], dim, size)
        return a

    def sos_map(self, imgs, maps, dim, G, recon):
        a = np.ascontiguousarray(imgs, np.complex64)
        m = np.ascontiguousarray(maps, np.complex64)
        size = np.array([G, G, G if dim == 3 else 1], np.uint32)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.complex64)
        self.lib.orc_sos_map(a.view(np.float32).ravel(), m.view(np.float32).ravel(), a.shape[0], dim, size, rec,
                             out.view(np.float32))
        return out

    def recon(self, traj4, dcf, kdata, dim, reconSize, os_, W, L, recon, threads=1) -> np.ndarray:
        t = np.array(traj4, np.float32, copy=True, order="C")
        kd = np.ascontiguousarray(kdata, np.complex64)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.float32)
        rc = self.lib.orc_recon(t, np.ascontiguousarray(dcf, np.float32), kd.view(np.float32).ravel(),
                                t.shape[0], kd.shape[0], dim, reconSize, os_, W, L, rec, out, threads)
        assert rc == 0
        return out

    # -- components with no reference counterpart ---------------------------
    def deapod_map_f64(self, dim, G, W, lut, recon) -> np.ndarray:
        """Deapodization map in FP64 (no counterpart in the reference, which
        does not deapodize).  The kernel's taps around the grid centre
        c0 = G/2 -- offsets d with dk = |d| < W/2 and weight lut[ki], the
        reference geometry and LUT index (GridLut.cpp:120-136) -- are
        transformed to the image: after the backward FFT and fftShift,
        pixel p holds sum_d w(d) e^{2 pi i (c0 + d).(p - G/2) / G}, whose
        modulus is |sum_d w(d) cos(2 pi d.(p - G/2) / G)| (the tap set is
        symmetric).  The map is that modulus over the centred crop (offset
        (G - R)/2 per axis), divided by its value at the centre pixel,
        floored at 1e-6.  Returns recon-size float64, x fastest."""
        hw = np.float32(W) / np.float32(2)
        reach = int(np.ceil(hw)) + 1
        taps = []
        rng = range(-reach, reach + 1)
        for dz in (rng if dim == 3 else [0]):
            for dy in rng:
                for dx in rng:
                    ki = self.lib.orc_tap_lut_index(float(dx), float(dy), float(dz), float(hw), len(lut))
                    if ki >= 0:
                        taps.append((dx, dy, dz, float(lut[ki])))
        t = np.array(taps, np.float64)
        R = list(recon) + [1] * (3 - len(recon))
        off = [(G - R[0]) // 2, (G - R[1]) // 2, (G - R[2]) // 2 if dim == 3 else 0]
        ax = [2 * np.pi * (np.arange(R[i]) + off[i] - (G // 2 if i < dim else 0)) / G for i in range(3)]
        out = np.zeros((R[2], R[1], R[0]), np.float64)
        for dx, dy, dz, w in t:
            ph = dz * ax[2][:, None, None] + dy * ax[1][None, :, None] + dx * ax[0][None, None, :]
            out += w * np.cos(ph)
        m = np.abs(out) / t[:, 3].sum()
        return np.maximum(m, 1e-6).ravel()

    # -- components with no reference counterpart (fr_oracle_ext.c) ---------
    MLP_IN, MLP_HIDDEN = 5, 64
    MLP_PARAMS = 64 * 5 + 64 + 64 * 64 + 64 + 64 + 1

    def _ext_sigs(self):
        lib = self.lib
        if getattr(self, "_ext", False):
            return lib
        lib.orc_dcf_analytic.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_double, _f32p]
        lib.orc_degrid_f64.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, C.c_float, _f32p, C.c_int, _f64p,
                                       C.c_int, _f64p]
        lib.orc_grid_real_f64.argtypes = [_f32p, _f64p, C.c_size_t, C.c_int, C.c_uint, C.c_float, _f32p, C.c_int,
                                          _f64p]
        lib.orc_dcf_pipe_f64.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, C.c_float, _f32p, C.c_int, C.c_int,
                                         _f64p]
        lib.orc_density_counts.argtypes = [_f32p, C.c_size_t, C.c_int, C.c_uint, _i32p, C.c_int, _i32p]
        lib.orc_dcf_features.argtypes = [_i32p, _f32p, C.c_size_t, C.c_int, _i32p, C.c_int, C.c_float, _f32p]
        lib.orc_mlp_forward.argtypes = [_f32p, _f32p, C.c_size_t, _f64p]
        lib.orc_mlp_forward_residual.argtypes = [_f32p, _f32p, C.c_size_t, _f64p]
        lib.orc_mlp_backward.argtypes = [_f32p, _f32p, _f32p, C.c_void_p, C.c_size_t, _f64p]
        lib.orc_mlp_backward.restype = C.c_double
        self._ext = True
        return lib

    def dcf_analytic(self, traj4, dim, power):
        t = np.ascontiguousarray(traj4, np.float32)
        out = np.zeros(t.shape[0], np.float32)
        self._ext_sigs().orc_dcf_analytic(t, t.shape[0], dim, float(power), out)
        return out

    def degrid_f64(self, traj_norm4, grid, dim, G, W, lut):
        t = np.ascontiguousarray(traj_norm4, np.float32)
        g = np.ascontiguousarray(grid, np.complex128).reshape(-1, cells_of(dim, G))
        out = np.zeros((g.shape[0], t.shape[0]), np.complex128)
        self._ext_sigs().orc_degrid_f64(t, t.shape[0], dim, G, W, np.ascontiguousarray(lut, np.float32), len(lut),
                                        g.view(np.float64).ravel(), g.shape[0], out.view(np.float64).ravel())
        return out

    def grid_real_f64(self, traj_norm4, w, dim, G, W, lut):
        t = np.ascontiguousarray(traj_norm4, np.float32)
        out = np.zeros(cells_of(dim, G), np.float64)
        self._ext_sigs().orc_grid_real_f64(t, np.ascontiguousarray(w, np.float64), t.shape[0], dim, G, W,
                                           np.ascontiguousarray(lut, np.float32), len(lut), out)
        return out

    def dcf_pipe_f64(self, traj_norm4, dim, G, W, lut, iterations, w0=None):
        t = np.ascontiguousarray(traj_norm4, np.float32)
        w = np.ones(t.shape[0], np.float64) if w0 is None else np.array(w0, np.float64, copy=True)
        rc = self._ext_sigs().orc_dcf_pipe_f64(t, t.shape[0], dim, G, W, np.ascontiguousarray(lut, np.float32),
                                               len(lut), iterations, w)
        assert rc == 0
        return w

    def density_counts(self, traj_norm4, dim, G, radii):
        t = np.ascontiguousarray(traj_norm4, np.float32)
        r = np.ascontiguousarray(radii, np.int32)
        out = np.zeros((t.shape[0], len(r)), np.int32)
        assert self._ext_sigs().orc_density_counts(t, t.shape[0], dim, G, r, len(r), out) == 0
        return out

    def dcf_features(self, counts, raw_traj4, dim, radii, kmax):
        c = np.ascontiguousarray(counts, np.int32)
        r = np.ascontiguousarray(radii, np.int32)
        out = np.zeros((c.shape[0], len(r) + 1), np.float32)
        self._ext_sigs().orc_dcf_features(c, np.ascontiguousarray(raw_traj4, np.float32), c.shape[0], dim, r, len(r),
                                          float(kmax), out)
        return out

    def mlp_forward(self, params, x, residual=False):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros(x.shape[0], np.float64)
        fn = self._ext_sigs().orc_mlp_forward_residual if residual else self._ext_sigs().orc_mlp_forward
        fn(np.ascontiguousarray(params, np.float32), x, x.shape[0], out)
        return out

    def mlp_backward(self, params, x, target, weight=None):
        x = np.ascontiguousarray(x, np.float32)
        g = np.zeros(self.MLP_PARAMS, np.float64)
        w = None if weight is None else np.ascontiguousarray(weight, np.float32)
        loss = self._ext_sigs().orc_mlp_backward(np.ascontiguousarray(params, np.float32), x,
                                                 np.ascontiguousarray(target, np.float32),
                                                 None if w is None else w.ctypes.data, x.shape[0], g)
        return loss, g


class RefLib:
    """The reference's own CPU sources, compiled with stub headers."""

    def __init__(self, path: str | None = None):
        path = path or _b.ref_lib_path()
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        self.lib = lib
        lib.ref_kb_lut.argtypes = [C.c_float, C.c_float, C.c_int, _f32p]
        lib.ref_grid.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                 C.c_float, C.c_float, C.c_uint, C.c_int, _f32p, _f32p]
        lib.ref_shift_sos.argtypes = [_f32p, C.c_int, C.c_int, C.c_uint, _u32p, _f32p]
        lib.ref_pils_op.argtypes = [C.c_int, _f32p, C.c_void_p, C.c_int, C.c_int, C.c_uint, C.c_int, _u32p,
                                    C.c_void_p]
        lib.ref_recon_pils.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                       C.c_float, C.c_float, C.c_uint, C.c_int, _u32p, _f32p]
        lib.ref_recon.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                  C.c_float, C.c_float, C.c_uint, C.c_int, _u32p, _f32p]

    @staticmethod
    def available() -> bool:
        return os.path.exists(_b.ref_lib_path())

    def kb_lut(self, W, os_, L):
        out = np.zeros(L, np.float32)
        self.lib.ref_kb_lut(W, os_, L, out)
        return out

    def grid(self, traj4, dcf, kdata, samples, acquisitions, dim, reconSize, os_, W, L, threads=1):
        kd = np.ascontiguousarray(kdata, np.complex64)
        G = int(np.float32(reconSize) * np.float32(os_))
        out = np.zeros((kd.shape[0], cells_of(dim, G)), np.complex64)
        tn = np.zeros((traj4.shape[0], 4), np.float32)
        self.lib.ref_grid(np.ascontiguousarray(traj4, np.float32), np.ascontiguousarray(dcf, np.float32),
                          kd.view(np.float32).ravel(), samples, acquisitions, dim, kd.shape[0], reconSize,
                          os_, W, L, threads, out.view(np.float32).ravel(), tn)
        return out, tn

    def shift_sos(self, imgs, dim, G, recon):
        a = np.ascontiguousarray(imgs, np.complex64)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.complex64)
        self.lib.ref_shift_sos(a.view(np.float32).ravel(), a.shape[0], dim, G, rec, out.view(np.float32))
        return out

    def pils_op(self, op, imgs, dim, G, res=22, maps=None, recon=(1, 1, 1)):
        a = np.array(imgs, np.complex64, copy=True, order="C")
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.complex64)
        m = np.ascontiguousarray(maps, np.complex64) if maps is not None else None
        self.lib.ref_pils_op(op, a.view(np.float32).ravel(), m.ctypes.data if m is not None else None, a.shape[0],
                             dim, G, res, rec, out.ctypes.data)
        return out if op == 2 else a

    def recon_pils(self, traj4, dcf, kdata, samples, acquisitions, dim, reconSize, os_, W, L, recon, threads=1):
        kd = np.ascontiguousarray(kdata, np.complex64)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.float32)
        self.lib.ref_recon_pils(np.ascontiguousarray(traj4, np.float32), np.ascontiguousarray(dcf, np.float32),
                                kd.view(np.float32).ravel(), samples, acquisitions, dim, kd.shape[0], reconSize,
                                os_, W, L, threads, rec, out)
        return out

    def recon(self, traj4, dcf, kdata, samples, acquisitions, dim, reconSize, os_, W, L, recon, threads=1):
        kd = np.ascontiguousarray(kdata, np.complex64)
        rec = np.array(recon, np.uint32)
        out = np.zeros(int(np.prod(rec)), np.float32)
        self.lib.ref_recon(np.ascontiguousarray(traj4, np.float32), np.ascontiguousarray(dcf, np.float32),
                           kd.view(np.float32).ravel(), samples, acquisitions, dim, kd.shape[0], reconSize,
                           os_, W, L, threads, rec, out)
        return out
