"""Python mirror of the gridding / recon path over the C ABI, on torch CUDA
tensors (torch provides device memory and streams only; all compute is the
library's).

Names follow the reference (ReconData/GridLut.h, ConvKernel.h,
ImageFilter/ImageFilter.h): ``kb_lut`` is ConvKernel, ``GridPlan`` is
GridLut::plan/execute, ``fft``/``fft_shift``/``sos``/``crop`` are the
ImageFilter operations, ``Recon`` is the Program/Main.cpp pipeline.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, u3


def _torch():
    import torch
    return torch


def _stream(stream):
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def kb_lut(kernel_width: float, overgrid_factor: float, length: int) -> np.ndarray:
    """ConvKernel(kWidth, overGridFactor, length).getKernelData() (ConvKernel.cpp:7-30)."""
    lib = capi.load()
    out = (C.c_float * length)()
    check(lib.fr_kb_lut(kernel_width, overgrid_factor, length, out), "fr_kb_lut")
    return np.frombuffer(out, np.float32).copy()


def kernel_launches() -> int:
    """Kernels launched by the library so far in this process."""
    return int(capi.load().fr_kernel_launches())


def grid_size(recon_size: int, overgrid_factor: float) -> int:
    """GridLut.cpp:45: unsigned(reconSize * overGridFactor) in float."""
    return int(np.float32(recon_size) * np.float32(overgrid_factor))


def _plan_desc(dim, grid_size, kernel_width, lut, tile, coil_group, chunk, checkerboard, tap_lists,
               deterministic=False):
    """fr_plan_desc over ``lut`` (a float32 array the caller keeps alive)."""
    d = capi.PlanDesc()
    d.dim = dim
    d.grid_size = grid_size
    d.kernel_width = kernel_width
    d.lut_length = len(lut)
    d.lut = lut.ctypes.data_as(C.POINTER(C.c_float))
    for i in range(3):
        d.tile[i] = int(tile[i]) if i < len(tile) else 0
    d.coil_group = coil_group
    d.chunk = chunk
    d.flags = ((capi.FR_PLAN_CHECKERBOARD if checkerboard else 0) | (0 if tap_lists else capi.FR_PLAN_NO_TAP_LISTS) |
               (capi.FR_PLAN_DETERMINISTIC if deterministic else 0))
    return d


class GridPlan:
    """GridLut::plan + execute on the device.

    ``set_trajectory`` normalises (ReconData::normalizeTraj) and bins;
    ``grid`` grids all channels (cuGridLut::execute)."""

    def __init__(self, dim: int, grid_size: int, kernel_width: float = 4.0, lut=None, lut_length: int = 512,
                 overgrid_factor: float = 2.0, tile=(0, 0, 0), coil_group: int = 0, chunk: int = 0,
                 checkerboard: bool = False, tap_lists: bool = True, deterministic: bool = False):
        self.lib = capi.load()
        if lut is None:
            lut = kb_lut(kernel_width, overgrid_factor, lut_length)
        self.lut = np.ascontiguousarray(lut, np.float32)
        d = _plan_desc(dim, grid_size, kernel_width, self.lut, tile, coil_group, chunk, checkerboard, tap_lists,
                       deterministic)
        h = C.c_void_p()
        check(self.lib.fr_plan_create(C.byref(d), C.byref(h)), "fr_plan_create")
        self.h = h
        self.dim, self.G, self.n = dim, grid_size, 0
        self.W = kernel_width

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fr_plan_destroy(self.h)
            self.h = None

    @property
    def cells(self) -> int:
        return self.G ** self.dim

    def set_trajectory(self, traj, stream=None):
        assert traj.is_cuda and traj.dtype == _torch().float32 and traj.shape[-1] == 4
        traj = traj.contiguous()
        self._traj_keep = traj
        check(self.lib.fr_plan_set_trajectory(self.h, _ptr(traj), traj.shape[0], C.c_void_p(_stream(stream))),
              "fr_plan_set_trajectory")
        self.n = traj.shape[0]

    def normalized_trajectory(self, stream=None):
        torch = _torch()
        out = torch.empty((self.n, 4), dtype=torch.float32, device="cuda")
        check(self.lib.fr_plan_normalized_trajectory(self.h, _ptr(out), C.c_void_p(_stream(stream))),
              "fr_plan_normalized_trajectory")
        return out

    def bounds(self):
        a = [(C.c_float * 3)() for _ in range(4)]
        check(self.lib.fr_plan_bounds(self.h, *a), "fr_plan_bounds")
        return [np.frombuffer(x, np.float32)[:self.dim].copy() for x in a]

    def sample_ranges(self, stream=None):
        torch = _torch()
        s = torch.empty((self.n, 3), dtype=torch.int32, device="cuda")
        e = torch.empty((self.n, 3), dtype=torch.int32, device="cuda")
        check(self.lib.fr_plan_sample_ranges(self.h, _ptr(s), _ptr(e), C.c_void_p(_stream(stream))),
              "fr_plan_sample_ranges")
        return s, e

    def stats(self):
        v = [C.c_longlong() for _ in range(4)]
        check(self.lib.fr_plan_stats(self.h, *[C.byref(x) for x in v]), "fr_plan_stats")
        return dict(tiles=v[0].value, pairs=v[1].value, items=v[2].value, slots=v[3].value)

    def tap_words(self) -> int:
        """4-byte words per sample of the plan's tap lists (0: none)."""
        q = C.c_int()
        check(self.lib.fr_plan_tap_words(self.h, C.byref(q)), "fr_plan_tap_words")
        return q.value

    def bins(self, stream=None):
        torch = _torch()
        st = self.stats()
        off = torch.empty(st["tiles"] + 1, dtype=torch.int64, device="cuda")
        pairs = torch.empty(max(st["pairs"], 1), dtype=torch.int32, device="cuda")
        check(self.lib.fr_plan_bins(self.h, _ptr(off), _ptr(pairs), C.c_void_p(_stream(stream))), "fr_plan_bins")
        return off, pairs[:st["pairs"]]

    def profile(self, enable: bool = True):
        """Record CUDA events around the tile scatter kernel of every grid call."""
        check(self.lib.fr_plan_profile(self.h, 1 if enable else 0), "fr_plan_profile")

    def profile_read(self):
        """(total ms, launches) of the scatter kernel since the last read."""
        ms = C.c_double()
        k = C.c_int()
        check(self.lib.fr_plan_profile_read(self.h, C.byref(ms), C.byref(k)), "fr_plan_profile_read")
        return ms.value, k.value

    def grid(self, kdata, dcf, out=None, stream=None):
        """kdata: (C, N) complex64 CUDA; dcf: (N,) float32 CUDA -> (C, G^d) complex64."""
        torch = _torch()
        assert kdata.dtype == torch.complex64 and kdata.is_cuda and dcf.is_cuda
        kdata = kdata.contiguous()
        dcf = dcf.contiguous()
        ch = kdata.shape[0]
        if out is None:
            out = torch.empty((ch, self.cells), dtype=torch.complex64, device="cuda")
        check(self.lib.fr_grid(self.h, _ptr(kdata), _ptr(dcf), ch, _ptr(out), C.c_void_p(_stream(stream))),
              "fr_grid")
        return out

    def degrid(self, grid, out=None, stream=None):
        """grid: (C, G^d) complex64 CUDA -> (C, N) complex64 samples (adjoint of ``grid`` without DCF)."""
        torch = _torch()
        assert grid.dtype == torch.complex64 and grid.is_cuda
        grid = grid.contiguous().reshape(-1, self.cells)
        ch = grid.shape[0]
        if out is None:
            out = torch.empty((ch, self.n), dtype=torch.complex64, device="cuda")
        check(self.lib.fr_degrid(self.h, _ptr(grid), ch, _ptr(out), C.c_void_p(_stream(stream))), "fr_degrid")
        return out

    def update(self, kdata, new, begin: int, dcf, grid, stream=None):
        """Streaming acquisition (fr_grid_update): replace samples [begin, begin + new.shape[1]) of
        ``kdata`` (C, N) complex64 by ``new`` (C, count) and add the gridded change into ``grid``
        (the output of ``grid(kdata, dcf)`` for this plan), both in place."""
        torch = _torch()
        assert kdata.dtype == torch.complex64 and kdata.is_cuda and kdata.is_contiguous()
        assert grid.dtype == torch.complex64 and grid.is_cuda and grid.is_contiguous()
        new = new.contiguous()
        ch, count = new.shape
        check(self.lib.fr_grid_update(self.h, _ptr(kdata), _ptr(new), begin, count, _ptr(dcf.contiguous()), ch,
                                      _ptr(grid), C.c_void_p(_stream(stream))), "fr_grid_update")
        return grid

    def grid_real(self, w, out=None, stream=None):
        """Real-valued gridding of per-sample weights: (N,) float32 -> (G^d,) float32."""
        torch = _torch()
        w = w.contiguous()
        if out is None:
            out = torch.empty(self.cells, dtype=torch.float32, device="cuda")
        check(self.lib.fr_grid_real(self.h, _ptr(w), _ptr(out), C.c_void_p(_stream(stream))), "fr_grid_real")
        return out

    def dcf_pipe(self, iterations: int = 20, w0=None, stream=None):
        """Pipe-Menon iterative DCF on this plan's trajectory and kernel."""
        torch = _torch()
        w = torch.ones(self.n, dtype=torch.float32, device="cuda") if w0 is None else w0.clone().contiguous()
        check(self.lib.fr_dcf_pipe(self.h, int(iterations), _ptr(w), C.c_void_p(_stream(stream))), "fr_dcf_pipe")
        return w


def grid_partitioned(dim: int, grid_size: int, traj, kdata, dcf, partition: int, kernel_width: float = 4.0,
                     lut=None, lut_length: int = 512, overgrid_factor: float = 2.0, tile=(0, 0, 0),
                     coil_group: int = 0, chunk: int = 0, checkerboard: bool = False, tap_lists: bool = True,
                     out=None, stream=None):
    """cuGridLut's partitioned plan (fr_grid_partitioned): the trajectory
    normalised once, then planned and gridded ``partition`` samples at a time
    into one grid.  traj: (N, 4) float32 raw coordinates; kdata: (C, N)
    complex64; dcf: (N,) float32 -> (C, G^d) complex64."""
    torch = _torch()
    lib = capi.load()
    assert traj.is_cuda and traj.dtype == torch.float32 and traj.shape[-1] == 4
    assert kdata.dtype == torch.complex64 and kdata.is_cuda and dcf.is_cuda
    if lut is None:
        lut = kb_lut(kernel_width, overgrid_factor, lut_length)
    lut = np.ascontiguousarray(lut, np.float32)
    d = _plan_desc(dim, grid_size, kernel_width, lut, tile, coil_group, chunk, checkerboard, tap_lists)
    traj, kdata, dcf = traj.contiguous(), kdata.contiguous(), dcf.contiguous()
    ch = kdata.shape[0]
    if out is None:
        out = torch.empty((ch, grid_size ** dim), dtype=torch.complex64, device="cuda")
    check(lib.fr_grid_partitioned(C.byref(d), _ptr(traj), traj.shape[0], _ptr(kdata), _ptr(dcf), ch, _ptr(out),
                                  int(partition), C.c_void_p(_stream(stream))), "fr_grid_partitioned")
    return out


def dcf_analytic(traj, dim: int, power: float = 1.0, stream=None):
    """|k|^power of raw (un-normalised) Point<float> coordinates on the device."""
    torch = _torch()
    assert traj.is_cuda and traj.dtype == torch.float32 and traj.shape[-1] == 4
    traj = traj.contiguous()
    out = torch.empty(traj.shape[0], dtype=torch.float32, device="cuda")
    check(capi.load().fr_dcf_analytic(_ptr(traj), traj.shape[0], dim, float(power), _ptr(out),
                                      C.c_void_p(_stream(stream))), "fr_dcf_analytic")
    return out


class FFT:
    """cuFFT::plan / excute: in-place unnormalised C2C over a batch of images."""

    def __init__(self, dim: int, size, batch: int, sign: int = +1):
        self.lib = capi.load()
        h = C.c_void_p()
        check(self.lib.fr_fft_create(dim, u3(size), batch, sign, C.byref(h)), "fr_fft_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fr_fft_destroy(self.h)
            self.h = None

    def __call__(self, data, stream=None):
        check(self.lib.fr_fft_execute(self.h, _ptr(data), C.c_void_p(_stream(stream))), "fr_fft_execute")
        return data


def _size3(dim, G):
    return (G, G, G if dim == 3 else 1)


def fft_shift(imgs, dim: int, G: int, stream=None):
    """ImageFilter::fftShift on (C, G^d) complex64, in place."""
    lib = capi.load()
    check(lib.fr_fft_shift(_ptr(imgs), imgs.shape[0], dim, u3(_size3(dim, G)), C.c_void_p(_stream(stream))),
          "fr_fft_shift")
    return imgs


def crop(imgs, dim: int, G: int, crop_size, stream=None):
    torch = _torch()
    cs = list(crop_size) + [1] * (3 - len(crop_size))
    out = torch.empty((imgs.shape[0], int(np.prod(cs))), dtype=torch.complex64, device="cuda")
    lib = capi.load()
    check(lib.fr_crop(_ptr(imgs), imgs.shape[0], dim, u3(_size3(dim, G)), u3(cs), _ptr(out),
                      C.c_void_p(_stream(stream))), "fr_crop")
    return out


def sos(imgs, dim: int, G: int, recon, deapod=None, stream=None, out=None):
    """ImageFilter::SOS(reconSize) then |.|: (C, G^d) complex64 -> recon float32."""
    torch = _torch()
    rs = list(recon) + [1] * (3 - len(recon))
    if out is None:
        out = torch.empty(int(np.prod(rs)), dtype=torch.float32, device="cuda")
    lib = capi.load()
    check(lib.fr_sos(_ptr(imgs), imgs.shape[0], dim, u3(_size3(dim, G)), u3(rs), _ptr(deapod), _ptr(out),
                     C.c_void_p(_stream(stream))), "fr_sos")
    return out


def low_filter(imgs, dim: int, G: int, res: int, stream=None):
    """ImageFilter::lowFilter(res) on (C, G^d) complex64, in place."""
    lib = capi.load()
    check(lib.fr_low_filter(_ptr(imgs), imgs.shape[0], dim, u3(_size3(dim, G)), res, C.c_void_p(_stream(stream))),
          "fr_low_filter")
    return imgs


def normalize_channels(imgs, dim: int, G: int, stream=None):
    """ImageFilter::normalize on (C, G^d) complex64, in place."""
    lib = capi.load()
    check(lib.fr_normalize_channels(_ptr(imgs), imgs.shape[0], dim, u3(_size3(dim, G)),
                                    C.c_void_p(_stream(stream))), "fr_normalize_channels")
    return imgs


def sos_map(imgs, maps, dim: int, G: int, recon, stream=None):
    """ImageFilter::SOS(map, reconSize): complex recon-size image."""
    torch = _torch()
    rs = list(recon) + [1] * (3 - len(recon))
    out = torch.empty(int(np.prod(rs)), dtype=torch.complex64, device="cuda")
    lib = capi.load()
    check(lib.fr_sos_map(_ptr(imgs), _ptr(maps), imgs.shape[0], dim, u3(_size3(dim, G)), u3(rs), _ptr(out),
                         C.c_void_p(_stream(stream))), "fr_sos_map")
    return out


class CropSoS:
    """Pruned backward FFT + crop + SoS of a checkerboard-flushed grid
    (fr_fft_crop_sos_*)."""

    def __init__(self, dim: int, G: int, channels: int, out_size):
        self.lib = capi.load()
        self.out_size = tuple(list(out_size) + [1] * (3 - len(out_size)))
        h = C.c_void_p()
        check(self.lib.fr_fft_crop_sos_create(dim, G, channels, u3(self.out_size), C.byref(h)),
              "fr_fft_crop_sos_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fr_fft_crop_sos_destroy(self.h)
            self.h = None

    def __call__(self, grid, deapod=None, stream=None, out=None):
        torch = _torch()
        if out is None:
            out = torch.empty(int(np.prod(self.out_size)), dtype=torch.float32, device="cuda")
        check(self.lib.fr_fft_crop_sos_execute(self.h, _ptr(grid), _ptr(deapod), _ptr(out),
                                               C.c_void_p(_stream(stream))), "fr_fft_crop_sos_execute")
        return out


class Recon:
    """The Program/Main.cpp pipeline as one object (fr_recon_*)."""

    def __init__(self, dim: int, recon_size: int, overgrid_factor: float, channels: int, out_size=None,
                 kernel_width: float = 4.0, lut_length: int = 512, max_samples: int = 0, tile=(0, 0, 0),
                 coil_group: int = 0, deapodize: bool = False, use_cufft: bool = False, pruned_fft: bool = False,
                 grid_budget: int = 0, deterministic: bool = False):
        self.lib = capi.load()
        d = capi.ReconDesc()
        d.dim = dim
        d.recon_size = recon_size
        d.overgrid_factor = overgrid_factor
        d.kernel_width = kernel_width
        d.lut_length = lut_length
        out_size = out_size or ((recon_size,) * dim + ((1,) if dim == 2 else ()))
        self.out_size = tuple(list(out_size) + [1] * (3 - len(out_size)))
        for i in range(3):
            d.out_size[i] = self.out_size[i]
            d.tile[i] = int(tile[i]) if i < len(tile) else 0
        d.channels = channels
        d.max_samples = max_samples
        d.coil_group = coil_group
        d.flags = ((capi.FR_RECON_DEAPODIZE if deapodize else 0) | (capi.FR_RECON_CUFFT if use_cufft else 0) |
                   (capi.FR_RECON_PRUNED_FFT if pruned_fft else 0) |
                   (capi.FR_RECON_DETERMINISTIC if deterministic else 0))
        d.grid_budget = grid_budget  # bytes of grid workspace: coils in slabs (0: all at once)
        h = C.c_void_p()
        check(self.lib.fr_recon_create(C.byref(d), C.byref(h)), "fr_recon_create")
        self.h = h
        self.dim, self.channels = dim, channels

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fr_recon_destroy(self.h)
            self.h = None

    def run(self, traj, dcf, kdata, out=None, stream=None):
        torch = _torch()
        n = traj.shape[0]
        if out is None:
            out = torch.empty(int(np.prod(self.out_size)), dtype=torch.float32, device="cuda")
        check(self.lib.fr_recon_run(self.h, _ptr(traj), _ptr(dcf), _ptr(kdata), n, _ptr(out),
                                    C.c_void_p(_stream(stream))), "fr_recon_run")
        return out

    def run_host(self, traj, dcf, kdata, out, stream=None):
        """Host (CPU, ideally pinned) tensors in and out."""
        n = traj.shape[0]
        check(self.lib.fr_recon_run_host(self.h, _ptr(traj), _ptr(dcf), _ptr(kdata), n, _ptr(out),
                                         C.c_void_p(_stream(stream))), "fr_recon_run_host")
        return out

    def submit_host(self, traj, dcf, kdata, out, stream=None):
        """Queues one volume of host (pinned) tensors and returns at once:
        its upload and the previous image's download overlap the recon of
        the volume before.  The tensors must stay alive and unchanged until
        sync()."""
        n = traj.shape[0]
        check(self.lib.fr_recon_submit_host(self.h, _ptr(traj), _ptr(dcf), _ptr(kdata), n, _ptr(out),
                                            C.c_void_p(_stream(stream))), "fr_recon_submit_host")
        return out

    def sync(self, stream=None):
        """Waits until every submitted volume's image is in its host tensor."""
        check(self.lib.fr_recon_sync(self.h, C.c_void_p(_stream(stream))), "fr_recon_sync")

    def _plan(self):
        h = C.c_void_p()
        check(self.lib.fr_recon_plan(self.h, C.byref(h)), "fr_recon_plan")
        return h

    def tap_words(self) -> int:
        """4-byte tap-list words per sample of the recon's plan (0: the scatter evaluates the taps)."""
        q = C.c_int()
        check(self.lib.fr_plan_tap_words(self._plan(), C.byref(q)), "fr_plan_tap_words")
        return q.value

    def profile(self, enable: bool = True):
        """Record CUDA events around the tile scatter kernel of every run."""
        check(self.lib.fr_plan_profile(self._plan(), 1 if enable else 0), "fr_plan_profile")

    def profile_read(self):
        ms = C.c_double()
        k = C.c_int()
        check(self.lib.fr_plan_profile_read(self._plan(), C.byref(ms), C.byref(k)), "fr_plan_profile_read")
        return ms.value, k.value

    def stage_ms(self):
        v = [C.c_float() for _ in range(4)]
        check(self.lib.fr_recon_stage_ms(self.h, *[C.byref(x) for x in v]), "fr_recon_stage_ms")
        return dict(plan=v[0].value, grid=v[1].value, fft=v[2].value, sos=v[3].value)
