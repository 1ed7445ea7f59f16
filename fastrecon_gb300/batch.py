"""Batched gridding: many frames of uneven sample counts in one persistent
launch, optionally replayed from a captured CUDA graph, with an autotuner
for tile shape, bin chunk and coil group (fr_batch_* in the C ABI).  No
counterpart in the reference, which grids one dataset per
GridLut::execute."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check
from .gridding import _ptr, _stream, _torch, kb_lut


def _desc(dim, grid_size, kernel_width, lut, tile=(0, 0, 0), coil_group=0, chunk=0, checkerboard=False):
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
    d.flags = capi.FR_PLAN_CHECKERBOARD if checkerboard else 0
    return d


def _offsets(counts):
    off = np.zeros(len(counts) + 1, np.uint64)
    off[1:] = np.cumsum(np.asarray(counts, np.uint64))
    return off, (C.c_size_t * len(off))(*[int(v) for v in off])


class GridBatch:
    """Frames f = 0..F-1 with counts[f] samples each; k-space frame-major
    (frame f: channels x counts[f]), grid out frames x channels x G^d."""

    def __init__(self, dim: int, grid_size: int, kernel_width: float = 4.0, lut=None, lut_length: int = 512,
                 overgrid_factor: float = 2.0, tile=(0, 0, 0), coil_group: int = 0, chunk: int = 0,
                 checkerboard: bool = False):
        self.lib = capi.load()
        if lut is None:
            lut = kb_lut(kernel_width, overgrid_factor, lut_length)
        self.lut = np.ascontiguousarray(lut, np.float32)
        self.desc = _desc(dim, grid_size, kernel_width, self.lut, tile, coil_group, chunk, checkerboard)
        h = C.c_void_p()
        check(self.lib.fr_batch_create(C.byref(self.desc), C.byref(h)), "fr_batch_create")
        self.h = h
        self.dim, self.G = dim, grid_size
        self.frames = 0

    @classmethod
    def from_desc(cls, desc: capi.PlanDesc, lut):
        tile = [desc.tile[i] for i in range(3)]
        return cls(desc.dim, desc.grid_size, desc.kernel_width, lut=lut, tile=tile, coil_group=desc.coil_group,
                   chunk=desc.chunk, checkerboard=bool(desc.flags & capi.FR_PLAN_CHECKERBOARD))

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fr_batch_destroy(self.h)
            self.h = None

    @property
    def cells(self) -> int:
        return self.G ** self.dim

    def set_trajectories(self, traj, counts, stream=None):
        """traj: (sum(counts), 4) float32 CUDA, the frames' raw trajectories concatenated."""
        traj = traj.contiguous()
        self._traj_keep = traj
        self.off, coff = _offsets(counts)
        self.frames = len(counts)
        check(self.lib.fr_batch_set_trajectories(self.h, _ptr(traj), coff, self.frames, C.c_void_p(_stream(stream))),
              "fr_batch_set_trajectories")

    def stats(self):
        v = [C.c_longlong() for _ in range(4)]
        b = C.c_int()
        check(self.lib.fr_batch_stats(self.h, *[C.byref(x) for x in v], C.byref(b)), "fr_batch_stats")
        return dict(frames=v[0].value, samples=v[1].value, items=v[2].value, slots=v[3].value, ctas=b.value)

    def _out(self, channels, out):
        torch = _torch()
        if out is None:
            out = torch.empty((self.frames, channels, self.cells), dtype=torch.complex64, device="cuda")
        return out

    def grid(self, kdata_flat, dcf, channels: int, out=None, stream=None):
        """kdata_flat: complex64 CUDA, frame-major blocks (channels x n_f each)."""
        out = self._out(channels, out)
        check(self.lib.fr_batch_grid(self.h, _ptr(kdata_flat), _ptr(dcf), channels, _ptr(out),
                                     C.c_void_p(_stream(stream))), "fr_batch_grid")
        return out

    def capture(self, kdata_flat, dcf, channels: int, out=None, stream=None):
        """Capture the batch gridding into a CUDA graph bound to these buffers."""
        out = self._out(channels, out)
        self._bound = (kdata_flat, dcf, out)
        check(self.lib.fr_batch_capture(self.h, _ptr(kdata_flat), _ptr(dcf), channels, _ptr(out),
                                        C.c_void_p(_stream(stream))), "fr_batch_capture")
        return out

    def replay(self, stream=None):
        check(self.lib.fr_batch_replay(self.h, C.c_void_p(_stream(stream))), "fr_batch_replay")


def autotune(dim, grid_size, traj, counts, kdata_flat, dcf, channels, kernel_width=4.0, lut=None,
             overgrid_factor=2.0, lut_length=512, repeats=3, stream=None):
    """Fastest (tile, chunk, coil_group) for this batch; returns (GridBatch, ms)."""
    torch = _torch()
    if lut is None:
        lut = kb_lut(kernel_width, overgrid_factor, lut_length)
    lut = np.ascontiguousarray(lut, np.float32)
    base = _desc(dim, grid_size, kernel_width, lut)
    best = capi.PlanDesc()
    ms = C.c_float()
    _, coff = _offsets(counts)
    scratch = torch.empty((len(counts), channels, grid_size ** dim), dtype=torch.complex64, device="cuda")
    check(capi.load().fr_batch_autotune(C.byref(base), _ptr(traj.contiguous()), coff, len(counts), _ptr(kdata_flat),
                                        _ptr(dcf), channels, _ptr(scratch), repeats, C.byref(best), C.byref(ms),
                                        C.c_void_p(_stream(stream))), "fr_batch_autotune")
    del scratch
    b = GridBatch.from_desc(best, lut)
    return b, ms.value
