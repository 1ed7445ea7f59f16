"""GPU: the tap-lane scatter (grid_lanes_kernel, the default for coil groups
of 16: a lane owns 4 taps of a bin record and adds them for all 32 coil
floats) against the per-warp tap-list scatter it replaces
(FR_SCATTER_WARP_LISTS=1) and against the reference.  Both add the same
fixed-point values, so with the same records in every work item
(deterministic plans) the grids agree bit for bit."""
import os

import numpy as np
import pytest

from conftest import load_case, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need CUDA"
    from fastrecon_gb300 import build
    build.build()
    return t


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


class _warp_lists:
    """Plans created inside use the per-warp tap-list scatter."""

    def __enter__(self):
        os.environ["FR_SCATTER_WARP_LISTS"] = "1"

    def __exit__(self, *a):
        os.environ.pop("FR_SCATTER_WARP_LISTS", None)


def _kspace(coils, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((coils, n)) + 1j * rng.standard_normal((coils, n))).astype(np.complex64)


def _grid(torch, c, kd, coil_group=16, **kw):
    import fastrecon_gb300 as fr
    p = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], coil_group=coil_group, deterministic=True, **kw)
    p.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    assert p.tap_words() > 0
    g = p.grid(torch.from_numpy(np.ascontiguousarray(kd)).cuda(), torch.from_numpy(c["dcf"]).cuda())
    torch.cuda.synchronize()
    return p, g.cpu().numpy()


@pytest.mark.parametrize("name,tile,chunk", [
    ("koosh3d_small", (8, 8, 8), 0),
    ("koosh3d_small", (8, 8, 8), 512),      # split tiles: partials in the reduction's layout
    ("koosh3d_small", (16, 4, 2), 512),
    ("koosh3d_small", (4, 4, 4), 0),
    ("koosh3d_odd", (8, 4, 16), 0),
    ("koosh3d_odd", (6, 6, 6), 0),          # x extent not a multiple of 4: the generic flush
    ("radial2d_small", (16, 16, 1), 0),
    ("radial2d_oddgrid", (32, 32, 1), 0),   # odd grid: the generic flush
    ("aniso2d_w5", (16, 8, 1), 512),
])
@pytest.mark.parametrize("coils", [16, 13, 32])
def test_lanes_equal_warp_lists_and_reference(torch, oracle, name, tile, chunk, coils):
    c = load_case(name)
    n = c["traj"].shape[0]
    kd = _kspace(coils, n, coils + n)
    p, g = _grid(torch, c, kd, tile=tile, chunk=chunk)
    with _warp_lists():
        _, g0 = _grid(torch, c, kd, tile=tile, chunk=chunk)
    assert np.array_equal(_bits(g), _bits(g0))
    want = oracle.grid(c["traj_norm"], c["dcf"], kd, c["dim"], c["G"], c["W"], c["lut"], threads=4)
    err = rel_l2(g, want)
    print(f"{name} tile {tile} chunk {chunk} coils {coils}: tap lanes vs reference rel-L2 {err:.2e}, "
          f"split tiles {p.stats()['slots']}")
    assert err <= TOL


def test_lanes_dense_point(torch, oracle):
    """50,000 samples on one point, 16 coils: ~100 work items per centre
    tile, each with its own fixed-point scale; the error against the FP64
    gridding stays within twice the reference's own."""
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(11)
    n = 50000
    traj = np.zeros((n + 2, 4), np.float32)
    traj[0, :3] = -0.5
    traj[1, :3] = 0.49
    traj[2:, :3] = 0.013
    dcf = rng.uniform(0.5, 1.5, n + 2).astype(np.float32)
    kd = _kspace(16, n + 2, 3)
    lut = fr.kb_lut(4.0, 1.5, 512)
    grids = []
    for warp_lists in (False, True):
        os.environ.pop("FR_SCATTER_WARP_LISTS", None)
        if warp_lists:
            os.environ["FR_SCATTER_WARP_LISTS"] = "1"
        try:
            p = fr.GridPlan(3, 24, 4.0, lut=lut, chunk=512, deterministic=True)
            p.set_trajectory(torch.from_numpy(traj).cuda())
            grids.append(p.grid(torch.from_numpy(kd).cuda(), torch.from_numpy(dcf).cuda()).cpu().numpy())
        finally:
            os.environ.pop("FR_SCATTER_WARP_LISTS", None)
    assert np.array_equal(_bits(grids[0]), _bits(grids[1]))
    tn, _, _, _, _ = oracle.normalize_traj(traj, 3, 24)
    want = oracle.grid_f64(tn, dcf, kd, 3, 24, 4.0, lut)
    ref = oracle.grid(tn, dcf, kd, 3, 24, 4.0, lut, threads=4)
    assert rel_l2(grids[0], want) <= max(1e-5, 2 * rel_l2(ref, want))


def test_lanes_recon_checkerboard_and_empty_tiles(torch, oracle):
    """The recon path (checkerboard flush, empty tiles left unwritten, pruned
    FFT) with 16 coils: the image equals the warp-list scatter's bit for bit
    and the reference recon at 1e-5."""
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    t = synth.kooshball_3d(1500, 64)
    dcf = synth.ramp_dcf(t, 3, 2.0)
    kd = synth.kspace(t, 3, 32, 16, seed=4)
    td, dd, kdd = torch.from_numpy(t).cuda(), torch.from_numpy(dcf).cuda(), torch.from_numpy(kd).cuda()
    rec = fr.Recon(3, 32, 1.5, 16, max_samples=t.shape[0], deterministic=True)
    img = rec.run(td, dd, kdd).cpu().numpy()
    with _warp_lists():
        rec0 = fr.Recon(3, 32, 1.5, 16, max_samples=t.shape[0], deterministic=True)
        img0 = rec0.run(td, dd, kdd).cpu().numpy()
    assert np.array_equal(_bits(img), _bits(img0))
    want = oracle.recon(t, dcf, kd, 3, 32, 1.5, 4.0, 512, (32, 32, 32))
    err = rel_l2(img, want)
    print(f"16-coil recon, tap lanes vs reference rel-L2 {err:.2e}")
    assert err <= TOL


def test_lanes_sample_partitions(torch, oracle):
    """Sample partitions add each range's tiles to the grid (accumulating
    flush) with 16 coils: equal to the single plan to 3e-6, to the reference
    at 1e-5."""
    import fastrecon_gb300 as fr
    c = load_case("koosh3d_small")
    n = c["traj"].shape[0]
    kd = _kspace(16, n, 21)
    td = torch.from_numpy(c["traj"]).cuda()
    kdd = torch.from_numpy(kd).cuda()
    dd = torch.from_numpy(c["dcf"]).cuda()
    _, g1 = _grid(torch, c, kd)
    gp = fr.grid_partitioned(3, c["G"], td, kdd, dd, 1700, kernel_width=c["W"], lut=c["lut"],
                             coil_group=16).cpu().numpy()
    assert rel_l2(gp, g1) <= 3e-6
    want = oracle.grid(c["traj_norm"], c["dcf"], kd, 3, c["G"], c["W"], c["lut"], threads=4)
    assert rel_l2(gp, want) <= TOL
