"""GPU: the scatter that reads the plan's tap lists (the taps of every sample
evaluated once per trajectory) against the reference and against the scatter
that evaluates the taps itself (FR_PLAN_NO_TAP_LISTS)."""
import numpy as np
import pytest

from conftest import CASE_NAMES, load_case, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need CUDA"
    from fastrecon_gb300 import build
    build.build()
    return t


def _grid(torch, c, kd, tap_lists=True, **kw):
    import fastrecon_gb300 as fr
    p = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], tap_lists=tap_lists, **kw)
    p.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    g = p.grid(torch.from_numpy(np.ascontiguousarray(kd)).cuda(), torch.from_numpy(c["dcf"]).cuda())
    torch.cuda.synchronize()
    return p, g.cpu().numpy()


@pytest.mark.parametrize("name", CASE_NAMES)
def test_tap_lists_match_reference(torch, oracle, name):
    c = load_case(name)
    p, g = _grid(torch, c, c["kdata"])
    assert p.tap_words() > 0
    _, g0 = _grid(torch, c, c["kdata"], tap_lists=False)
    err = rel_l2(g, c["grid"])
    print(f"{name}: tap-list scatter vs reference rel-L2 {err:.2e}, vs geometry scatter {rel_l2(g, g0):.2e}")
    assert err <= TOL
    # two independent fixed-point roundings (one scale per item here, one per
    # coil float in the geometry scatter's coil-major path), each ~1e-6
    assert rel_l2(g, g0) <= 3e-6
    assert np.array_equal(g == 0, c["grid"] == 0)


@pytest.mark.parametrize("coils,cg", [(1, 4), (3, 4), (5, 8), (7, 8), (12, 16), (16, 16), (17, 16), (33, 16)])
def test_tap_lists_coil_groups(torch, oracle, coils, cg):
    """Every coil group width (4, 8, 16 coils per pass), odd coil counts (the
    sample-major copy's rows padded to an even count) and partial last
    groups."""
    c = load_case("koosh3d_small")
    rng = np.random.default_rng(coils)
    n = c["traj"].shape[0]
    kd = (rng.standard_normal((coils, n)) + 1j * rng.standard_normal((coils, n))).astype(np.complex64)
    p, g = _grid(torch, c, kd, coil_group=cg)
    assert p.tap_words() > 0
    want = oracle.grid(c["traj_norm"], c["dcf"], kd, 3, c["G"], c["W"], c["lut"], threads=4)
    assert rel_l2(g, want) <= TOL


@pytest.mark.parametrize("tile", [(8, 8, 8), (16, 4, 2), (4, 4, 4), (8, 4, 16)])
def test_tap_lists_tile_shapes(torch, oracle, tile):
    """Tiles smaller than the kernel footprint put a sample's taps in up to
    3 tiles per axis (more runs per slot)."""
    c = load_case("koosh3d_odd")
    p, g = _grid(torch, c, c["kdata"], tile=tile, coil_group=4)
    assert p.tap_words() > 0
    assert rel_l2(g, c["grid"]) <= TOL


def test_tap_lists_split_tiles_and_dense_point(torch, oracle):
    """50,000 samples on one point: the centre tiles are split into many work
    items (partials reduced in item order), each item's fixed-point scale
    comes from its own records."""
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(5)
    n = 50000
    traj = np.zeros((n + 2, 4), np.float32)
    traj[0, :3] = -0.5
    traj[1, :3] = 0.49
    traj[2:, :3] = 0.013
    dcf = rng.uniform(0.5, 1.5, n + 2).astype(np.float32)
    kd = (rng.standard_normal((4, n + 2)) + 1j * rng.standard_normal((4, n + 2))).astype(np.complex64)
    G = 24
    lut = fr.kb_lut(4.0, 1.5, 512)
    p = fr.GridPlan(3, G, 4.0, lut=lut, chunk=512)
    p.set_trajectory(torch.from_numpy(traj).cuda())
    assert p.tap_words() > 0 and p.stats()["slots"] > 0
    g = p.grid(torch.from_numpy(kd).cuda(), torch.from_numpy(dcf).cuda()).cpu().numpy()
    tn, _, _, _, _ = oracle.normalize_traj(traj, 3, G)
    want = oracle.grid_f64(tn, dcf, kd, 3, G, 4.0, lut)
    ref = oracle.grid(tn, dcf, kd, 3, G, 4.0, lut, threads=4)
    err, err_ref = rel_l2(g, want), rel_l2(ref, want)
    print(f"dense point: tap-list scatter vs FP64 {err:.2e}, reference FP32 vs FP64 {err_ref:.2e}")
    assert err <= max(1e-5, 2 * err_ref)


def test_tap_lists_repeatable(torch):
    """Tiles held by one work item grid to the same bits on every run
    (integer adds are order-free); with split tiles, runs agree to 1e-6."""
    c = load_case("koosh3d_small")
    p, g1 = _grid(torch, c, c["kdata"], chunk=16384)
    assert p.stats()["slots"] == 0
    g2 = p.grid(torch.from_numpy(c["kdata"]).cuda(), torch.from_numpy(c["dcf"]).cuda()).cpu().numpy()
    assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32))
    p, g1 = _grid(torch, c, c["kdata"], chunk=512)
    g2 = p.grid(torch.from_numpy(c["kdata"]).cuda(), torch.from_numpy(c["dcf"]).cuda()).cpu().numpy()
    assert rel_l2(g1, g2) <= 1e-6


def test_out_of_memory_paths_with_injected_failures(torch):
    """Host-side fault injection (FR_FAIL_ALLOC_BYTES: device reservations of
    that many bytes or more fail as cudaMalloc would).  A plan whose tap lists
    cannot be allocated falls back to the geometry scatter and stays correct;
    a plan that cannot hold the trajectory returns FR_ERR_OUT_OF_MEMORY (3)
    from fr_plan_set_trajectory, and so does a recon object's creation; with
    the injection removed the same calls succeed."""
    import os

    import fastrecon_gb300 as fr
    from fastrecon_gb300.capi import FastreconError
    c = load_case("koosh3d_small")
    n = c["traj"].shape[0]
    # one work item per tile (no split-tile partials): the tap slots are the
    # plan's largest reservation
    p0, _ = _grid(torch, c, c["kdata"], chunk=16384)
    words = p0.tap_words()
    assert words > 0 and p0.stats()["slots"] == 0
    try:
        os.environ["FR_FAIL_ALLOC_BYTES"] = str(n * words * 4)  # the tap slots and nothing else
        p, g = _grid(torch, c, c["kdata"], chunk=16384)
        assert p.tap_words() == 0
        assert rel_l2(g, c["grid"]) <= TOL
        os.environ["FR_FAIL_ALLOC_BYTES"] = str(n * 8)  # below the trajectory copy
        p = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"])
        with pytest.raises(FastreconError) as ei:
            p.set_trajectory(torch.from_numpy(c["traj"]).cuda())
        assert ei.value.status == 3
        os.environ["FR_FAIL_ALLOC_BYTES"] = "64"
        with pytest.raises(FastreconError) as ei:
            fr.Recon(c["dim"], c["recon"], c["os"], c["coils"], max_samples=n)
        assert ei.value.status == 3
    finally:
        os.environ.pop("FR_FAIL_ALLOC_BYTES", None)
    p, g = _grid(torch, c, c["kdata"])
    assert p.tap_words() > 0 and rel_l2(g, c["grid"]) <= TOL


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_deterministic_plans_repeat_bit_for_bit(torch, oracle):
    """FR_PLAN_DETERMINISTIC: the records of split tiles are put in sample
    order after the bin fill, so every work item holds the same records and
    the grid repeats bit for bit across plans and runs -- here with small
    work items (many split tiles, up to ~50 items per tile) and the
    50,000-sample dense point; the grid still equals the reference at 1e-5."""
    import fastrecon_gb300 as fr
    c = load_case("koosh3d_small")
    kd = torch.from_numpy(c["kdata"]).cuda()
    dcf = torch.from_numpy(c["dcf"]).cuda()
    traj = torch.from_numpy(c["traj"]).cuda()
    grids = []
    for _ in range(3):
        p = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], chunk=512, deterministic=True)
        p.set_trajectory(traj)
        assert p.stats()["slots"] > 0 and p.tap_words() > 0
        grids.append(p.grid(kd, dcf).cpu().numpy())
        grids.append(p.grid(kd, dcf).cpu().numpy())
    for g in grids[1:]:
        assert np.array_equal(_bits(g), _bits(grids[0]))
    assert rel_l2(grids[0], c["grid"]) <= TOL

    rng = np.random.default_rng(9)
    n = 50000
    tr = np.zeros((n + 2, 4), np.float32)
    tr[0, :3] = -0.5
    tr[1, :3] = 0.49
    tr[2:, :3] = 0.013
    d2 = rng.uniform(0.5, 1.5, n + 2).astype(np.float32)
    k2 = (rng.standard_normal((4, n + 2)) + 1j * rng.standard_normal((4, n + 2))).astype(np.complex64)
    lut = fr.kb_lut(4.0, 1.5, 512)
    outs = []
    for _ in range(3):
        p = fr.GridPlan(3, 24, 4.0, lut=lut, chunk=512, deterministic=True)
        p.set_trajectory(torch.from_numpy(tr).cuda())
        outs.append(p.grid(torch.from_numpy(k2).cuda(), torch.from_numpy(d2).cuda()).cpu().numpy())
    for g in outs[1:]:
        assert np.array_equal(_bits(g), _bits(outs[0]))
    tn, _, _, _, _ = oracle.normalize_traj(tr, 3, 24)
    want = oracle.grid_f64(tn, d2, k2, 3, 24, 4.0, lut)
    ref = oracle.grid(tn, d2, k2, 3, 24, 4.0, lut, threads=4)
    assert rel_l2(outs[0], want) <= max(1e-5, 2 * rel_l2(ref, want))


def test_deterministic_recon_repeats_bit_for_bit(torch):
    """The recon object with FR_RECON_DETERMINISTIC: the same image bits on
    every run (default records per work item, split centre tiles)."""
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    t = synth.kooshball_3d(4000, 128)
    dcf = synth.ramp_dcf(t, 3, 2.0)
    kd = synth.kspace(t, 3, 64, 8, seed=2, xp=torch, device="cuda")
    td, dd = torch.from_numpy(t).cuda(), torch.from_numpy(dcf).cuda()
    rec = fr.Recon(3, 64, 1.5, 8, max_samples=t.shape[0], deterministic=True)
    imgs = [rec.run(td, dd, kd).cpu().numpy() for _ in range(4)]
    for im in imgs[1:]:
        assert np.array_equal(_bits(im), _bits(imgs[0]))
