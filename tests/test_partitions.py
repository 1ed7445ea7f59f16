"""Sample partitions (fr_grid_partitioned): cuGridLut's partitioned plan
(cuGridLut::setNumOfPartitions, cuGridLut.h:40-42; cuGridLut.cu:128-149,
182-220).  The trajectory is normalised once with the whole trajectory's
bounds, then planned and gridded in sample ranges that add into one grid;
the result must equal the single-plan grid (float rounding aside: each
range's tile sums are rounded to float before they are added) and the
reference's algorithm at the project's 1e-5 bar."""
import numpy as np
import pytest

from conftest import load_case, rel_l2

TOL = 1e-5


def test_partitioned_rejects_bad_arguments_without_gpu(frlib):
    assert frlib.fr_grid_partitioned(None, None, 0, None, None, 1, None, 0, None) == 1  # FR_ERR_INVALID_ARGUMENT


def _single(torch, c, kd, **kw):
    import fastrecon_gb300 as fr
    p = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], **kw)
    p.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    return p.grid(kd, torch.from_numpy(c["dcf"]).cuda()).cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "koosh3d_odd", "spiral2d_w3"])
@pytest.mark.parametrize("parts", [2, 3, 7])
def test_partitioned_equals_single_plan(oracle, name, parts):
    import torch

    import fastrecon_gb300 as fr
    c = load_case(name)
    n = c["traj"].shape[0]
    kd = torch.from_numpy(c["kdata"]).cuda()
    traj = torch.from_numpy(c["traj"]).cuda()
    dcf = torch.from_numpy(c["dcf"]).cuda()
    part = -(-n // parts)
    g = fr.grid_partitioned(c["dim"], c["G"], traj, kd, dcf, part, kernel_width=c["W"], lut=c["lut"]).cpu().numpy()
    single = _single(torch, c, kd)
    e_single, e_ref = rel_l2(g, single), rel_l2(g, c["grid"])
    print(f"{name} in {parts} partitions: vs single plan rel-L2 {e_single:.2e}, vs reference {e_ref:.2e}")
    assert e_ref <= TOL
    assert e_single <= 3e-6
    assert np.array_equal(g == 0, c["grid"] == 0)


@pytest.mark.gpu
def test_partitioned_variants(oracle):
    """Checkerboard output, the geometry scatter (no tap lists), odd coil
    counts and a partition that does not divide the samples; one partition
    (partition >= n or 0) is the single plan itself."""
    import torch

    import fastrecon_gb300 as fr
    c = load_case("koosh3d_small")
    n = c["traj"].shape[0]
    rng = np.random.default_rng(3)
    kd_np = (rng.standard_normal((5, n)) + 1j * rng.standard_normal((5, n))).astype(np.complex64)
    kd = torch.from_numpy(kd_np).cuda()
    traj = torch.from_numpy(c["traj"]).cuda()
    dcf = torch.from_numpy(c["dcf"]).cuda()
    want = oracle.grid(c["traj_norm"], c["dcf"], kd_np, 3, c["G"], c["W"], c["lut"], threads=4)
    for kw in [dict(), dict(tap_lists=False), dict(checkerboard=True)]:
        g = fr.grid_partitioned(3, c["G"], traj, kd, dcf, n // 3 + 17, kernel_width=c["W"], lut=c["lut"], **kw)
        g = g.cpu().numpy()
        if kw.get("checkerboard"):
            idx = np.indices((c["G"],) * 3).sum(0).reshape(-1)
            g = g * np.where(idx % 2, -1.0, 1.0).astype(np.float32)
        assert rel_l2(g, want) <= TOL, kw
    # one work item per tile (no split tiles, whose record sets vary from run
    # to run) makes the single plan repeat bit for bit
    single = _single(torch, c, kd, chunk=16384)
    for part in (0, n, 10 * n):
        g = fr.grid_partitioned(3, c["G"], traj, kd, dcf, part, kernel_width=c["W"], lut=c["lut"], chunk=16384)
        assert np.array_equal(g.cpu().numpy().view(np.uint32), single.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.slow
def test_partitioned_kooshball_full_trajectory(oracle):
    """The 3D kooshball benchmark's full trajectory (50,000 golden-means
    spokes x 256, 384^3 grid), 2 coils, in 4 partitions against one plan."""
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    cfg = dict(synth.CONFIGS["kooshball3d"])
    cfg["coils"] = 2
    traj, dcf, kd = synth.make_case(**cfg, xp=torch, device="cuda")
    G = fr.grid_size(256, 1.5)
    lut = oracle.kb_lut(4.0, 1.5, 512)
    tt, dd = torch.from_numpy(traj).cuda(), torch.from_numpy(dcf).cuda()
    n = traj.shape[0]
    g = fr.grid_partitioned(3, G, tt, kd, dd, -(-n // 4), lut=lut)
    p = fr.GridPlan(3, G, 4.0, lut=lut)
    p.set_trajectory(tt)
    single = p.grid(kd, dd)
    err = (torch.linalg.vector_norm(g - single) / torch.linalg.vector_norm(single)).item()
    print(f"kooshball 50,000x256 in 4 partitions vs one plan: rel-L2 {err:.2e}")
    assert err <= 3e-6
