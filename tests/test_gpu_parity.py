"""GPU parity: the sm_103a path (through the C ABI) against the oracle and the
golden fixtures of the reference's own CPU code.

Bars:
* integer work (trajectory normalisation, per-sample cell ranges, tile
  bins, fftShift permutation, SoS arithmetic on identical inputs): bit-exact;
* floating-point gridding and recon: relative L2 <= 1e-5 against the
  reference's FP32 CPU results (summation order differs), with the error
  against the FP64 oracle printed.
"""
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


def cu(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def make_plan(c, **kw):
    import fastrecon_gb300 as fr
    return fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], **kw)


# ---------------------------------------------------------------- plan ----

def test_normalized_trajectory_bit_exact(torch, case):
    p = make_plan(case)
    p.set_trajectory(cu(torch, case["traj"]))
    tn = p.normalized_trajectory().cpu().numpy()
    assert np.array_equal(bits(tn), bits(case["traj_norm"]))


def test_bounds_match_oracle(torch, oracle, case):
    p = make_plan(case)
    p.set_trajectory(cu(torch, case["traj"]))
    raw_lo, raw_hi, n_lo, n_hi = p.bounds()
    tn, tr, sc, lo, hi = oracle.normalize_traj(case["traj"], case["dim"], case["G"])
    lo0, hi0 = oracle.comp_bounds(case["traj"], case["dim"])
    assert np.array_equal(raw_lo, lo0) and np.array_equal(raw_hi, hi0)
    assert np.array_equal(bits(n_lo), bits(lo)) and np.array_equal(bits(n_hi), bits(hi))


def test_sample_ranges_bit_exact(torch, oracle, case):
    p = make_plan(case)
    p.set_trajectory(cu(torch, case["traj"]))
    s, e = p.sample_ranges()
    s0, e0 = oracle.sample_range(case["traj_norm"], case["dim"], case["G"], case["W"] / 2)
    assert np.array_equal(s.cpu().numpy(), s0) and np.array_equal(e.cpu().numpy(), e0)


@pytest.mark.parametrize("tile", [None, (8, 8, 8), (16, 4, 2), (5, 7, 3)])
def test_bins_bit_exact(torch, oracle, case, tile):
    dim = case["dim"]
    if tile is None:
        tile = (32, 32, 1) if dim == 2 else (8, 8, 8)
    if dim == 2:
        tile = (tile[0], tile[1], 1)
    cg = 4 if tile[0] % 4 == 0 else 16  # tile x must be a multiple of 32/floats-per-cell
    p = make_plan(case, tile=tile, coil_group=cg)
    p.set_trajectory(cu(torch, case["traj"]))
    off, pairs = p.bins()
    off = off.cpu().numpy()
    pairs = pairs.cpu().numpy().astype(np.int64)
    s0, e0 = oracle.sample_range(case["traj_norm"], dim, case["G"], case["W"] / 2)
    tlo, thi = oracle.sample_tiles(s0, e0, dim, tile)
    G = case["G"]
    nt = [-(-G // tile[0]), -(-G // tile[1]), (-(-G // tile[2])) if dim == 3 else 1]
    want = [[] for _ in range(nt[0] * nt[1] * nt[2])]
    for smp in range(len(s0)):
        if tlo[smp, 0] > thi[smp, 0]:
            continue
        for tz in range(tlo[smp, 2], thi[smp, 2] + 1):
            for ty in range(tlo[smp, 1], thi[smp, 1] + 1):
                for tx in range(tlo[smp, 0], thi[smp, 0] + 1):
                    want[(tz * nt[1] + ty) * nt[0] + tx].append(smp)
    assert len(off) == len(want) + 1
    for t, lst in enumerate(want):
        got = np.sort(pairs[off[t]:off[t + 1]])
        assert np.array_equal(got, np.array(lst, np.int64)), f"tile {t}"


# ---------------------------------------------------------------- grid ----

def test_grid_vs_reference(torch, oracle, case):
    p = make_plan(case)
    p.set_trajectory(cu(torch, case["traj"]))
    g = p.grid(cu(torch, case["kdata"]), cu(torch, case["dcf"])).cpu().numpy()
    err = rel_l2(g, case["grid"])
    g64 = oracle.grid_f64(case["traj_norm"], case["dcf"], case["kdata"], case["dim"], case["G"], case["W"],
                          case["lut"])
    print(f"{case['name']}: GPU vs reference rel-L2 {err:.2e}, GPU vs FP64 oracle {rel_l2(g, g64):.2e}, "
          f"reference vs FP64 {rel_l2(case['grid'], g64):.2e}")
    assert err <= TOL
    # cells no sample touches are exactly zero, as in the reference
    assert np.array_equal(g == 0, case["grid"] == 0)


@pytest.mark.parametrize("coils,cg", [(1, 4), (3, 4), (5, 8), (12, 16), (16, 16), (17, 8), (32, 32), (33, 16)])
def test_grid_coil_groups(torch, oracle, coils, cg):
    c = load_case("koosh3d_small")
    rng = np.random.default_rng(coils)
    n = c["traj"].shape[0]
    kd = (rng.standard_normal((coils, n)) + 1j * rng.standard_normal((coils, n))).astype(np.complex64)
    p = make_plan(c, coil_group=cg)
    p.set_trajectory(cu(torch, c["traj"]))
    g = p.grid(cu(torch, kd), cu(torch, c["dcf"])).cpu().numpy()
    want = oracle.grid(c["traj_norm"], c["dcf"], kd, 3, c["G"], c["W"], c["lut"], threads=4)
    assert rel_l2(g, want) <= TOL


@pytest.mark.parametrize("tile,cg", [((32, 32, 1), 8), ((16, 8, 1), 4), ((64, 16, 1), 16), ((8, 8, 1), 32)])
def test_grid_tile_shapes_2d(torch, oracle, tile, cg):
    c = load_case("radial2d_small")
    p = make_plan(c, tile=tile, coil_group=cg)
    p.set_trajectory(cu(torch, c["traj"]))
    g = p.grid(cu(torch, c["kdata"]), cu(torch, c["dcf"])).cpu().numpy()
    assert rel_l2(g, c["grid"]) <= TOL


@pytest.mark.parametrize("tile,cg", [((8, 8, 8), 16), ((16, 8, 4), 8), ((4, 4, 4), 4), ((32, 4, 2), 32)])
def test_grid_tile_shapes_3d(torch, oracle, tile, cg):
    c = load_case("koosh3d_small")
    p = make_plan(c, tile=tile, coil_group=cg)
    p.set_trajectory(cu(torch, c["traj"]))
    g = p.grid(cu(torch, c["kdata"]), cu(torch, c["dcf"])).cpu().numpy()
    assert rel_l2(g, c["grid"]) <= TOL


def test_grid_split_tiles(torch, oracle):
    """Tiny chunks force every busy tile through the partial/reduce path."""
    c = load_case("koosh3d_small")
    p = make_plan(c, chunk=7)
    p.set_trajectory(cu(torch, c["traj"]))
    st = p.stats()
    assert st["slots"] > 0
    g = p.grid(cu(torch, c["kdata"]), cu(torch, c["dcf"])).cpu().numpy()
    assert rel_l2(g, c["grid"]) <= TOL


def test_grid_empty_trajectory(torch):
    import fastrecon_gb300 as fr
    lut = fr.kb_lut(4.0, 2.0, 512)
    p = fr.GridPlan(2, 64, 4.0, lut=lut)
    p.set_trajectory(torch.zeros((0, 4), dtype=torch.float32, device="cuda"))
    g = p.grid(torch.zeros((2, 0), dtype=torch.complex64, device="cuda"),
               torch.zeros(0, dtype=torch.float32, device="cuda"))
    assert g.shape == (2, 64 * 64) and bool((g == 0).all())


def test_grid_nonfinite_and_outside_samples(torch, oracle):
    """NaN/inf coordinates and samples outside the grid contribute nothing,
    matching the reference (components other than x are scaled by x's range
    and may leave [0, G-1])."""
    rng = np.random.default_rng(5)
    n = 3000
    t = np.zeros((n, 4), np.float32)
    t[:, 0] = rng.uniform(-0.5, 0.5, n)
    t[:, 1] = rng.uniform(-2.0, 2.0, n)
    t[::97, 1] = np.nan
    t[::89, 1] = np.inf
    t[::83, 1] = 1e30
    dcf = rng.uniform(0, 1, n).astype(np.float32)
    kd = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
    import fastrecon_gb300 as fr
    G = 48
    lut = fr.kb_lut(4.0, 1.5, 512)
    p = fr.GridPlan(2, G, 4.0, lut=lut)
    p.set_trajectory(cu(torch, t))
    tn, *_ = oracle.normalize_traj(t, 2, G)
    s, e = p.sample_ranges()
    s0, e0 = oracle.sample_range(tn, 2, G, 2.0)
    assert np.array_equal(s.cpu().numpy(), s0) and np.array_equal(e.cpu().numpy(), e0)
    g = p.grid(cu(torch, kd), cu(torch, dcf)).cpu().numpy()
    want = oracle.grid(tn, dcf, kd, 2, G, 4.0, lut)
    assert rel_l2(g, want) <= TOL


def test_grid_single_dense_point(torch, oracle):
    """50,000 samples at one location: one very heavy tile, split into many
    work items and summed by the partial-reduce kernel.  50,000 FP32 terms
    per cell: the bar is the reference's own FP32 error against FP64."""
    n = 50000
    rng = np.random.default_rng(2)
    t = np.zeros((n, 4), np.float32)
    t[0, :3] = -0.5
    t[1, :3] = 0.5  # set the bounds
    t[2:, :3] = 0.01
    dcf = rng.uniform(0.5, 1.0, n).astype(np.float32)
    kd = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
    import fastrecon_gb300 as fr
    lut = fr.kb_lut(4.0, 1.5, 512)
    G = 24
    p = fr.GridPlan(3, G, 4.0, lut=lut)
    p.set_trajectory(cu(torch, t))
    assert p.stats()["slots"] > 1
    g = p.grid(cu(torch, kd), cu(torch, dcf)).cpu().numpy()
    tn, *_ = oracle.normalize_traj(t, 3, G)
    want = oracle.grid_f64(tn, dcf, kd, 3, G, 4.0, lut)
    ref32 = oracle.grid(tn, dcf, kd, 3, G, 4.0, lut)
    err, err_ref = rel_l2(g, want), rel_l2(ref32, want)
    print(f"dense point: GPU vs FP64 {err:.2e}, reference FP32 vs FP64 {err_ref:.2e}")
    assert err <= max(TOL, 2 * err_ref)


def test_grid_repeatable(torch):
    c = load_case("koosh3d_small")
    p = make_plan(c)
    p.set_trajectory(cu(torch, c["traj"]))
    a = p.grid(cu(torch, c["kdata"]), cu(torch, c["dcf"])).cpu().numpy()
    b = p.grid(cu(torch, c["kdata"]), cu(torch, c["dcf"])).cpu().numpy()
    assert rel_l2(a, b) <= 1e-6


# ---------------------------------------------------------- image stage ----

@pytest.mark.parametrize("dim,G,rec", [(2, 64, 32), (2, 31, 21), (3, 30, 20), (3, 21, 14), (2, 48, 48)])
def test_shift_and_sos_bit_exact(torch, oracle, dim, G, rec):
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(G)
    C = 3
    x = (rng.standard_normal((C, G ** dim)) + 1j * rng.standard_normal((C, G ** dim))).astype(np.complex64)
    xs = np.stack([oracle.fft_shift(x[c], dim, G) for c in range(C)])
    xd = cu(torch, x)
    fr.fft_shift(xd, dim, G)
    assert np.array_equal(xd.cpu().numpy(), xs)
    recon = (rec, rec, rec if dim == 3 else 1)
    want = np.abs(oracle.sos(xs, dim, G, recon)).astype(np.float32)
    got = fr.sos(xd, dim, G, recon).cpu().numpy()
    assert np.array_equal(bits(got), bits(want))


def test_crop_exact(torch):
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(9)
    G, dim = 20, 3
    x = (rng.standard_normal((2, G ** 3)) + 1j * rng.standard_normal((2, G ** 3))).astype(np.complex64)
    got = fr.crop(cu(torch, x), dim, G, (10, 12, 14)).cpu().numpy().reshape(2, 14, 12, 10)
    want = x.reshape(2, G, G, G)[:, 3:17, 4:16, 5:15]
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dim,G", [(2, 64), (2, 31), (3, 30), (3, 21)])
def test_fft_vs_oracle(torch, oracle, dim, G):
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(G + dim)
    x = (rng.standard_normal((2, G ** dim)) + 1j * rng.standard_normal((2, G ** dim))).astype(np.complex64)
    xd = cu(torch, x)
    fr.FFT(dim, (G, G, G if dim == 3 else 1), 2, +1)(xd)
    assert rel_l2(xd.cpu().numpy(), oracle.fft(x, dim, G, +1, 4)) <= TOL


def test_checkerboard_fold_equals_shift(torch, case):
    """Gridding with the (-1)^(x+y+z) flush + FFT == FFT + fftShift (even G)."""
    if case["G"] % 2:
        pytest.skip("checkerboard folding needs an even grid")
    import fastrecon_gb300 as fr
    dim, G = case["dim"], case["G"]
    size = (G, G, G if dim == 3 else 1)
    a = make_plan(case)
    a.set_trajectory(cu(torch, case["traj"]))
    ga = a.grid(cu(torch, case["kdata"]), cu(torch, case["dcf"]))
    fr.FFT(dim, size, ga.shape[0], +1)(ga)
    fr.fft_shift(ga, dim, G)
    b = make_plan(case, checkerboard=True)
    b.set_trajectory(cu(torch, case["traj"]))
    gb = b.grid(cu(torch, case["kdata"]), cu(torch, case["dcf"]))
    fr.FFT(dim, size, gb.shape[0], +1)(gb)
    assert rel_l2(gb.cpu().numpy(), ga.cpu().numpy()) <= TOL


# ---------------------------------------------------------------- recon ----

def test_recon_vs_reference(torch, case):
    import fastrecon_gb300 as fr
    dim = case["dim"]
    r = fr.Recon(dim, case["recon"], case["os"], case["coils"], kernel_width=case["W"], lut_length=case["L"],
                 max_samples=case["traj"].shape[0])
    img = r.run(cu(torch, case["traj"]), cu(torch, case["dcf"]), cu(torch, case["kdata"])).cpu().numpy()
    err = rel_l2(img, case["image"])
    print(f"{case['name']}: recon rel-L2 vs reference {err:.2e}")
    assert err <= TOL


def test_recon_host_buffers_match_device(torch, case):
    import fastrecon_gb300 as fr
    r = fr.Recon(case["dim"], case["recon"], case["os"], case["coils"], kernel_width=case["W"],
                 lut_length=case["L"], max_samples=case["traj"].shape[0])
    dev = r.run(cu(torch, case["traj"]), cu(torch, case["dcf"]), cu(torch, case["kdata"])).cpu().numpy()
    out = torch.empty(dev.shape[0], dtype=torch.float32).pin_memory()
    r.run_host(torch.from_numpy(case["traj"]).pin_memory(), torch.from_numpy(case["dcf"]).pin_memory(),
               torch.from_numpy(case["kdata"]).pin_memory(), out)
    assert rel_l2(out.numpy(), case["image"]) <= TOL
    assert rel_l2(out.numpy(), dev) <= 1e-6


def test_recon_submitted_volumes_match_one_call(torch, case):
    """fr_recon_submit_host: volumes queued back to back (two staging slots,
    uploads and downloads overlapping the recon of the volume before) give
    the images of one fr_recon_run_host call each, including a volume with
    fewer samples between full ones.  Equal to rounding: the bin fill orders a
    tile's records by atomics, so a dense tile's split into work items (each
    with its own fixed-point scale) varies from run to run by ~1e-7."""
    import fastrecon_gb300 as fr
    r = fr.Recon(case["dim"], case["recon"], case["os"], case["coils"], kernel_width=case["W"],
                 lut_length=case["L"], max_samples=case["traj"].shape[0])
    n = case["traj"].shape[0]
    vols = []
    for k, m in enumerate([n, n // 2, n, n]):
        kd = np.ascontiguousarray(case["kdata"][:, :m] * np.complex64(1.0 + 0.5 * k - 0.25j * k))
        vols.append([torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
                     for a in (case["traj"][:m], case["dcf"][:m], kd)])
    nout = int(np.prod(r.out_size))
    want = []
    for v in vols:
        out = torch.empty(nout, dtype=torch.float32).pin_memory()
        r.run_host(*v, out)
        want.append(out.numpy().copy())
    got = [torch.full((nout,), float("nan"), dtype=torch.float32).pin_memory() for _ in vols]
    for v, out in zip(vols, got):
        r.submit_host(*v, out)
    r.sync()
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel_l2(g.numpy(), w) <= 1e-6, k
    assert rel_l2(got[0].numpy(), case["image"]) <= TOL


def test_deapodization_flattens_point_response(torch):
    """A unit sample at k = 0 images to a constant; the kernel's apodization
    rolls it off toward the edges, and deapodization restores it."""
    import fastrecon_gb300 as fr
    n = 3
    G = 128
    t = np.zeros((n, 4), np.float32)
    t[0, :2] = -0.5
    t[1, :2] = 0.5 - 1.0 / G  # scale (G-1)/(1 - 1/G) = G: k = 0 lands on cell G/2
    dcf = np.array([0, 0, 1], np.float32)
    kd = np.ones((1, n), np.complex64)
    flat = fr.Recon(2, 64, 2.0, 1, deapodize=True)
    raw = fr.Recon(2, 64, 2.0, 1, deapodize=False)
    a = flat.run(cu(torch, t), cu(torch, dcf), cu(torch, kd)).cpu().numpy().reshape(64, 64)
    b = raw.run(cu(torch, t), cu(torch, dcf), cu(torch, kd)).cpu().numpy().reshape(64, 64)
    assert b[32, 32] > 1.2 * b[32, 0] and b[32, 32] > 1.2 * b[0, 0]  # apodized
    assert np.max(np.abs(a / a[32, 32] - 1)) < 1e-3


@pytest.mark.parametrize("dim,recon,os_,W,coils", [(2, 64, 2.0, 4.0, 3), (2, 128, 2.0, 5.0, 2), (3, 32, 1.5, 4.0, 2),
                                                  (3, 24, 2.0, 4.0, 4)])
def test_deapodization_vs_fp64_oracle(torch, oracle, dim, recon, os_, W, coils):
    """The deapodization map the recon divides by (GPU: the kernel's taps
    seeded at the grid centre, transformed by the recon's own FFT) against
    the FP64 oracle's direct sum over the taps, and the deapodized image
    against the reference algorithm's image divided by that map."""
    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    traj = synth.radial_2d(48, 2 * recon) if dim == 2 else synth.kooshball_3d(300, 2 * recon)
    dcf = synth.ramp_dcf(traj, dim, float(dim - 1))
    kd = synth.kspace(traj, dim, recon, coils, seed=3)
    G = fr.grid_size(recon, os_)
    out = (recon,) * dim
    imgs = {}
    for dp in (False, True):
        r = fr.Recon(dim, recon, os_, coils, kernel_width=W, deapodize=dp)
        imgs[dp] = r.run(cu(torch, traj), cu(torch, dcf), cu(torch, kd)).cpu().numpy().astype(np.float64)
    lut = oracle.kb_lut(W, os_, 512)
    m64 = oracle.deapod_map_f64(dim, G, W, lut, out)
    mask = imgs[True] > 1e-3 * imgs[True].max()
    m_gpu = imgs[False][mask] / imgs[True][mask]
    err_map = rel_l2(m_gpu, m64[mask])
    ref = oracle.recon(traj, dcf, kd, dim, recon, os_, W, 512, out + ((1,) if dim == 2 else ()))
    err_img = rel_l2(imgs[True], ref.astype(np.float64) / m64)
    print(f"deapodization {dim}D G={G}: map vs FP64 oracle rel-L2 {err_map:.2e}, image vs reference / map "
          f"{err_img:.2e}, map range {m64.min():.3f}..{m64.max():.3f}")
    assert err_map <= 1e-5
    assert err_img <= 1e-5


# ----------------------------------------------------------------- PILS ----

def test_pils_ops_bit_exact(torch):
    """lowFilter / normalize / SOS(map) kernels against the reference's own
    ImageFilter outputs (tests/golden/pils_ops.npz), bit for bit."""
    import os
    import fastrecon_gb300 as fr
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "pils_ops.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files if k.endswith("_in")})
    for key in keys:
        dim, G = int(key.split("_")[0][1:]), int(key.split("_")[1][1:])
        x = z[key + "_in"]
        for res in (22, 5):
            xd = cu(torch, x)
            fr.gridding.low_filter(xd, dim, G, res)
            assert np.array_equal(bits(xd.cpu().numpy().view(np.float32)),
                                  bits(z[f"{key}_low{res}"].view(np.float32))), key
        xd = cu(torch, x)
        fr.gridding.normalize_channels(xd, dim, G)
        assert np.array_equal(bits(xd.cpu().numpy().view(np.float32)), bits(z[key + "_norm"].view(np.float32))), key
        rec = (G // 2, G // 2, G // 2 if dim == 3 else 1)
        out = fr.gridding.sos_map(cu(torch, x), cu(torch, z[key + "_map"]), dim, G, rec).cpu().numpy()
        assert np.array_equal(bits(out.view(np.float32)), bits(z[key + "_sosmap"].view(np.float32))), key


# ------------------------------------------------------ pruned transform ----

@pytest.mark.parametrize("dim,G,out", [(2, 64, (32, 32)), (2, 60, (40, 24)), (3, 30, (20, 20, 20)),
                                       (3, 40, (24, 16, 10)), (3, 48, (48, 48, 48)), (2, 384, (256, 256)),
                                       (3, 64, (40, 36, 32)), (2, 320, (256, 200)), (2, 160, (100, 100)),
                                       (3, 128, (100, 100, 100)), (2, 128, (64, 64)), (2, 192, (96, 160)),
                                       (2, 240, (128, 128)), (2, 256, (200, 180)), (2, 480, (300, 300)),
                                       (2, 512, (256, 256)), (2, 640, (400, 320)), (3, 160, (100, 80, 60)),
                                       (3, 192, (128, 128, 128)), (3, 240, (160, 150, 140))])
def test_pruned_fft_crop_sos_matches_cufft(torch, dim, G, out):
    """fr_fft_crop_sos on a checkerboard-modulated grid == cuFFT + fftShift +
    crop + SoS of the same grid."""
    import fastrecon_gb300 as fr
    rng = np.random.default_rng(G)
    C = 5
    g = (rng.standard_normal((C, G ** dim)) + 1j * rng.standard_normal((C, G ** dim))).astype(np.complex64)
    idx = np.indices((G,) * dim).sum(0).ravel()
    cb = (g * np.where(idx % 2, -1, 1)[None]).astype(np.complex64)
    want_d = cu(torch, g)
    size = (G, G, G if dim == 3 else 1)
    fr.FFT(dim, size, C, +1)(want_d)
    fr.fft_shift(want_d, dim, G)
    outs = tuple(out) + ((1,) if dim == 2 else ())
    want = fr.sos(want_d, dim, G, outs).cpu().numpy()
    got = fr.gridding.CropSoS(dim, G, C, outs)(cu(torch, cb)).cpu().numpy()
    assert rel_l2(got, want) <= TOL


def test_recon_cufft_path_vs_reference(torch):
    import fastrecon_gb300 as fr
    for name in ("radial2d_small", "koosh3d_small"):
        c = load_case(name)
        r = fr.Recon(c["dim"], c["recon"], c["os"], c["coils"], kernel_width=c["W"], lut_length=c["L"],
                     use_cufft=True)
        img = r.run(cu(torch, c["traj"]), cu(torch, c["dcf"]), cu(torch, c["kdata"])).cpu().numpy()
        assert rel_l2(img, c["image"]) <= TOL


def test_recon_pruned_fft_path_vs_reference(torch):
    import fastrecon_gb300 as fr
    for name in ("radial2d_small", "koosh3d_small"):
        c = load_case(name)
        r = fr.Recon(c["dim"], c["recon"], c["os"], c["coils"], kernel_width=c["W"], lut_length=c["L"],
                     pruned_fft=True)
        img = r.run(cu(torch, c["traj"]), cu(torch, c["dcf"]), cu(torch, c["kdata"])).cpu().numpy()
        assert rel_l2(img, c["image"]) <= TOL
