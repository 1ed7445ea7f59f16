"""CPU: the oracle reproduces the golden fixtures generated by the reference's
own compiled CPU code bit for bit, and its third-party stand-ins (I0, FFT)
agree with independent implementations."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_case, rel_l2


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_luts_bit_exact(oracle):
    z = np.load(os.path.join(GOLDEN, "luts.npz"))
    for key in z.files:
        w, o, l = key.split("_")
        lut = oracle.kb_lut(float(w[1:]), float(o[2:]), int(l[1:]))
        assert np.array_equal(bits(lut), bits(z[key])), key
        assert lut[0] == 1.0


def test_bessel_i0_vs_scipy(oracle):
    sp = pytest.importorskip("scipy.special")
    xs = np.linspace(0.0, 40.0, 401)
    got = np.array([oracle.lib.orc_bessel_i0(float(x)) for x in xs])
    assert np.max(np.abs(got / sp.i0(xs) - 1)) < 1e-13
    assert np.isnan(oracle.lib.orc_bessel_i0(float("nan")))


def test_normalize_bit_exact(oracle, case):
    tn, tr, sc, lo, hi = oracle.normalize_traj(case["traj"], case["dim"], case["G"])
    assert np.array_equal(bits(tn), bits(case["traj_norm"]))


def test_grid_bit_exact(oracle, case):
    tn = case["traj_norm"]
    g = oracle.grid(tn, case["dcf"], case["kdata"], case["dim"], case["G"], case["W"], case["lut"], threads=2)
    assert np.array_equal(bits(g.view(np.float32)), bits(case["grid"].view(np.float32)))


def test_recon_bit_exact(oracle, case):
    rec = (case["recon"],) * 2 + ((case["recon"] if case["dim"] == 3 else 1),)
    img = oracle.recon(case["traj"], case["dcf"], case["kdata"], case["dim"], case["recon"], case["os"], case["W"],
                       case["L"], rec, threads=2)
    assert np.array_equal(bits(img), bits(case["image"]))


def test_band_split_oracle_bit_exact(oracle, case):
    """The band-parallel gridding used for full-size checks gives the golden
    (reference-built) grid and image bit for bit, and the band-parallel FP64
    oracle equals the sequential one."""
    tn = case["traj_norm"]
    for threads in (1, 3, 8):
        g = oracle.grid_bands(tn, case["dcf"], case["kdata"], case["dim"], case["G"], case["W"], case["lut"],
                              threads=threads)
        assert np.array_equal(bits(g.view(np.float32)), bits(case["grid"].view(np.float32))), threads
    rec = (case["recon"],) * 2 + ((case["recon"] if case["dim"] == 3 else 1),)
    img = oracle.recon_bands(case["traj"], case["dcf"], case["kdata"], case["dim"], case["recon"], case["os"],
                             case["W"], case["L"], rec, threads=5)
    assert np.array_equal(bits(img), bits(case["image"]))
    g64 = oracle.grid_f64(tn, case["dcf"], case["kdata"], case["dim"], case["G"], case["W"], case["lut"])
    g64b = oracle.grid_f64_bands(tn, case["dcf"], case["kdata"], case["dim"], case["G"], case["W"], case["lut"],
                                 threads=7)
    assert np.array_equal(g64, g64b)


def test_fp64_oracle_close(oracle, case):
    """The FP32 reference grid vs the FP64 oracle: the reference's own
    rounding error, stated per fixture."""
    g64 = oracle.grid_f64(case["traj_norm"], case["dcf"], case["kdata"], case["dim"], case["G"], case["W"],
                          case["lut"])
    err = rel_l2(case["grid"], g64)
    print(f"{case['name']}: reference FP32 grid vs FP64 oracle rel-L2 = {err:.2e}")
    assert err < 1e-6


def test_fft_vs_numpy(oracle):
    rng = np.random.default_rng(3)
    for dim, G in [(2, 30), (2, 64), (3, 12), (3, 21)]:
        x = (rng.standard_normal((2, G ** dim)) + 1j * rng.standard_normal((2, G ** dim))).astype(np.complex64)
        got = oracle.fft(x, dim, G, +1, 2)
        shp = (2,) + (G,) * dim
        want = np.fft.ifftn(x.reshape(shp).astype(np.complex128), axes=tuple(range(1, dim + 1))) * G ** dim
        assert rel_l2(got.reshape(shp), want) < 1e-6


def test_shift_is_fftshift_for_even(oracle):
    rng = np.random.default_rng(4)
    for dim, G in [(2, 16), (3, 8)]:
        x = (rng.standard_normal(G ** dim) + 1j * rng.standard_normal(G ** dim)).astype(np.complex64)
        got = oracle.fft_shift(x, dim, G).reshape((G,) * dim)
        assert np.array_equal(got, np.fft.fftshift(x.reshape((G,) * dim)))


def test_sample_mass_matches_grid_sum(oracle):
    """sum over cells of the grid == sum_s dcf*data*mass(s) (linearity)."""
    c = load_case("koosh3d_small")
    m = oracle.sample_mass(c["traj_norm"], 3, c["G"], c["W"], c["lut"], 2)
    want = (c["dcf"].astype(np.float64)[None] * c["kdata"].astype(np.complex128) * m[None]).sum(1)
    got = c["grid"].astype(np.complex128).sum(1)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-5


def test_oracle_vs_reference_random(oracle):
    """Where the reference build exists, the oracle matches it on fresh random
    inputs too (not only on the stored fixtures)."""
    from oracle.pyoracle import RefLib
    if not RefLib.available():
        pytest.skip("reference build not present on this machine")
    ref = RefLib()
    rng = np.random.default_rng(11)
    n = 700
    for dim in (2, 3):
        t = np.zeros((n, 4), np.float32)
        t[:, :dim] = rng.uniform(-0.5, 0.5, (n, dim))
        dcf = rng.uniform(0, 1, n).astype(np.float32)
        kd = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
        g_ref, tn_ref = ref.grid(t, dcf, kd, n, 1, dim, 12, 1.5, 4.0, 512, 1)
        tn, *_ = oracle.normalize_traj(t, dim, 18)
        assert np.array_equal(bits(tn), bits(tn_ref))
        g = oracle.grid(tn, dcf, kd, dim, 18, 4.0, oracle.kb_lut(4.0, 1.5, 512))
        assert np.array_equal(bits(g.view(np.float32)), bits(g_ref.view(np.float32)))


def _pils_cases():
    z = np.load(os.path.join(GOLDEN, "pils_ops.npz"))
    for key in sorted({k.rsplit("_", 1)[0] for k in z.files if k.endswith("_in")}):
        dim, G = int(key.split("_")[0][1:]), int(key.split("_")[1][1:])
        yield key, dim, G, z


def test_pils_ops_bit_exact(oracle):
    """ImageFilter::lowFilter / normalize / SOS(map) restated bit-for-bit."""
    for key, dim, G, z in _pils_cases():
        x = z[key + "_in"]
        for res in (22, 5):
            assert np.array_equal(bits(oracle.low_filter(x, dim, G, res).view(np.float32)),
                                  bits(z[f"{key}_low{res}"].view(np.float32))), key
        assert np.array_equal(bits(oracle.normalize_channels(x, dim, G).view(np.float32)),
                              bits(z[key + "_norm"].view(np.float32))), key
        rec = (G // 2, G // 2, G // 2 if dim == 3 else 1)
        got = oracle.sos_map(x, z[key + "_map"], dim, G, rec)
        assert np.array_equal(bits(got.view(np.float32)), bits(z[key + "_sosmap"].view(np.float32))), key


def test_deapod_map_oracle_vs_fft(oracle):
    """The FP64 deapodization map (direct sum over the kernel's taps) equals
    the backward FFT of the taps seeded at the grid centre, fftShift-ed,
    cropped and normalised by the centre pixel (numpy FFT in float64)."""
    for dim, G, R, W, os_ in [(2, 64, 32, 4.0, 2.0), (2, 31, 16, 5.0, 2.0), (3, 24, 16, 4.0, 1.5)]:
        lut = oracle.kb_lut(W, os_, 512)
        got = oracle.deapod_map_f64(dim, G, W, lut, (R,) * dim)
        hw = np.float32(W) / np.float32(2)
        g = np.zeros((G,) * dim, np.float64)
        c0 = G // 2
        reach = int(np.ceil(hw)) + 1
        for d in np.ndindex(*((2 * reach + 1,) * dim)):
            d = [x - reach for x in d]
            dz = d[0] if dim == 3 else 0
            ki = oracle.lib.orc_tap_lut_index(float(d[-1]), float(d[-2]), float(dz), float(hw), len(lut))
            if ki >= 0:
                g[tuple(c0 + x for x in d)] = lut[ki]
        img = np.fft.fftshift(np.fft.ifftn(g) * g.size)
        off = (G - R) // 2
        crop = np.abs(img[(slice(off, off + R),) * dim]) / np.abs(img[(G // 2,) * dim])
        want = np.maximum(crop, 1e-6).ravel()
        assert np.max(np.abs(got - want)) < 1e-12, (dim, G)
