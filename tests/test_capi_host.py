"""CPU: the C-ABI library builds, loads, exports every symbol the header
declares, and its host-only entry points behave (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np

from conftest import GOLDEN, ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "fastrecon_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long|size_t|const char \*)\s*(fr_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ["fr_kb_lut", "fr_plan_create", "fr_plan_set_trajectory", "fr_grid", "fr_fft_create", "fr_sos",
              "fr_recon_run", "fr_recon_run_host"]:
        assert s in syms


def test_library_exports_all_declared_symbols(frlib):
    from fastrecon_gb300 import capi
    for s in header_symbols():
        assert hasattr(frlib, s), s
    assert set(header_symbols()) <= set(capi.exported_symbols()) | set(header_symbols())
    for s in capi.exported_symbols():
        assert s in header_symbols(), f"binding {s} not declared in the header"


def test_kb_lut_matches_reference_luts(frlib):
    import fastrecon_gb300 as fr
    z = np.load(os.path.join(GOLDEN, "luts.npz"))
    for key in z.files:
        w, o, l = key.split("_")
        lut = fr.kb_lut(float(w[1:]), float(o[2:]), int(l[1:]))
        assert np.array_equal(lut.view(np.uint32), z[key].view(np.uint32)), key


def test_status_strings(frlib):
    for s in range(10):
        assert frlib.fr_status_string(s)
    assert frlib.fr_status_string(0) == b"ok"
    assert b"0.1" in frlib.fr_version()


def test_argument_validation_without_gpu(frlib):
    """Invalid descriptors are rejected before any CUDA call."""
    from fastrecon_gb300 import capi
    lut = (C.c_float * 512)()
    d = capi.PlanDesc()
    d.dim = 4
    d.grid_size = 64
    d.kernel_width = 4.0
    d.lut_length = 512
    d.lut = C.cast(lut, C.POINTER(C.c_float))
    h = C.c_void_p()
    assert frlib.fr_plan_create(C.byref(d), C.byref(h)) == 1  # FR_ERR_INVALID_ARGUMENT
    assert b"dim" in frlib.fr_last_error()
    d.dim = 2
    d.grid_size = 0
    assert frlib.fr_plan_create(C.byref(d), C.byref(h)) == 7  # FR_ERR_UNSUPPORTED
    d.grid_size = 64
    d.lut_length = 1
    assert frlib.fr_plan_create(C.byref(d), C.byref(h)) == 1
    assert frlib.fr_kb_lut(4.0, 2.0, 1, lut) == 1
    assert frlib.fr_grid(None, None, None, 1, None, None) == 1
    assert frlib.fr_fft_create(5, None, 1, 1, C.byref(h)) == 1
    rd = capi.ReconDesc()
    rd.dim = 2
    rd.channels = 0
    assert frlib.fr_recon_create(C.byref(rd), C.byref(h)) == 1
    # host-buffer entry points: null handles and buffers are rejected up front
    assert frlib.fr_recon_run_host(None, None, None, None, 0, None, None) == 1
    assert frlib.fr_recon_submit_host(None, None, None, None, 0, None, None) == 1
    assert frlib.fr_recon_sync(None, None) == 1


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from fastrecon_gb300 import capi
    try:
        capi.load(str(tmp_path / "missing.so"))
    except capi.FastreconError as e:
        assert "not built" in str(e)
    else:
        raise AssertionError("loading a missing library must raise")


def lut_table(frlib, W, L):
    thr = (C.c_float * (L + 1))()
    smax, kc = C.c_float(), C.c_float()
    assert frlib.fr_lut_index_table(W, L, thr, C.byref(smax), C.byref(kc)) == 0
    return np.frombuffer(thr, np.float32).copy(), np.float32(smax.value), np.float32(kc.value)


def device_lookup(s, thr, smax, kc, L, rel_err):
    """The scatter kernel's index: approximate sqrt (relative error rel_err),
    k0 = (int)fma(a, kc, 0.25) clamped to L-1, +1 when s >= thr[k0+1]."""
    a = (np.sqrt(s.astype(np.float64)) * (1.0 + rel_err)).astype(np.float32)
    g = (a.astype(np.float64) * np.float64(kc) + np.float64(np.float32(0.25))).astype(np.float32)
    k0 = np.minimum(g.astype(np.int64), L - 1)
    k = k0 + (s >= thr[k0 + 1]).astype(np.int64)
    return np.where(s < smax, k, -1)


def test_lut_index_table_is_exact(frlib, oracle):
    """The square-root-free LUT index of the scatter kernel equals the
    reference's roundf(sqrtf(s)/kHW*(L-1)) for every threshold, its float
    neighbours, the kernel edge and random s, with the approximate square
    root off by up to 2^-20 relative in either direction."""
    rng = np.random.default_rng(0)
    for W, L in [(4.0, 512), (4.0, 32), (5.0, 32), (3.0, 64), (6.0, 1024), (4.5, 512), (4.0, 4096)]:
        thr, smax, kc = lut_table(frlib, W, L)
        fin = thr[np.isfinite(thr)]
        cand = [fin, np.nextafter(fin, np.float32(0)), np.nextafter(fin, np.float32(np.inf)),
                np.array([0.0, smax, np.nextafter(smax, np.float32(0)), np.nextafter(smax, np.float32(np.inf))],
                         np.float32),
                rng.uniform(0, float(smax) * 1.05, 200000).astype(np.float32),
                (rng.uniform(0, 1, 50000) ** 4 * float(smax)).astype(np.float32)]
        s = np.abs(np.concatenate(cand)).astype(np.float32)
        want = oracle.lut_index_of_s(s, W / 2, L)
        for err in (-2.0 ** -20, 0.0, 2.0 ** -20):
            got = device_lookup(s, thr, smax, kc, L, err)
            bad = np.nonzero(got != want)[0]
            assert bad.size == 0, (W, L, err, s[bad[:5]], got[bad[:5]], want[bad[:5]])
