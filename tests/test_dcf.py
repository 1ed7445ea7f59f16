"""Density compensation and degridding (no counterpart in the reference):
analytic |k|^p DCF, degridding (the adjoint of gridding), real-valued
gridding and the Pipe-Menon iteration.  The oracle is the FP64 CPU
restatement in oracle/fr_oracle_ext.c; CPU tests pin it with identities of
the published algorithm (adjointness, the Pipe-Menon fixed point), GPU tests
compare the kernels with it."""
import numpy as np
import pytest

from conftest import CASE_NAMES, load_case, rel_l2
from fastrecon_gb300 import synth

TOL_GRID = 1e-5   # FP32 accumulation vs FP64 oracle
TOL_PIPE = 1e-4   # 20 FP32 iterations vs FP64 oracle


def _case_with_norm(oracle, name):
    c = load_case(name)
    return c, c["traj_norm"].astype(np.float32)


# ---------------------------------------------------------------- oracle (CPU)

def test_oracle_analytic_dcf_matches_numpy(oracle):
    t = synth.radial_2d(16, 64)
    for p in (1.0, 2.0):
        assert np.array_equal(oracle.dcf_analytic(t, 2, p), synth.ramp_dcf(t, 2, p))
    t3 = synth.kooshball_3d(40, 32)
    assert np.array_equal(oracle.dcf_analytic(t3, 3, 2.0), synth.ramp_dcf(t3, 3, 2.0))


@pytest.mark.parametrize("name", CASE_NAMES)
def test_oracle_degrid_is_adjoint_of_grid(oracle, name):
    """<grid(k), g> = <k, degrid(g)> for the real kernel matrix (dcf = 1)."""
    c, tn = _case_with_norm(oracle, name)
    rng = np.random.default_rng(3)
    n = tn.shape[0]
    k = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    cells = c["G"] ** c["dim"]
    g = rng.standard_normal(cells) + 1j * rng.standard_normal(cells)
    gk = oracle.grid_f64(tn, np.ones(n, np.float32), k[None], c["dim"], c["G"], c["W"], c["lut"])[0]
    dg = oracle.degrid_f64(tn, g[None], c["dim"], c["G"], c["W"], c["lut"])[0]
    lhs = np.vdot(g, gk)
    rhs = np.vdot(dg, k.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1.0)


def test_oracle_pipe_reaches_fixed_point(oracle):
    """After the iteration, degrid(grid(w)) is close to 1 at every sample."""
    t = synth.radial_2d(32, 64)
    tn = oracle.normalize_traj(t, 2, 64)[0]
    lut = oracle.kb_lut(4.0, 2.0, 512)
    w = oracle.dcf_pipe_f64(tn, 2, 64, 4.0, lut, 30)
    g = oracle.grid_real_f64(tn, w, 2, 64, 4.0, lut)
    p = oracle.degrid_f64(tn, g.astype(np.complex128)[None], 2, 64, 4.0, lut)[0].real
    assert np.median(np.abs(p - 1)) < 0.02
    # the radial density ~1/|k|: Pipe weights grow with |k| away from the centre
    r = np.hypot(t[:, 0], t[:, 1])
    assert np.corrcoef(r, w)[0, 1] > 0.8


def test_oracle_density_counts_bruteforce(oracle):
    t = synth.golden_angle_2d(24, 32)
    G = 48
    tn = oracle.normalize_traj(t, 2, G)[0]
    radii = [1, 2, 4, 8]
    cnt = oracle.density_counts(tn, 2, G, radii)
    cell = np.clip(np.floor(tn[:, :2] + np.float32(0.5)).astype(np.int64), 0, G - 1)
    for s in (0, 5, 100, len(tn) - 1):
        for k, r in enumerate(radii):
            inside = np.all(np.abs(cell - cell[s]) <= r, axis=1)
            assert cnt[s, k] == inside.sum()


# ---------------------------------------------------------------- GPU kernels

@pytest.mark.gpu
def test_gpu_analytic_dcf_bit_exact(oracle):
    import torch

    import fastrecon_gb300 as fr
    for t, dim in ((synth.radial_2d(64, 128), 2), (synth.kooshball_3d(100, 64), 3)):
        td = torch.from_numpy(t).cuda()
        for p in (1.0, 2.0):
            got = fr.dcf_analytic(td, dim, p).cpu().numpy()
            assert np.array_equal(got, oracle.dcf_analytic(t, dim, p))
        got = fr.dcf_analytic(td, dim, 1.5).cpu().numpy()
        want = oracle.dcf_analytic(t, dim, 1.5)
        assert np.max(np.abs(got - want) / np.maximum(want, 1e-30)) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASE_NAMES)
@pytest.mark.parametrize("checkerboard", [False, True])
def test_gpu_degrid_matches_oracle(oracle, name, checkerboard):
    import torch

    import fastrecon_gb300 as fr
    c, tn = _case_with_norm(oracle, name)
    if checkerboard and c["G"] % 2:
        pytest.skip("checkerboard plans need an even grid")
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"], checkerboard=checkerboard)
    plan.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    g = c["grid"].reshape(c["coils"], -1).astype(np.complex64)
    got = plan.degrid(torch.from_numpy(g).cuda()).cpu().numpy()
    gin = g.astype(np.complex128)
    if checkerboard:
        G = c["G"]
        idx = np.indices((G,) * c["dim"]).sum(0)  # (z, y, x) sum, parity only
        gin = gin * np.where(idx.ravel() % 2, -1.0, 1.0)[None]
    want = oracle.degrid_f64(tn, gin, c["dim"], c["G"], c["W"], c["lut"])
    assert rel_l2(got, want) <= TOL_GRID


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASE_NAMES)
def test_gpu_grid_real_matches_oracle(oracle, name):
    import torch

    import fastrecon_gb300 as fr
    c, tn = _case_with_norm(oracle, name)
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"])
    plan.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    w = c["dcf"].astype(np.float32)
    got = plan.grid_real(torch.from_numpy(w).cuda()).cpu().numpy()
    want = oracle.grid_real_f64(tn, w.astype(np.float64), c["dim"], c["G"], c["W"], c["lut"])
    assert rel_l2(got, want) <= TOL_GRID


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "spiral2d_w3", "radial2d_oddgrid"])
def test_gpu_pipe_matches_oracle(oracle, name):
    import torch

    import fastrecon_gb300 as fr
    c, tn = _case_with_norm(oracle, name)
    plan = fr.GridPlan(c["dim"], c["G"], c["W"], lut=c["lut"])
    plan.set_trajectory(torch.from_numpy(c["traj"]).cuda())
    got = plan.dcf_pipe(20).cpu().numpy()
    want = oracle.dcf_pipe_f64(tn, c["dim"], c["G"], c["W"], c["lut"], 20)
    assert rel_l2(got, want) <= TOL_PIPE


@pytest.mark.gpu
def test_gpu_pipe_medium_split_tiles(oracle):
    """A trajectory dense enough that centre tiles are split into several
    work items (partial tiles) still matches the FP64 iteration."""
    import torch

    import fastrecon_gb300 as fr
    t = synth.radial_2d(256, 128)
    G = 128
    lut = oracle.kb_lut(4.0, 2.0, 512)
    plan = fr.GridPlan(2, G, 4.0, lut=lut, chunk=1024)
    plan.set_trajectory(torch.from_numpy(t).cuda())
    assert plan.stats()["slots"] > 0
    got = plan.dcf_pipe(20).cpu().numpy()
    tn = oracle.normalize_traj(t, 2, G)[0]
    want = oracle.dcf_pipe_f64(tn, 2, G, 4.0, lut, 20)
    assert rel_l2(got, want) <= TOL_PIPE
