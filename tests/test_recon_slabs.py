"""Out-of-core coils (fr_recon_desc.grid_budget): the grid workspace holds a
slab of coils at a time; each slab's |x|^2 is added to the image in coil
order, so the image must equal the one made with every coil at once."""
import numpy as np
import pytest

from conftest import load_case, rel_l2


def _run(torch, c, budget, **kw):
    import fastrecon_gb300 as fr
    r = fr.Recon(c["dim"], c["recon"], c["os"], c["coils"], kernel_width=c["W"], lut_length=c["L"],
                 grid_budget=budget, **kw)
    img = r.run(torch.from_numpy(c["traj"]).cuda(), torch.from_numpy(c["dcf"]).cuda(),
                torch.from_numpy(c["kdata"]).cuda())
    return img.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "radial2d_oddgrid"])
@pytest.mark.parametrize("mode", [dict(), dict(use_cufft=True), dict(deapodize=True), dict(pruned_fft=True)])
def test_slabs_equal_single_pass(name, mode):
    import torch
    c = load_case(name)
    if c["coils"] < 2:
        pytest.skip("one coil")
    cells = c["G"] ** c["dim"]
    whole = _run(torch, c, 0, **mode)
    for coils_per_slab in (1, 2, c["coils"] - 1):
        got = _run(torch, c, coils_per_slab * cells * 8 + 7, **mode)
        assert rel_l2(got, whole) <= 1e-6, coils_per_slab
    # the reference image itself (parity bar of the recon tests)
    if not mode:
        assert rel_l2(_run(torch, c, cells * 8, **mode), c["image"]) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radial2d_small", "koosh3d_small", "radial2d_oddgrid", "koosh3d_odd"])
@pytest.mark.parametrize("coils_per_slab", [1, 2])
def test_slabs_vs_oracle(oracle, name, coils_per_slab):
    """Coils in slabs against the oracle's image (the reference pipeline,
    Program/Main.cpp:101-181) at the recon bar 1e-5, with and without the
    pruned register FFT."""
    import torch
    c = load_case(name)
    cells = c["G"] ** c["dim"]
    rec = (c["recon"],) * 2 + ((c["recon"] if c["dim"] == 3 else 1),)
    want = oracle.recon(c["traj"], c["dcf"], c["kdata"], c["dim"], c["recon"], c["os"], c["W"], c["L"], rec,
                        threads=2)
    for mode in (dict(), dict(use_cufft=True)):
        got = _run(torch, c, coils_per_slab * cells * 8, **mode)
        err = rel_l2(got, want)
        print(f"{name} {mode} {coils_per_slab} coil(s) per slab: image vs oracle rel-L2 {err:.2e}")
        assert err <= 1e-5


@pytest.mark.gpu
def test_slab_budget_smaller_than_one_coil_still_runs():
    import torch
    c = load_case("radial2d_small")
    whole = _run(torch, c, 0)
    assert rel_l2(_run(torch, c, 1), whole) <= 1e-6  # at least one coil per slab


@pytest.mark.gpu
@pytest.mark.parametrize("coils_per_slab", [1, 3, 4])
def test_slabs_3d_register_fft(coils_per_slab):
    """A 3D grid size with the register FFT stages (64^3), 5 coils."""
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    t = synth.kooshball_3d(300, 64)
    kd = synth.kspace(t, 3, 32, 5, seed=3, xp=torch, device="cuda")
    td = torch.from_numpy(t).cuda()
    dcf = fr.dcf_analytic(td, 3, 2.0)
    imgs = []
    for budget in (0, coils_per_slab * 64 ** 3 * 8):
        r = fr.Recon(3, 32, 2.0, 5, grid_budget=budget, deapodize=True)
        imgs.append(r.run(td, dcf, kd).cpu().numpy())
    assert rel_l2(imgs[1], imgs[0]) <= 1e-6


@pytest.mark.gpu
def test_register_fft_masks_unwritten_tiles():
    """The register FFT path leaves the grid's empty tiles unwritten and reads
    them as zero: after a run whose samples covered them, a run whose samples
    leave them empty must still equal the full-grid (cuFFT) path."""
    import torch

    import fastrecon_gb300 as fr
    from fastrecon_gb300 import synth
    a = synth.kooshball_3d(300, 64)
    b = a.copy()
    b[:, 2] *= 0.3  # flattened in z: tiles the first run filled are empty now
    rec = fr.Recon(3, 32, 2.0, 4)
    ref = fr.Recon(3, 32, 2.0, 4, use_cufft=True)
    for t in (a, b, a):
        td = torch.from_numpy(t).cuda()
        kd = synth.kspace(t, 3, 32, 4, seed=5, xp=torch, device="cuda")
        dcf = fr.dcf_analytic(td, 3, 2.0)
        got = rec.run(td, dcf, kd).cpu().numpy()
        want = ref.run(td, dcf, kd).cpu().numpy()
        assert rel_l2(got, want) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [dict(), dict(use_cufft=True)])
def test_submitted_volumes_with_slabs(mode):
    """fr_recon_submit_host with coils in slabs: equal to one
    fr_recon_run_host per volume."""
    import torch
    c = load_case("koosh3d_small")
    if c["coils"] < 2:
        pytest.skip("one coil")
    import fastrecon_gb300 as fr
    r = fr.Recon(c["dim"], c["recon"], c["os"], c["coils"], kernel_width=c["W"], lut_length=c["L"],
                 max_samples=c["traj"].shape[0], grid_budget=c["G"] ** 3 * 8, **mode)
    nout = int(np.prod(r.out_size))
    vols = [[torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
             for a in (c["traj"], c["dcf"], c["kdata"] * np.complex64(s))] for s in (1.0, -2.0, 0.5j)]
    want = []
    for v in vols:
        out = torch.empty(nout, dtype=torch.float32).pin_memory()
        want.append(r.run_host(*v, out).numpy().copy())
    got = [torch.empty(nout, dtype=torch.float32).pin_memory() for _ in vols]
    for v, out in zip(vols, got):
        r.submit_host(*v, out)
    r.sync()
    for g, w in zip(got, want):
        assert rel_l2(g.numpy(), w) <= 1e-6
    assert rel_l2(got[0].numpy(), c["image"]) <= 1e-5
