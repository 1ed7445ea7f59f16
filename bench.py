#!/usr/bin/env python
"""Headline benchmark: full non-Cartesian reconstruction of the 3D radial
kooshball workload (50,000 golden-means spokes x 256 samples = 12.8 M samples
per coil, 16 coils, 384^3 grid at oversampling 1.5, Kaiser-Bessel width 4,
LUT 512, 256^3 sum-of-squares output) on one GB300.

One step = normalise + bin the trajectory, grid all coils, batched backward
FFT (fftShift folded into the gridding flush), crop + sum of squares.
value = samples x coils gridded per second over the whole step (Msamples/s);
ms_per_step is the recon time.  Inputs (1.9 GB) exceed L2 (129 MB), so no
explicit L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU algorithm (the CPU oracle, a
C restatement of GridLut/ImageFilter, with the reference's OpenMP threading)
on this host's cores: every timed step is one complete recon of the same
workload, measured (about 15 s per kooshball step on 16 cores).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s gridded; recon ms; learned vs Pipe-DCF time at NRMSE≤1%"
UNIT = "Msamples/s"
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "kooshball3d": dict(dim=3, spokes=50000, readout=256, coils=16, recon=256, os=1.5, width=4.0, lut=512,
                        dcf_power=2.0,
                        desc="3D radial kooshball: 50,000 golden-means spokes x 256 samples (12.8 M/coil), "
                             "16 coils, |k|^2 DCF, KB width 4, LUT 512, os 1.5 -> 384^3 grid, 256^3 SoS"),
    # reduced kooshball with the same sample-density profile, for ncu captures
    "kooshball3d_prof": dict(dim=3, spokes=12500, readout=128, coils=16, recon=128, os=1.5, width=4.0, lut=512,
                             dcf_power=2.0,
                             desc="reduced 3D kooshball for profiling: 12,500 golden-means spokes x 128 samples, "
                                  "16 coils, os 1.5 -> 192^3 grid"),
    # the kooshball's 384^3 transform with 2 coils (0.9 GB grid), for ncu captures of the FFT stages
    "kooshball3d_fft": dict(dim=3, spokes=2000, readout=256, coils=2, recon=256, os=1.5, width=4.0, lut=512,
                            dcf_power=2.0,
                            desc="3D kooshball, 2,000 spokes x 256, 2 coils, os 1.5 -> 384^3 grid (FFT profiling)"),
    "radial2d": dict(dim=2, spokes=256, readout=512, coils=8, recon=256, os=2.0, width=4.0, lut=512,
                     dcf_power=1.0,
                     desc="2D radial: 256 spokes x 512 samples, 8 coils, |k| DCF, KB width 4, LUT 512, "
                          "os 2 -> 512^2 grid, 256^2 SoS"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="kooshball3d")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-spiral and learned-vs-Pipe DCF measurements")
    ap.add_argument("--profile", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (ncu --profile-from-start off)")
    return ap.parse_args()


def dist_env():
    from fastrecon_gb300 import replicas
    return replicas.env()


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.strip().split(",") for r in self.f.read().splitlines() if r.strip()]
        self.f.close()
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(w, torch, device):
    import numpy as np

    from fastrecon_gb300 import synth
    traj = synth.radial_2d(w["spokes"], w["readout"]) if w["dim"] == 2 else \
        synth.kooshball_3d(w["spokes"], w["readout"])
    dcf = synth.ramp_dcf(traj, w["dim"], w["dcf_power"])
    kd = synth.kspace(traj, w["dim"], w["recon"], w["coils"], seed=0, xp=torch, device=device)
    return (torch.from_numpy(traj).to(device), torch.from_numpy(dcf).to(device), kd, np.float32)


def scatter_kernel(taps: bool, coils: int) -> str:
    """The scatter kernel the recon launches: with tap lists, the tap-lane
    scatter for coil groups of 16 (9 coils and more) unless
    FR_SCATTER_WARP_LISTS=1, the per-warp tap-list scatter otherwise."""
    if not taps:
        return "grid_tiles_kernel"
    if coils > 8 and os.environ.get("FR_SCATTER_WARP_LISTS", "0") in ("", "0"):
        return "grid_lanes_kernel"
    return "grid_taps_kernel"


def algorithmic_bytes(w):
    """Gridding algorithmic bytes per launch: coordinates (4d B) + DCF (4 B)
    per sample, 8 B per sample and coil, 8 B per grid cell and coil written
    once."""
    import numpy as np
    N = w["spokes"] * w["readout"]
    G = int(np.float32(w["recon"]) * np.float32(w["os"]))
    d, C = w["dim"], w["coils"]
    return N * (4 * d + 4) + N * C * 8 + C * G ** d * 8


# --------------------------------------------------------------------------
# The reference's CPU path (the oracle, a C restatement of the reference's
# algorithm), timed on this host's cores: the reference arm and cpu_baseline
# --------------------------------------------------------------------------

def ref_inputs(w):
    """The workload's raw trajectory, DCF and k-space as host arrays, from the
    same seeded generator as the measured arm.  The k-space is synthesised on
    the GPU when one is present (input synthesis only: nothing of the timed
    region runs there) and copied to host memory."""
    from fastrecon_gb300 import synth
    traj = synth.radial_2d(w["spokes"], w["readout"]) if w["dim"] == 2 else \
        synth.kooshball_3d(w["spokes"], w["readout"])
    dcf = synth.ramp_dcf(traj, w["dim"], w["dcf_power"])
    try:
        import torch
        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    if gpu:
        kd = synth.kspace(traj, w["dim"], w["recon"], w["coils"], seed=0, xp=torch, device="cuda").cpu().numpy()
        torch.cuda.empty_cache()
    else:
        kd = synth.kspace(traj, w["dim"], w["recon"], w["coils"], seed=0)
    return traj, dcf, kd


class RefRecon:
    """One reconstruction as Program/Main.cpp:101-181 runs it, with the
    reference's threading, on the CPU oracle:
    * ReconData::normalizeTraj, one thread (ReconData.cpp:201-225);
    * GridLut::execute: OpenMP over coils, threads = min(coils, cores)
      (GridLut.cpp:53-78, Main.cpp:111);
    * ImageFilter::fftExecute: one single-threaded backward FFT per coil,
      coils spread over the host threads (FFT.cpp:56-90).  FFTW3f is absent
      on these hosts: scipy.fft (pocketfft, single precision, unnormalised
      backward transform) stands in for it;
    * ImageFilter::fftShift: the reference's swap loops per coil, coils over
      the threads (ImageFilter.cpp:40-53);
    * ImageFilter::SOS, one thread (ImageFilter.cpp:159-209), then |.|."""

    def __init__(self, w, traj, dcf, kd):
        import numpy as np

        from oracle.pyoracle import Oracle
        self.o = Oracle()
        self.w, self.traj, self.dcf, self.kd = w, traj, dcf, np.ascontiguousarray(kd, np.complex64)
        self.dim = w["dim"]
        self.G = int(np.float32(w["recon"]) * np.float32(w["os"]))
        self.lut = self.o.kb_lut(w["width"], w["os"], w["lut"])
        self.ncpu = os.cpu_count() or 1
        self.tg = min(w["coils"], self.ncpu)
        self.rec = (w["recon"], w["recon"], w["recon"] if self.dim == 3 else 1)
        try:
            import scipy.fft as sfft
            self.sfft = sfft
            self.fft_desc = "scipy.fft (pocketfft, complex64, one thread per coil) standing in for FFTW3f"
        except ImportError:
            self.sfft = None
            self.fft_desc = "the oracle's FP64 mixed-radix FFT standing in for FFTW3f"

    def _fft_one(self, g):
        if self.sfft is None:
            g[:] = self.o.fft(g[None], self.dim, self.G, +1, 1)[0]
            return
        shp = (self.G,) * self.dim
        g.reshape(shp)[...] = self.sfft.ifftn(g.reshape(shp), norm="forward", workers=1)

    def step(self, n=None, fft_coils=None):
        """One recon (of the first n samples and fft_coils coils when given:
        warm-up only); returns seconds per stage."""
        from concurrent.futures import ThreadPoolExecutor
        w, o, dim, G = self.w, self.o, self.dim, self.G
        n = n or self.traj.shape[0]
        t0 = time.perf_counter()
        tn, *_ = o.normalize_traj(self.traj[:n], dim, G)
        grid = o.grid(tn, self.dcf[:n], self.kd[:, :n], dim, G, w["width"], self.lut, threads=self.tg)
        t1 = time.perf_counter()
        cs = range(fft_coils if fft_coils is not None else grid.shape[0])
        with ThreadPoolExecutor(self.ncpu) as ex:
            list(ex.map(lambda c: self._fft_one(grid[c]), cs))
            t2 = time.perf_counter()
            list(ex.map(lambda c: o.fft_shift_inplace(grid[c], dim, G), cs))
        t3 = time.perf_counter()
        img = abs(o.sos(grid, dim, G, self.rec).real)
        t4 = time.perf_counter()
        del grid, img
        return {"grid": t1 - t0, "fft": t2 - t1, "shift": t3 - t2, "sos": t4 - t3, "total": t4 - t0}

    def describe(self, warm):
        w = self.w
        return (f"complete recon per step: all {w['spokes']} spokes x {w['readout']} samples x {w['coils']} coils "
                f"gridded ({self.tg} threads, OpenMP over coils as GridLut::execute), backward FFT of every coil "
                f"({self.fft_desc}; coils over {self.ncpu} threads as FFT.cpp), fftShift per coil, SOS; measured, "
                f"not extrapolated{warm}")


def fp64_errors(w, traj, dcf, kd, torch):
    """GPU grid (fr_grid, default tiling and work items) vs the oracle's FP64
    gridding and its FP32 restatement of the reference, on the first 2 coils
    of the workload (in the workload's coil group: the benchmark's scatter
    kernel) and on the whole 2D radial configuration."""
    import numpy as np

    import fastrecon_gb300 as fr
    from oracle.pyoracle import Oracle
    o = Oracle()

    def rel(a, b):
        a = np.asarray(a).astype(np.complex128).ravel()
        b = np.asarray(b).astype(np.complex128).ravel()
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    out = {}
    # the workload's 2 coils in the coil group the recon uses for all of its
    # coils, so that they go through the same scatter kernel as the benchmark
    cg = 4
    while cg < w["coils"] and cg < 16:
        cg *= 2
    cases = [(w, traj, dcf, kd[:2], f"{w['desc'].split(':')[0]}, 2 of {w['coils']} coils")]
    if w is not WORKLOADS["radial2d"]:
        r2 = WORKLOADS["radial2d"]
        t2, d2, k2, _ = make_inputs(r2, torch, traj.device)
        cases.append((r2, t2, d2, k2, "2D radial 256 x 512, 8 coils"))
    for wk, t, d, k, name in cases:
        G = fr.grid_size(wk["recon"], wk["os"])
        lut = o.kb_lut(wk["width"], wk["os"], wk["lut"])
        plan = fr.GridPlan(wk["dim"], G, wk["width"], lut=lut, coil_group=cg if wk is w else 0)
        plan.set_trajectory(t)
        g = plan.grid(k.contiguous(), d).cpu().numpy()
        del plan
        tn, *_ = o.normalize_traj(t.cpu().numpy(), wk["dim"], G)
        kn = k.cpu().numpy()
        g64 = o.grid_f64_bands(tn, d.cpu().numpy(), kn, wk["dim"], G, wk["width"], lut)
        ref = o.grid_bands(tn, d.cpu().numpy(), kn, wk["dim"], G, wk["width"], lut)
        out[name] = {"gpu_vs_fp64": rel(g, g64), "gpu_vs_reference_fp32": rel(g, ref),
                     "reference_fp32_vs_fp64": rel(ref, g64)}
        del g, g64, ref
    return out


def run_reference(args, w):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    traj, dcf, kd = ref_inputs(w)
    r = RefRecon(w, traj, dcf, kd)
    # warm-up steps (untimed): a small slice of the gridding and one coil's
    # transform, enough to page in the code and start the thread pools
    n_warm = max(w["readout"], (w["spokes"] // 64) * w["readout"])
    for _ in range(args.warmup):
        r.step(n=n_warm, fft_coils=1)
    stages = []
    for _ in range(args.steps):
        stages.append(r.step())
    t = statistics.mean(s["total"] for s in stages)
    N = w["spokes"] * w["readout"]
    value = N * w["coils"] / t / 1e6
    stage_ms = {k: 1e3 * statistics.mean(s[k] for s in stages) for k in stages[0]}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "samples_per_coil": N, "coils": w["coils"]},
            "stage_ms": stage_ms,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": r.ncpu, "kind": "port",
                             "sample": r.describe("; warm-up steps: 1/64 of the spokes and one coil's FFT")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference CPU algorithm (the oracle's C restatement of GridLut/ImageFilter, pinned bit for bit "
                    "to the reference's own CPU sources where they build; those need Qt/GSL/FFTW and are not "
                    "carried to this host)"}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
# Our arm
# --------------------------------------------------------------------------

def run_ours(args, w):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    __graft_entry__.build()
    import fastrecon_gb300 as fr

    dev = torch.device("cuda", local)
    traj, dcf, kd, _ = make_inputs(w, torch, dev)
    N = traj.shape[0]
    C = w["coils"]
    dim = w["dim"]
    G = fr.grid_size(w["recon"], w["os"])
    out_size = (w["recon"], w["recon"], w["recon"] if dim == 3 else 1)
    rec = fr.Recon(dim, w["recon"], w["os"], C, out_size=out_size, kernel_width=w["width"], lut_length=w["lut"],
                   max_samples=N)
    img = torch.empty(int(np.prod(out_size)), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(max(3, args.warmup)):
        rec.run(traj, dcf, kd, out=img)
    rec.profile(True)
    rec.profile_read()
    barrier()
    clocks = Clocks(local) if rank == 0 else None
    time.sleep(0.2 if clocks else 0)
    l0 = fr.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if args.profile:
        torch.cuda.profiler.start()
    e0.record(stream)
    for _ in range(args.steps):
        rec.run(traj, dcf, kd, out=img)
    e1.record(stream)
    barrier()
    if args.profile:
        torch.cuda.profiler.stop()
    ck = clocks.stop() if clocks else None
    launches = fr.kernel_launches() - l0
    elapsed = e0.elapsed_time(e1)  # ms
    scatter_ms, scatter_n = rec.profile_read()
    rec.profile(False)
    taps = rec.tap_words() > 0
    from fastrecon_gb300 import replicas
    elapsed = replicas.max_over_ranks(elapsed, dist, device=dev)  # replicas: the slowest rank's time
    ms = elapsed / args.steps
    value = ws * N * C * args.steps / (elapsed / 1e3) / 1e6

    # stage breakdown (separate pass with per-stage events)
    os.environ["FR_TIMING"] = "1"
    rec_t = fr.Recon(dim, w["recon"], w["os"], C, out_size=out_size, kernel_width=w["width"], lut_length=w["lut"],
                     max_samples=N)
    os.environ.pop("FR_TIMING")
    stages = []
    for _ in range(3):
        rec_t.run(traj, dcf, kd, out=img)
        stages.append(rec_t.stage_ms())
    del rec_t
    stage_ms = {k: statistics.median(s[k] for s in stages) for k in stages[0]}

    # end to end through the host-buffer C-ABI call
    e2e = None
    if not args.no_e2e:
        h_traj = traj.cpu().pin_memory()
        h_dcf = dcf.cpu().pin_memory()
        h_kd = kd.cpu().pin_memory()
        h_img = torch.empty(img.shape[0], dtype=torch.float32).pin_memory()
        for _ in range(2):
            rec.run_host(h_traj, h_dcf, h_kd, h_img)
        barrier()
        k2 = max(3, min(args.steps, 40))
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(k2):
            rec.run_host(h_traj, h_dcf, h_kd, h_img)
        e1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
        el2 = e0.elapsed_time(e1)
        el2 = replicas.max_over_ranks(el2, dist, device=dev)
        # the same volumes submitted back to back (fr_recon_submit_host): each
        # step's upload and the previous image's download overlap the recon
        # of the step before; one sync after the last step
        for _ in range(2):
            rec.submit_host(h_traj, h_dcf, h_kd, h_img)
        rec.sync()
        barrier()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(k2):
            rec.submit_host(h_traj, h_dcf, h_kd, h_img)
        rec.sync()
        e1.record(stream)
        barrier()
        wall_p = time.perf_counter() - t0
        el3 = e0.elapsed_time(e1)
        el3 = replicas.max_over_ranks(el3, dist, device=dev)
        e2e = {"value": ws * N * C * k2 / (el3 / 1e3) / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": int(h_traj.numel() * 4 + h_dcf.numel() * 4 + h_kd.numel() * 8),
               "d2h_bytes_per_step": int(h_img.numel() * 4), "ms_per_step": el3 / k2,
               "wall_ms_per_step": wall_p * 1e3 / k2, "steps": k2,
               "api": "fr_recon_submit_host x steps + fr_recon_sync (pipelined host-buffer volumes)",
               "one_call": {"value": ws * N * C * k2 / (el2 / 1e3) / 1e6, "ms_per_step": el2 / k2,
                            "wall_ms_per_step": wall * 1e3 / k2,
                            "api": "fr_recon_run_host per step (returns with the image)"}}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = measured_peak()
    algo = algorithmic_bytes(w)
    per_launch_ms = scatter_ms / max(scatter_n, 1)
    achieved = algo / (per_launch_ms / 1e3) / 1e9
    traffic = None
    kernel = scatter_kernel(taps, C)
    tr_path = os.path.join(ROOT, "profiles", kernel.replace("_kernel", "") + "_traffic.txt")
    if os.path.exists(tr_path):
        for line in open(tr_path):
            if line.startswith(args.workload + " "):
                traffic = float(line.split()[1])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded trajectory; exact k-space of a Gaussian-profile ellipsoid phantom x Gaussian "
                "coil maps, 1% complex noise",
        "config": {"workload": w["desc"], "samples_per_coil": N, "coils": C, "grid": G,
                   "l2": (f"inputs {N * (20 + 8 * C) / 1e9:.2f} GB per step exceed the 129 MB L2; no flush needed"
                          if N * (20 + 8 * C) > 129e6 else "inputs smaller than the 129 MB L2; steps back to back"),
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "recon_ms": ms,
        "stage_ms": stage_ms,
        "roofline": {"bound": "hbm",
                     "kernel": kernel + (" (KB scatter from the plan's tap lists)" if taps else " (KB scatter)"),
                     "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": algo, "kernel_ms": per_launch_ms, "launches": scatter_n,
                     "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s"},
        "gpu_launches": int(launches),
        "clocks": ck,
        "e2e": e2e,
    }
    if not args.no_cpu_baseline and ws == 1:
        # one complete recon of the same workload by the reference's CPU
        # algorithm on this host (a bounded sample of the CPU work: ~15 s)
        r = RefRecon(w, traj.cpu().numpy(), dcf.cpu().numpy(), kd.cpu().numpy())
        r.step(n=max(w["readout"], (w["spokes"] // 64) * w["readout"]), fft_coils=1)
        st = r.step()
        line["cpu_baseline"] = {"value": N * C / st["total"] / 1e6, "unit": UNIT, "cores": r.ncpu, "kind": "port",
                                "sample": r.describe(" (one step, after a small warm-up)"),
                                "ms_per_step": st["total"] * 1e3,
                                "stage_ms": {k: v * 1e3 for k, v in st.items()}}
        del r
        # the oracle as checker: relative L2 error of the GPU grid against
        # the FP64 gridding oracle and against the reference's FP32
        # algorithm, for this workload (2 of its coils) and the 2D radial
        line["fp64_rel_l2"] = fp64_errors(w, traj, dcf, kd, torch)
    if not args.no_extras and ws == 1:
        import bench_extras
        del rec, traj, dcf, kd
        torch.cuda.empty_cache()
        for key, fn in (("radial2d", bench_extras.radial2d), ("batched_spiral", bench_extras.batched_spiral),
                        ("learned_dcf", bench_extras.learned_vs_pipe)):
            try:
                line[key] = fn(torch)
            except Exception as e:  # reported, not fatal: the headline line stands
                line[key] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
