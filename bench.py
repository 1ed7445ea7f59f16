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
C restatement of GridLut/ImageFilter, OpenMP) on this host's cores on a
bounded sample of the same workload and extrapolates a full step.
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
# CPU baseline: the oracle (reference algorithm) on a bounded sample
# --------------------------------------------------------------------------

def cpu_step(w, traj, dcf, kd, threads_grid, threads_fft, spoke_frac, fft_coils):
    """One bounded CPU recon step; returns (extrapolated full-step seconds,
    description)."""
    import numpy as np

    from oracle.pyoracle import Oracle
    o = Oracle()
    R = w["readout"]
    S = max(1, int(w["spokes"] * spoke_frac))
    n = S * R
    N = w["spokes"] * R
    C = w["coils"]
    dim = w["dim"]
    G = int(np.float32(w["recon"]) * np.float32(w["os"]))
    lut = o.kb_lut(w["width"], w["os"], w["lut"])
    t0 = time.perf_counter()
    tn, *_ = o.normalize_traj(traj[:n], dim, G)
    grid = o.grid(tn, dcf[:n], kd[:, :n], dim, G, w["width"], lut, threads=threads_grid)
    t1 = time.perf_counter()
    sub = o.fft(grid[:fft_coils], dim, G, +1, threads_fft)
    for c in range(fft_coils):
        sub[c] = o.fft_shift(sub[c], dim, G)
    t2 = time.perf_counter()
    rec = (w["recon"], w["recon"], w["recon"] if dim == 3 else 1)
    o.sos(grid, dim, G, rec)
    t3 = time.perf_counter()
    full = (t1 - t0) * (N / n) + (t2 - t1) * (C / fft_coils) + (t3 - t2)
    desc = (f"{S} of {w['spokes']} spokes x {R} samples x {C} coils gridded ({threads_grid} threads, OpenMP over "
            f"coils as GridLut::execute), backward FFT + fftShift of {fft_coils} of {C} coils (oracle mixed-radix "
            f"FFT, stand-in for FFTW3f, {threads_fft} threads), SoS of all coils; full step extrapolated linearly "
            f"(grid x {N / n:.1f}, FFT x {C / fft_coils:.1f})")
    return full, desc, (t3 - t0)


def cpu_sample_inputs(w, kd_full=None):
    import numpy as np

    from fastrecon_gb300 import synth
    traj = synth.radial_2d(w["spokes"], w["readout"]) if w["dim"] == 2 else \
        synth.kooshball_3d(w["spokes"], w["readout"])
    dcf = synth.ramp_dcf(traj, w["dim"], w["dcf_power"])
    return traj, dcf


def cpu_fractions(w):
    if w["dim"] == 3:
        return 1.0 / 8, 2
    return 1.0, w["coils"]


def run_reference(args, w):
    import numpy as np
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    ncpu = os.cpu_count() or 1
    frac, fft_coils = cpu_fractions(w)
    traj, dcf = cpu_sample_inputs(w)
    n = int(w["spokes"] * frac) * w["readout"]
    from fastrecon_gb300 import synth
    kd = synth.kspace(traj[:n], w["dim"], w["recon"], w["coils"], seed=0)
    tg = min(w["coils"], ncpu)
    for _ in range(args.warmup):
        cpu_step(w, traj, dcf, kd, tg, ncpu, frac, fft_coils)
    fulls, desc, wall = [], "", 0.0
    for _ in range(args.steps):
        f, desc, wl = cpu_step(w, traj, dcf, kd, tg, ncpu, frac, fft_coils)
        fulls.append(f)
        wall += wl
    t = statistics.mean(fulls)
    N = w["spokes"] * w["readout"]
    value = N * w["coils"] / t / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "samples_per_coil": N, "coils": w["coils"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": max(tg, ncpu), "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference CPU algorithm (oracle port of GridLut/ImageFilter; the reference's own sources "
                    "need Qt/GSL/FFTW and x86-only builds are not carried to this host)"}
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
    tr_path = os.path.join(ROOT, "profiles", "grid_tiles_traffic.txt")
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
        "roofline": {"bound": "hbm", "kernel": "grid_tiles_kernel (KB scatter)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": algo, "kernel_ms": per_launch_ms, "launches": scatter_n,
                     "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s"},
        "gpu_launches": int(launches),
        "clocks": ck,
        "e2e": e2e,
    }
    if not args.no_cpu_baseline and ws == 1:
        frac, fft_coils = cpu_fractions(w)
        ncpu = os.cpu_count() or 1
        ctraj, cdcf = cpu_sample_inputs(w)
        n = int(w["spokes"] * frac) * w["readout"]
        ckd = kd[:, :n].cpu().numpy()
        full, desc, _ = cpu_step(w, ctraj, cdcf, ckd, min(C, ncpu), ncpu, frac, fft_coils)
        line["cpu_baseline"] = {"value": N * C / full / 1e6, "unit": UNIT, "cores": ncpu, "kind": "port",
                                "sample": desc, "ms_per_step": full * 1e3}
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
