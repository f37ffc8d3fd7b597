#!/usr/bin/env python3
"""Benchmark of the all-pairs 2D-histogram MI + MIST hot path on one GB300.

Metric: DOF-pair x frame updates per second at 50 bins. One step = one
pg_entropy (per-DOF extrema/shift/binning, every pair's 2D histogram ->
entropy -> MI) plus one pg_mist (spanning tree over the resident MI matrix)
over the whole synthetic system; units per step = D(D-1)/2 * F.

Default workload (the protein-dimer-scale configuration the metric's target is
quoted on): a seeded synthetic linear chain of 2,500 atoms = 7,494 DOFs,
500,000 frames, FP32 values (15 GB resident), 50 bins for every type, 20% of
the dihedrals bimodal with a two-state Markov switch (p = 1e-3 / frame), 5% of
the bonds bimodal, 8 AR(1) latents. Inputs are far larger than L2, so no
flush is needed between steps.

  value : device-resident inputs, CUDA events on the library's stream
  e2e   : the public C ABI with pinned HOST columns in and the .par body + MIST
          edges out, host<->device copies inside the timed region
  --impl reference : the reference algorithm on the host cores (the oracle
          port, OpenMP over all threads) on a bounded DOF sample of the same
          workload

N > 1 (torchrun): each rank runs its own independent system (its own seed) on
its GPU; there is no collective in the data path, only a barrier and a max
over ranks of the timed region ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (n_atoms, frames, double_prec, bimodal dih, bimodal bond, latents)
    "protein_dimer_7494dof_500k": (2500, 500_000, 0, 0.2, 0.05, 8),
    "precision_path_2994dof_100k": (1000, 100_000, 0, 0.0, 0.0, 8),
    "plain_294dof_20k": (100, 20_000, 1, 0.0, 0.0, 8),
    "stress_14994dof_1m": (5000, 1_000_000, 0, 0.0, 0.0, 8),
    "small_600dof_50k": (203, 50_000, 0, 0.2, 0.05, 8),
}
DEFAULT = "protein_dimer_7494dof_500k"
METRIC = "DOF-pair x frame updates/s @50 bins (all-pairs 2D-histogram MI + MIST)"
UNIT = "updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT)
    ap.add_argument("--form", choices=["auto", "hist", "onehot"], default="auto")
    ap.add_argument("--bins", type=int, default=50)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample-atoms", type=int, default=0,
                    help="atoms of the bounded DOF sample timed on the host cores "
                         "(0: sized to ~2.5e10 pair-frame updates, about 10 s on 16 cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [ln.split(",") for ln in Path(self.file.name).read_text().splitlines() if ln.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU legs

def cpu_sample(args, wl):
    """Times the reference algorithm (oracle port, all host threads) on a
    DOF sample of the workload: the same generator, frame count and value
    distributions, cpu_sample_atoms atoms. Returns (updates/s, sample text, threads)."""
    n_atoms, F, prec, fbd, fbb, lat = wl
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    import parent_gb300 as pg
    na = args.cpu_sample_atoms
    if na <= 0:
        dofs = int((2 * 2.5e10 / F) ** 0.5)
        na = max(6, min(n_atoms, dofs // 3 + 2))
    t = pg.synth_host(na, F, double_prec=prec, seed=1234, n_latents=lat, frac_bimodal_dih=fbd,
                      frac_bimodal_bond=fbb)
    D = 3 * na - 6
    units = D * (D - 1) // 2 * F
    t0 = time.perf_counter()
    oracle.parent(t.bonds, t.angles, t.dihedrals, (args.bins,) * 6)
    dt = time.perf_counter() - t0
    sample = f"{D} DOFs ({na} atoms) x {F} frames of the same generator, {units:.3e} updates, {dt:.2f} s"
    return units / dt, sample, threads, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    wl = WORKLOADS[args.workload]
    if rank != 0:
        return 0
    vals = []
    for i in range(args.warmup + args.steps):
        v, sample, threads, dt = cpu_sample(args, wl)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    n_atoms, F = wl[0], wl[1]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "n_atoms": n_atoms, "frames": F, "bins": args.bins},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU leg

def run_gb300(args):
    import torch
    import parent_gb300 as pg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    n_atoms, F, prec, fbd, fbb, lat = WORKLOADS[args.workload]
    n_dih = n_atoms - 3
    D = 3 * n_atoms - 6
    P = D * (D - 1) // 2
    units = P * F
    bins = (args.bins,) * 6
    es = 8 if prec else 4

    eng = pg.Engine(local)
    # device-resident synthetic columns (bonds | angles | dihedrals)
    nb, na, nd = n_dih + 2, n_dih + 1, n_dih
    dbuf = eng.alloc(D * F * es)
    ptrs = (dbuf, dbuf + nb * F * es, dbuf + (nb + na) * F * es)
    eng.synth_device(n_atoms, F, prec, ptrs, F, seed=20260 + rank, n_latents=lat,
                     frac_bimodal_dih=fbd, frac_bimodal_bond=fbb)
    view = pg.BatView(n_dih, F, prec, 1, F, *ptrs)
    stream = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))

    def step():
        eng.entropy(view, bins, args.form, keep_result=False)
        eng.mist(n_dih)

    for _ in range(args.warmup):
        step()
    eng.synchronize()

    pair_ms, prep_ms, mist_ms = [], [], []
    launches0 = eng.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize(local)
    eng.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
        t = eng.timings()
        prep_ms.append(t[0]); pair_ms.append(t[1]); mist_ms.append(t[2])
    ev1.record(stream)
    ev1.synchronize()
    eng.synchronize()
    torch.cuda.synchronize(local)
    ms_total = ev0.elapsed_time(ev1)
    if dist:
        tt = torch.tensor([ms_total], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_total = float(tt.item())
        dist.barrier()
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    form = eng.last_form()
    ms_step = ms_total / args.steps
    value = units * world / (ms_total / 1e3 / args.steps)

    # ---- end to end through the public API, pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        import ctypes as C
        import numpy as np
        host = pg.C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(D * F * es, C.byref(host)))
        eng.memcpy(host.value, dbuf, D * F * es, 2)
        eng.synchronize()
        hview = pg.BatView(n_dih, F, prec, 0, F, host.value, host.value + nb * F * es,
                           host.value + (nb + na) * F * es)
        sizes = pg.block_sizes(n_dih)
        total = sum(sizes.values())
        hout = pg.C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(total * 8, C.byref(hout)))
        arr = np.ctypeslib.as_array(C.cast(hout, C.POINTER(C.c_double)), (total,))
        blocks, o = {}, 0
        for k, s in sizes.items():
            blocks[k] = arr[o:o + s]
            o += s
        body = pg.ParBody(n_dih, blocks)
        eng.entropy(hview, bins, args.form, out=body)   # warm the host path once
        eng.mist(n_dih)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            eng.entropy(hview, bins, args.form, out=body)
            edges, totals = eng.mist(n_dih)
        t1 = time.perf_counter()
        sec = (t1 - t0) / args.e2e_steps
        if dist:
            tt = torch.tensor([sec], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            sec = float(tt.item())
        e2e = {"value": units * world / sec, "unit": UNIT, "h2d_bytes_per_step": D * F * es,
               "d2h_bytes_per_step": total * 8 + (D - 1) * (4 * 4 + 8 + 8), "ms_per_step": sec * 1e3}
        pg._check(pg.lib().pg_host_free_pinned(host))
        pg._check(pg.lib().pg_host_free_pinned(hout))

    # ---- roofline of the dominant kernel (the pair kernel)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    pair_s = statistics.mean(pair_ms) / 1e3
    if form == "hist":
        red_peak = eng.probe_smem_red_rate()
        achieved = units / pair_s
        roofline = {"bound": "smem", "achieved": achieved / 1e9, "peak": red_peak / 1e9, "unit": "Gred/s",
                    "frac": achieved / red_peak, "traffic": None,
                    "note": "one shared-memory reduction per pair-frame update; peak = conflict-free "
                            "red.shared rate measured live on this GPU (pg_probe_smem_red_rate)"}
    else:
        achieved = 2.0 * args.bins * args.bins * units / pair_s / 1e12
        peak = 2.0 * float(peaks.get("bf16_tflops", 1900.0))
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": None,
                    "note": "2*B^2 one-hot FLOPs per update; peak = 2x measured cuBLAS bf16 (FP8 dense rate)"}
    prep_s = statistics.mean(prep_ms) / 1e3
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    prep_bytes = D * F * (es + 1)
    roofline_prep = {"bound": "hbm", "achieved": prep_bytes / prep_s / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": prep_bytes / prep_s / 1e9 / hbm,
                     "note": "algorithmic bytes D*F*(4|8 in + 1 bin out); peak of measured copy bandwidth"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, sample, threads, _ = cpu_sample(args, WORKLOADS[args.workload])
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "n_atoms": n_atoms, "dofs": D, "pairs": P, "frames": F,
                       "input": "fp64" if prec else "fp32", "bins": args.bins, "form": form,
                       "parallelism": f"replicas x{world}" if world > 1 else "single gpu",
                       "l2": "inputs (%.1f GB) larger than L2; no flush" % (D * F * es / 1e9)},
            "kernel_ms": {"prep": statistics.mean(prep_ms), "pairs": statistics.mean(pair_ms),
                          "mist": statistics.mean(mist_ms)},
            "roofline": roofline, "roofline_prep": roofline_prep,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.free(dbuf)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
