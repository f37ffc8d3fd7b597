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
# 64 independent systems: atoms ~ U[50,800], frames log-uniform in
# [5,000, 100,000], FP32, latents ~ U[2,16], one seed per system
BATCH = "batch64_50to800atoms_5k100kframes"
DEFAULT = "protein_dimer_7494dof_500k"
METRIC = "DOF-pair x frame updates/s @50 bins (all-pairs 2D-histogram MI + MIST)"
UNIT = "updates/s"


def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over all ranks (x itself without a process group): the
    timed region of a multi-rank run is the slowest rank's."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(base: int, rank: int) -> int:
    """Seed of a rank's own synthetic system: independent replicas, no shared data."""
    return base + 7919 * rank


def traffic_per_update(layout: str):
    """DRAM bytes per update of the pair kernel from the committed ncu capture
    (profiles/), or None: the capture is on a smaller case (2,994 DOFs x 100k
    frames) and is scaled by this launch's updates."""
    name = {"stream32": "pairs_hist32s_kernel_precision_path_2994dof_100k_50bins.md",
            "ring32": "pairs_hist32_kernel_precision_path_2994dof_100k_30bins.md",
            "16": "pairs_hist_kernel_precision_path_2994dof_100k.md"}[layout]
    try:
        for line in (ROOT / "profiles" / name).read_text().splitlines():
            if line.startswith("dram_bytes_per_update:"):
                return float(line.split(":")[1]), name
    except OSError:
        pass
    return None, name


def hist_layout(bins: int) -> str:
    """The histogram layout the library picks (parent_gb300/csrc/pg_autotune.cu
    hist_layout): the streamed 32-slot kernel up to 50 bins, else 16 slots;
    PG_HIST_SLOTS / PG_HIST_STREAM override it."""
    forced = os.environ.get("PG_HIST_SLOTS")
    if forced == "16":
        return "16"
    if forced == "32":
        return "ring32" if bins <= 50 else "16"
    if os.environ.get("PG_HIST_STREAM") == "0":
        return "ring32" if bins <= 35 else "16"
    return "stream32" if bins <= 50 else "16"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--shard", action="store_true",
                    help="one system split over the ranks (tile shards, one SUM reduction, MIST on rank 0; "
                         "strong scaling) instead of one independent system per rank")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + [BATCH], default=DEFAULT)
    ap.add_argument("--form", choices=["auto", "hist", "onehot"], default="auto")
    ap.add_argument("--bins", type=int, default=50)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample-atoms", type=int, default=0,
                    help="atoms of the bounded DOF sample timed on the host cores "
                         "(0: sized to ~8e10 pair-frame updates, about 10 s on 16 Grace cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--parity-pairs", type=int, default=10000,
                    help="pairs of the timed system checked against the FP64 oracle after the timed region "
                         "(plus bit-exact counts on 100 of them and the oracle's MIST on the GPU's body)")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size parity leg")
    ap.add_argument("--compare-forms", choices=["auto", "on", "off"], default="auto",
                    help="time one step of each form (tensor-core one-hot, shared-memory histogram) at 50 and "
                         "10 bins after the timed region (auto: on for the protein-dimer workload)")
    ap.add_argument("--batconv", action="store_true",
                    help="instead of the step: time the Cartesian -> BAT conversion of a synthetic chain "
                         "with the workload's atoms and frames (host coordinates in, device columns out)")
    ap.add_argument("--pipeline", action="store_true",
                    help="instead of the step: write the workload as a .bat and time the drop-in CLIs on it "
                         "(PARENT_gb300, get_PAR_MIE_gb300, get_PAR_MIST_gb300), as the reference's run.sh runs them")
    ap.add_argument("--mie", action="store_true",
                    help="instead of the step: time get_PAR_MIE's text for a .par body of the workload's size "
                         "with the host writer and with the device writer (files under $TMPDIR)")
    ap.add_argument("--ingest", action="store_true",
                    help="instead of the step: write the workload as a .bat (under $TMPDIR) and time "
                         "pg_bat_read (host columns) against pg_bat_read_device (device columns)")
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
        dofs = int((2 * 8e10 / F) ** 0.5)
        na = max(6, min(n_atoms, dofs // 3 + 2))
    t = pg.synth_host(na, F, double_prec=prec, seed=1234, n_latents=lat, frac_bimodal_dih=fbd,
                      frac_bimodal_bond=fbb)
    D = 3 * na - 6
    units = D * (D - 1) // 2 * F
    t0 = time.perf_counter()
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, (args.bins,) * 6)
    dt = time.perf_counter() - t0
    sample = f"{D} DOFs ({na} atoms) x {F} frames of the same generator, {units:.3e} updates, {dt:.2f} s"
    cpu_sample.last = (t, ref)  # the oracle's result on the sample, for parity_on_sample
    return units / dt, sample, threads, dt


def _mutual_all(n: int, body: dict):
    """Every pair's MI as get_mutual (util.cpp:47-81) forms it, in body order."""
    import numpy as np
    nb, na = n + 2, n + 1
    s1 = {"b": body["s1_b"], "a": body["s1_a"], "d": body["s1_d"]}
    out = []
    for key, t1, t2, n1 in (("bb", "b", "b", nb), ("ba", "b", "a", nb), ("bd", "b", "d", nb),
                            ("aa", "a", "a", na), ("ad", "a", "d", na), ("dd", "d", "d", n)):
        blk = body[key]
        if blk.size == 0:
            continue
        if t1 == t2:
            i, j = np.triu_indices(n1, 1)
            out.append(s1[t1][i] + s1[t2][j] - blk[::-1])
        else:
            out.append((s1[t1][:, None] + s1[t2][None, :]).ravel() - blk)
    return np.concatenate(out) if out else np.zeros(0)


def parity_on_sample(eng, bins, form):
    """The GPU path on the CPU baseline's sample against the oracle's FP64
    result there: the largest |dS| and |dMI| (nats) over every term."""
    import numpy as np
    t, ref = cpu_sample.last
    body = eng.entropy(t, bins, form)
    ds = max(float(np.max(np.abs(body.blocks[k] - ref[k]), initial=0.0)) for k in body.blocks)
    dmi = float(np.max(np.abs(_mutual_all(t.n_dih, body.blocks) - _mutual_all(t.n_dih, ref)), initial=0.0))
    return {"max_abs_dS_nats": ds, "max_abs_dMI_nats": dmi, "mi_tolerance_nats": 1e-5,
            "terms": int(sum(v.size for v in ref.values())), "form": eng.last_form(),
            "counts": "bit-exact (tests/test_gpu_parity.py)"}


def reference_exe():
    """The reference's own PARENT.x compiled from its sources (oracle/Makefile
    ref), if it was built and runs on this machine's architecture."""
    exe = ROOT / "oracle" / "_ref" / "PARENT.x"
    if not os.access(exe, os.X_OK):
        return None
    try:
        subprocess.run([str(exe)], capture_output=True, timeout=60)  # usage text, exit 1
    except OSError:  # built for another architecture
        return None
    return exe


def cpu_sample_reference(args, wl, exe):
    """The reference's own PARENT.x on the CPU sample of cpu_sample (written as
    a .bat file), all host threads: updates/s of its own "Calculation time"
    (the read of the .bat and the .par write excluded)."""
    import re
    import shutil
    import parent_gb300 as pg
    n_atoms, F, prec, fbd, fbb, lat = wl
    threads = os.cpu_count() or 1
    na = args.cpu_sample_atoms
    if na <= 0:
        dofs = int((2 * 8e10 / F) ** 0.5)
        na = max(6, min(n_atoms, dofs // 3 + 2))
    t = pg.synth_host(na, F, double_prec=prec, seed=1234, n_latents=lat, frac_bimodal_dih=fbd,
                      frac_bimodal_bond=fbb)
    D = 3 * na - 6
    units = D * (D - 1) // 2 * F
    d = Path(tempfile.mkdtemp(prefix="pg_ref_"))
    try:
        pg.write_bat(d / "s.bat", t)
        del t
        r = subprocess.run([str(exe), str(d / "s.bat"), str(d / "s.par")] + [str(args.bins)] * 6,
                           capture_output=True, text=True, env={**os.environ, "OMP_NUM_THREADS": str(threads)})
    finally:
        shutil.rmtree(d, ignore_errors=True)
    m = re.search(r"Calculation time: ([0-9.eE+-]+)", r.stdout)
    if r.returncode != 0 or m is None:
        raise RuntimeError("PARENT.x failed: " + (r.stdout + r.stderr)[-500:])
    dt = float(m.group(1))
    sample = (f"{D} DOFs ({na} atoms) x {F} frames of the same generator as a .bat, {units:.3e} updates, "
              f"{dt:.2f} s of the reference's own calculation time (MPI: one rank)")
    return units / dt, sample, threads, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    # the batch workload is sampled as one system of its largest atom count at
    # its mean frame count
    wl = WORKLOADS[args.workload] if args.workload in WORKLOADS else (800, 31_700, 0, 0.0, 0.0, 8)
    if rank != 0:
        return 0
    # the reference's own binary where it was built here (this architecture),
    # else the oracle port of its algorithm
    exe = reference_exe()
    kind = "reference" if exe is not None else "port"
    vals = []
    for i in range(args.warmup + args.steps):
        if exe is not None:
            v, sample, threads, dt = cpu_sample_reference(args, wl, exe)
        else:
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
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU leg

def batch_systems(seed: int = 64, n: int = 64):
    """(n_atoms, frames, latents, seed) of the batch workload's systems."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        atoms = int(rng.integers(50, 801))
        frames = int(round(float(np.exp(rng.uniform(np.log(5000.0), np.log(100000.0))))))
        lat = int(rng.integers(2, 17))
        out.append((atoms, frames, lat, 1000 + 17 * k))
    return out


def run_batch(args):
    """The batch workload: pg_entropy_batch (one pair launch over every
    system's tiles + one MIST launch, replayed from a captured CUDA graph)
    against the same 64 systems run one after another through pg_entropy +
    pg_mist. value = batched updates/s; the sequential figure is reported
    beside it."""
    import ctypes as C
    import numpy as np
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
    bins = (args.bins,) * 6
    systems = batch_systems(seed=replica_seed(64, rank))
    es = 4
    eng = pg.Engine(local)
    sizes = [(3 * a - 6) * f * es for a, f, _, _ in systems]
    total_bytes = sum(sizes)
    dbuf = eng.alloc(total_bytes)
    views, units = [], 0
    off = 0
    for (a, f, lat, sd), nbytes in zip(systems, sizes):
        nd = a - 3
        nb, na = nd + 2, nd + 1
        p = dbuf + off
        ptrs = (p, p + nb * f * es, p + (nb + na) * f * es)
        eng.synth_device(a, f, 0, ptrs, f, seed=replica_seed(sd, rank), n_latents=lat, frac_bimodal_dih=0.0,
                         frac_bimodal_bond=0.0)
        views.append(pg.BatView(nd, f, 0, 1, f, *ptrs))
        D = 3 * a - 6
        units += D * (D - 1) // 2 * f
        off += nbytes
    stream = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))

    def batched():
        eng.entropy_batch(views, bins, args.form, bodies=False, trees=True)

    def sequential():
        for v in views:
            eng.entropy(v, bins, args.form, keep_result=False)
            eng.mist(v.n_dihedrals)

    def timed(fn, steps):
        if dist:
            dist.barrier()
        torch.cuda.synchronize(local)
        eng.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            fn()
        ev1.record(stream)
        ev1.synchronize()
        eng.synchronize()
        torch.cuda.synchronize(local)
        ms = ev0.elapsed_time(ev1)
        ms = max_over_ranks(ms, dist, f"cuda:{local}")
        return ms / steps

    for _ in range(args.warmup):
        batched()
    launches0 = eng.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    ms_batch = timed(batched, args.steps)
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    graph_ms = float(eng.timings()[1])
    batch_form = eng.last_form()  # the form the batch ran (one-hot per system where the autotuner picks it)
    sequential()
    ms_seq = timed(sequential, max(1, min(args.steps, 2)))
    value = units * world / (ms_batch / 1e3)

    e2e = None
    if args.e2e_steps > 0:
        host = C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(total_bytes, C.byref(host)))
        eng.memcpy(host.value, dbuf, total_bytes, 2)
        eng.synchronize()
        hviews, off = [], 0
        for v, nbytes in zip(views, sizes):
            nd, f = v.n_dihedrals, v.n_frames
            p = host.value + off
            hviews.append(pg.BatView(nd, f, 0, 0, f, p, p + (nd + 2) * f * es, p + (2 * nd + 3) * f * es))
            off += nbytes
        body_elems = [sum(pg.block_sizes(v.n_dihedrals).values()) for v in views]
        hout = C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(sum(body_elems) * 8, C.byref(hout)))
        flat = np.ctypeslib.as_array(C.cast(hout, C.POINTER(C.c_double)), (sum(body_elems),))
        bodies, o = [], 0
        for v in views:
            blocks = {}
            for k, n in pg.block_sizes(v.n_dihedrals).items():
                blocks[k] = flat[o:o + n]
                o += n
            bodies.append(pg.ParBody(v.n_dihedrals, blocks))
        eng.entropy_batch(hviews, bins, args.form, bodies=bodies, trees=True)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            eng.entropy_batch(hviews, bins, args.form, bodies=bodies, trees=True)
        sec = (time.perf_counter() - t0) / args.e2e_steps
        sec = max_over_ranks(sec, dist, f"cuda:{local}")
        n_edges = sum(3 * v.n_dihedrals + 2 for v in views)
        e2e = {"value": units * world / sec, "unit": UNIT, "h2d_bytes_per_step": total_bytes,
               "d2h_bytes_per_step": sum(body_elems) * 8 + n_edges * 32 + 80 * len(views),
               "ms_per_step": sec * 1e3}
        pg._check(pg.lib().pg_host_free_pinned(host))
        pg._check(pg.lib().pg_host_free_pinned(hout))

    red_peak = eng.probe_smem_red_rate()
    achieved = units / (graph_ms / 1e3)
    roofline = {"bound": "smem", "achieved": achieved / 1e9, "peak": red_peak / 1e9, "unit": "Gred/s",
                "frac": achieved / red_peak, "traffic": None,
                "note": "whole captured graph (64 preps + one pair launch + one MIST launch) timed; one "
                        "shared-memory reduction per update; peak = live conflict-free red.shared rate"}
    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, sample, threads, _ = cpu_sample(args, (800, 31_700, 0, 0.0, 0.0, 8))
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": sample + " (one system of the batch's largest atom count at its mean frame count)"}
        parity = parity_on_sample(eng, bins, args.form)
    if rank == 0:
        Ds = [3 * a - 6 for a, _, _, _ in systems]
        Fs = [f for _, f, _, _ in systems]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": BATCH, "systems": len(systems), "dofs": [min(Ds), max(Ds)],
                       "frames": [min(Fs), max(Fs)], "updates_per_step": units, "input": "fp32",
                       "bins": args.bins, "form": batch_form,
                       "hist_layout": hist_layout(args.bins) if batch_form == "hist" else None,
                       "parallelism": f"replicas x{world}" if world > 1 else "single gpu",
                       "l2": "inputs (%.1f GB) larger than L2; no flush" % (total_bytes / 1e9)},
            "sequential": {"ms_per_step": ms_seq, "value": units * world / (ms_seq / 1e3),
                           "speedup_of_batch": ms_seq / ms_batch},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.free(dbuf)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_sharded(args):
    """One system split over the ranks (strong scaling), the reference's MPI
    decomposition GB300 style: every rank preprocesses the whole system and
    computes its range of the pair tiles (pg_entropy_shard) into a device
    tensor, one SUM reduction (NCCL) merges the shards on rank 0 without a
    host copy, and rank 0 runs MIST from the merged device body. A step is
    that whole sequence; units = the system's updates; time = max over ranks,
    CUDA events on the framework stream around the steps. e2e: the same with
    the columns in pinned host memory, uploaded by every rank inside each
    step, and the merged body and edges read back on rank 0. Rank 0 checks
    the merged body against a one-GPU pg_entropy body, bit for bit."""
    import ctypes as C

    import numpy as np
    import torch

    import parent_gb300 as pg
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n_atoms, F, prec, fbd, fbb, lat = WORKLOADS[args.workload]
    n_dih = n_atoms - 3
    D = 3 * n_atoms - 6
    units = D * (D - 1) // 2 * F
    bins = (args.bins,) * 6
    es = 8 if prec else 4
    eng = pg.Engine(local)
    nb, na = n_dih + 2, n_dih + 1
    dbuf = eng.alloc(D * F * es)
    ptrs = (dbuf, dbuf + nb * F * es, dbuf + (nb + na) * F * es)
    eng.synth_device(n_atoms, F, prec, ptrs, F, seed=20260, n_latents=lat, frac_bimodal_dih=fbd,
                     frac_bimodal_bond=fbb)  # the same system on every rank
    view = pg.BatView(n_dih, F, prec, 1, F, *ptrs)
    total = sum(pg.block_sizes(n_dih).values())
    merged = torch.zeros(total, dtype=torch.float64, device=f"cuda:{local}")
    torch.cuda.synchronize(local)
    body = pg.DeviceParBody(n_dih, merged.data_ptr())

    def step(v):
        eng.entropy_shard(v, bins, rank, world, "hist", out=body)  # returns with the shard written
        if dist:
            dist.reduce(merged, dst=0, op=dist.ReduceOp.SUM)
        if rank == 0:
            torch.cuda.current_stream().synchronize()
            return eng.mist(n_dih, body)
        return None

    for _ in range(args.warmup):
        step(view)
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    launches0 = eng.launch_count()
    for _ in range(args.steps):
        step(view)
    ev1.record()
    torch.cuda.synchronize(local)
    launches = eng.launch_count() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, f"cuda:{local}")
    if dist:
        dist.barrier()
    clk = clocks.stop()
    # e2e: pinned host columns uploaded by every rank inside each step
    e2e = None
    if args.e2e_steps > 0:
        host = pg.C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(D * F * es, C.byref(host)))
        eng.memcpy(host.value, dbuf, D * F * es, 2)
        eng.synchronize()
        hview = pg.BatView(n_dih, F, prec, 0, F, host.value, host.value + nb * F * es,
                           host.value + (nb + na) * F * es)
        hbody = np.empty(total)
        step(hview)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            step(hview)
            if rank == 0:
                hbody[:] = merged.cpu().numpy()
        sec = max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, dist, f"cuda:{local}")
        e2e = {"value": units / sec, "unit": UNIT, "h2d_bytes_per_step": D * F * es * world,
               "d2h_bytes_per_step": total * 8 + (D - 1) * (4 * 4 + 8 + 8), "ms_per_step": sec * 1e3}
        pg._check(pg.lib().pg_host_free_pinned(host))
    check = None
    if rank == 0:
        whole = eng.entropy(view, bins, "hist").flat()
        check = {"merged_equals_one_gpu_body": bool(np.array_equal(merged.cpu().numpy().view(np.uint64),
                                                                   whole.view(np.uint64)))}
        line = {
            "metric": METRIC, "value": units / (ms / 1e3 / args.steps), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "n_atoms": n_atoms, "dofs": D, "frames": F,
                       "input": "fp64" if prec else "fp32", "bins": args.bins, "form": "hist",
                       "parallelism": f"tile shards x{world}, one SUM reduction, MIST on rank 0",
                       "l2": "inputs (%.1f GB) larger than L2; no flush" % (D * F * es / 1e9)},
            "e2e": e2e, "check": check, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.free(dbuf)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_gb300(args):
    if args.workload == BATCH:
        return run_batch(args)
    if args.shard:
        return run_sharded(args)
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
    eng.synth_device(n_atoms, F, prec, ptrs, F, seed=replica_seed(20260, rank), n_latents=lat,
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
    ms_total = max_over_ranks(ms_total, dist, f"cuda:{local}")
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    form = eng.last_form()
    ms_step = ms_total / args.steps
    value = units * world / (ms_total / 1e3 / args.steps)

    # ---- end to end through the public API, pinned host buffers
    import ctypes as C
    import numpy as np
    e2e = None
    want_parity = rank == 0 and world == 1 and not args.no_parity and args.parity_pairs > 0
    host = None
    if args.e2e_steps > 0 or want_parity:
        # the step's input columns in pinned host memory (bonds | angles | dihedrals)
        host = pg.C.c_void_p()
        pg._check(pg.lib().pg_host_alloc_pinned(D * F * es, C.byref(host)))
        eng.memcpy(host.value, dbuf, D * F * es, 2)
        eng.synchronize()
    if args.e2e_steps > 0:
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
        parts = []
        for i in range(args.e2e_steps):
            w0 = time.perf_counter()
            # every step uploads its columns from the pinned host buffer: the
            # first by SM loads inside its call, each later one on the copy
            # engine during the previous step's kernels (pg_entropy_ahead)
            eng.entropy(hview, bins, args.form, out=body, next=hview if i + 1 < args.e2e_steps else None)
            te = eng.timings()
            w1 = time.perf_counter()
            edges, totals = eng.mist(n_dih)
            tm = eng.timings()
            parts.append({"entropy_wall_ms": (w1 - w0) * 1e3, "mist_wall_ms": (time.perf_counter() - w1) * 1e3,
                          "transfer_ms": float(te[3]), "prep_ms": float(te[0]), "pairs_ms": float(te[1]),
                          "entropy_device_ms": float(te[4]), "mist_ms": float(tm[2])})
        t1 = time.perf_counter()
        sec = (t1 - t0) / args.e2e_steps
        sec = max_over_ranks(sec, dist, f"cuda:{local}")
        e2e = {"value": units * world / sec, "unit": UNIT, "h2d_bytes_per_step": D * F * es,
               "d2h_bytes_per_step": total * 8 + (D - 1) * (4 * 4 + 8 + 8), "ms_per_step": sec * 1e3,
               "upload": "step 1 by SM loads in its call; steps 2.. on the copy engine during the previous "
                         "step's kernels (pg_entropy_ahead)", "breakdown": parts[-1]}
        pg._check(pg.lib().pg_host_free_pinned(hout))

    # ---- the metric's own comparison: each form at 50 and 10 bins (after the timed region)
    forms_cmp = None
    want_cmp = args.compare_forms == "on" or (args.compare_forms == "auto" and args.workload == DEFAULT)
    if want_cmp and rank == 0:
        forms_cmp = compare_forms(eng, view, n_dih, units, stream)

    # ---- full-size parity of the timed system itself (outside every timed region)
    parity_full = None
    if want_parity:
        parity_full = full_parity(args, eng, view, host.value, n_dih, F, prec, bins)
    if host is not None:
        pg._check(pg.lib().pg_host_free_pinned(host))

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
        bpu, prof = traffic_per_update(hist_layout(args.bins))
        roofline = {"bound": "smem", "achieved": achieved / 1e9, "peak": red_peak / 1e9, "unit": "Gred/s",
                    "frac": achieved / red_peak, "traffic": bpu * units if bpu else None,
                    "note": "one shared-memory reduction per pair-frame update; peak = conflict-free "
                            "red.shared rate measured live on this GPU (pg_probe_smem_red_rate); traffic = "
                            "DRAM bytes per update of the ncu capture in profiles/" + prof + " x this launch's "
                            "updates (bytes per launch)"}
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

    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, sample, threads, _ = cpu_sample(args, WORKLOADS[args.workload])
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
        parity = parity_on_sample(eng, bins, args.form)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "n_atoms": n_atoms, "dofs": D, "pairs": P, "frames": F,
                       "input": "fp64" if prec else "fp32", "bins": args.bins, "form": form,
                       "hist_layout": hist_layout(args.bins) if form == "hist" else None,
                       "parallelism": f"replicas x{world}" if world > 1 else "single gpu",
                       "l2": "inputs (%.1f GB) larger than L2; no flush" % (D * F * es / 1e9)},
            "kernel_ms": {"prep": statistics.mean(prep_ms), "pairs": statistics.mean(pair_ms),
                          "mist": statistics.mean(mist_ms)},
            "roofline": roofline, "roofline_prep": roofline_prep,
            "onehot_vs_hist": forms_cmp,
            "cpu_baseline": cpu, "parity": parity_full, "parity_cpu_sample": parity, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.free(dbuf)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def compare_forms(eng, view, n_dih: int, units: int, stream):
    """One step (pg_entropy + pg_mist, device-resident columns) of each form at
    50 and 10 bins, timed with CUDA events on the library's stream: the
    comparison the metric names (tensor-core one-hot against shared-memory
    histogram). The one-hot form's roofline is 2*B^2 FLOPs per update against
    the dense FP8 rate, taken as 2x the measured sustained cuBLAS bf16 rate
    (these are seconds-long kernels)."""
    import torch
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    fp8 = 2.0 * float(peaks.get("bf16_tflops_sustained", 1700.0))
    out = {"peak_fp8_tflops": fp8, "peak_note": "2x measured sustained cuBLAS bf16 (MEASURED_PEAKS.json)"}
    for b in (50, 10):
        row = {}
        for form in ("hist", "onehot"):
            eng.entropy(view, (b,) * 6, form, keep_result=False)  # first call of this geometry: buffers
            eng.mist(n_dih)
            eng.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            eng.entropy(view, (b,) * 6, form, keep_result=False)
            pair_ms = float(eng.timings()[1])
            eng.mist(n_dih)
            ev1.record(stream)
            ev1.synchronize()
            ms = ev0.elapsed_time(ev1)
            r = {"ms_per_step": ms, "pairs_ms": pair_ms, "value": units / (ms / 1e3), "form": eng.last_form()}
            if form == "onehot":
                tf = 2.0 * b * b * units / (pair_ms / 1e3) / 1e12
                r["roofline"] = {"bound": "tensor", "achieved": tf, "peak": fp8, "unit": "TFLOP/s", "frac": tf / fp8}
            row[form] = r
        row["hist_over_onehot_time"] = row["hist"]["ms_per_step"] / row["onehot"]["ms_per_step"]
        out[str(b)] = row
    out["target"] = "one-hot >= 3x less wall time than the histogram form at 50 bins"
    out["target_met"] = bool(out["50"]["hist_over_onehot_time"] >= 3.0)
    return out


def full_parity(args, eng, view, host_ptr: int, n_dih: int, F: int, prec: int, bins):
    """The timed system itself against the FP64 oracle: one more pg_entropy +
    pg_mist on the device-resident columns (the same call the timed steps
    make), then oracle.check.check_run on the host copy of the same columns:
    args.parity_pairs random pairs (S2D and MI terms), bit-exact counts on
    100 of them (pg_pair_counts, the histogram kernel), every 1D entropy, and
    the oracle's MIST (the reference's scan order) on the GPU's own body,
    which must reproduce the GPU's edge list."""
    import ctypes as C
    import numpy as np
    import parent_gb300 as pg
    from oracle import check
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    body = eng.entropy(view, bins, args.form)
    form = eng.last_form()
    edges, _ = eng.mist(n_dih)
    nb, na = n_dih + 2, n_dih + 1
    D = nb + na + n_dih
    dt = np.float64 if prec else np.float32
    flat = np.ctypeslib.as_array(C.cast(host_ptr, C.POINTER(C.c_double if prec else C.c_float)), (D * F,))
    cols = flat.reshape(D, F)
    b, a, d = cols[:nb], cols[nb:nb + na], cols[nb + na:]
    t0 = time.perf_counter()
    res = check.check_run(b, a, d, bins, body.blocks, edges,
                          gpu_counts=lambda pairs: eng.pair_counts(view, bins, pairs),
                          n_pairs=args.parity_pairs, n_count_pairs=100)
    res.update({"form": form, "counts_form": "hist", "oracle_threads": threads,
                "oracle_s": round(time.perf_counter() - t0, 2), "input": str(np.dtype(dt)),
                "system": "the timed system (same seed, columns and bins)"})
    return res


def run_ingest(args):
    """.bat ingest throughput: the workload written once as a .bat file, then
    read `steps` times by each reader (after `warmup` untimed reads, so the
    file is in the page cache for both). Prints one JSON line."""
    import shutil

    import parent_gb300 as pg
    n_atoms, F, prec, fbd, fbb, lat = WORKLOADS[args.workload]
    t = pg.synth_host(n_atoms, F, double_prec=prec, seed=20260, n_latents=lat, frac_bimodal_dih=fbd,
                      frac_bimodal_bond=fbb)
    d = Path(tempfile.mkdtemp(prefix="pg_ingest_"))
    try:
        path = d / "traj.bat"
        t0 = time.perf_counter()
        pg.write_bat(path, t)
        write_s = time.perf_counter() - t0
        del t
        size = path.stat().st_size
        res = {}
        for name, dev in (("host", None), ("device", 0)):
            times = []
            for k in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                b = pg.BatFile(path, device=dev)
                dt = time.perf_counter() - t0
                b.close()
                if k >= args.warmup:
                    times.append(dt)
            s = statistics.median(times)
            res[name] = {"s": round(s, 4), "GB_per_s": round(size / s / 1e9, 2), "runs": [round(x, 4) for x in times]}
        print(json.dumps({"metric": ".bat ingest (file -> DOF-major columns)", "file_bytes": size,
                          "write_s": round(write_s, 2), "host_reader": res["host"], "device_reader": res["device"],
                          "reader_threads": min(16, os.cpu_count() or 1), "page_cache": "warm",
                          "config": {"workload": args.workload, "n_atoms": n_atoms, "frames": F,
                                     "input": "fp64" if prec else "fp32"}}), flush=True)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return 0


def run_batconv(args):
    """Cartesian -> BAT throughput (pg_bat_from_cartesian): a jittering random
    chain of the workload's atoms and frames in pinned host memory, FP64 and
    FP32 columns out. Prints one JSON line."""
    import ctypes as C

    import numpy as np

    import parent_gb300 as pg
    n_atoms, F = WORKLOADS[args.workload][:2]
    nd = n_atoms - 3
    rng = np.random.default_rng(7)
    steps = rng.normal(size=(n_atoms, 3)).astype(np.float32)
    steps /= np.linalg.norm(steps, axis=1, keepdims=True)
    base = np.cumsum(0.15 * steps, axis=0, dtype=np.float32)
    xyz = np.empty((F, n_atoms, 3), np.float32)
    jit = (0.01 * rng.normal(size=(4096, n_atoms, 3))).astype(np.float32)
    for f0 in range(0, F, 4096):
        n = min(4096, F - f0)
        xyz[f0:f0 + n] = base[None] + jit[:n]
    dih = np.zeros((nd, 6), np.int32)
    for i in range(nd):
        dih[i] = [i + 1, i + 2, i + 3, i + 4, 0, i if i % 3 == 1 else -1]
    eng = pg.Engine(0)
    res = {}
    for prec in (1, 0):
        times, dev = [], []
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            eng.bat_from_cartesian(xyz, dih, double_prec=prec)
            dt = time.perf_counter() - t0
            ms = (C.c_double * 5)()
            pg.lib().pg_last_timings(eng.handle, ms)
            if k >= args.warmup:
                times.append(dt)
                dev.append(ms[4] / 1e3)
        s = statistics.median(times)
        res["fp64" if prec else "fp32"] = {"s": round(s, 4), "device_s": round(statistics.median(dev), 4),
                                           "frames_per_s": round(F / s), "dof_values_per_s": (3 * nd + 3) * F / s}
    eng.close()
    print(json.dumps({"metric": "Cartesian -> BAT conversion (xyz in host memory -> device BAT columns)",
                      "input_bytes": int(xyz.nbytes), "results": res,
                      "config": {"workload": args.workload, "n_atoms": n_atoms, "frames": F}}), flush=True)
    return 0


def run_mie(args):
    """MIE text throughput: a seeded random .par body with the workload's DOF
    count written by pg_write_mie_text (host threads) and by
    pg_write_mie_text_device (pair lines on the GPU); the two files must be
    identical. Prints one JSON line."""
    import hashlib
    import shutil

    import numpy as np

    import parent_gb300 as pg
    n_atoms = WORKLOADS[args.workload][0]
    nd = n_atoms - 3
    rng = np.random.default_rng(11)
    body = pg.ParBody.empty(nd)
    for v in body.blocks.values():
        v[:] = rng.normal(2.0, 1.5, v.size)
    lines = sum(v.size for v in body.blocks.values()) + 16  # one line per body value, 16 totals
    d = Path(tempfile.mkdtemp(prefix="pg_mie_"))
    eng = pg.Engine(0)
    res = {}
    try:
        for name in ("host", "device"):
            times = []
            for k in range(args.warmup + args.steps):
                path = d / f"{name}.txt"
                t0 = time.perf_counter()
                if name == "host":
                    pg.write_mie_text(path, body)
                else:
                    eng.write_mie_text(path, body)
                dt = time.perf_counter() - t0
                if k >= args.warmup:
                    times.append(dt)
            h = hashlib.sha1()
            with open(d / f"{name}.txt", "rb") as f:
                while chunk := f.read(1 << 24):
                    h.update(chunk)
            s = statistics.median(times)
            res[name] = {"s": round(s, 3), "lines_per_s": round(lines / s), "sha1": h.hexdigest(),
                         "bytes": (d / f"{name}.txt").stat().st_size}
    finally:
        eng.close()
        shutil.rmtree(d, ignore_errors=True)
    print(json.dumps({"metric": "MIE text (get_PAR_MIE.x output) written to a file", "lines": lines,
                      "identical": res["host"]["sha1"] == res["device"]["sha1"], "host_writer": res["host"],
                      "device_writer": res["device"], "host_threads": os.cpu_count(),
                      "config": {"workload": args.workload, "dofs": 3 * nd + 3}}), flush=True)
    return 0


def run_pipeline(args):
    """The reference's run.sh sequence on the drop-ins, wall clock per program:
    PARENT_gb300 (.bat -> .par), get_PAR_MIE_gb300 (MIE text to a file),
    get_PAR_MIST_gb300 (MIST text). Prints one JSON line."""
    import shutil

    import parent_gb300 as pg
    n_atoms, F, prec, fbd, fbb, lat = WORKLOADS[args.workload]
    t = pg.synth_host(n_atoms, F, double_prec=prec, seed=20260, n_latents=lat, frac_bimodal_dih=fbd,
                      frac_bimodal_bond=fbb)
    d = Path(tempfile.mkdtemp(prefix="pg_pipe_"))
    bins = [str(args.bins)] * 6
    res = {}
    try:
        bat, par = d / "traj.bat", d / "traj.par"
        t0 = time.perf_counter()
        pg.write_bat(bat, t)
        res["write_bat_s"] = round(time.perf_counter() - t0, 2)
        del t
        steps = [("PARENT_gb300", [str(bat), str(par)] + bins, None),
                 ("get_PAR_MIE_gb300", [str(par)], d / "mie.txt"),
                 ("get_PAR_MIST_gb300", [str(par), str(d / "mist.txt")], None)]
        for name, argv, stdout_path in steps:
            t0 = time.perf_counter()
            with open(stdout_path or os.devnull, "w") as out:
                r = subprocess.run([str(pg.BIN_DIR / name)] + argv, stdout=out, stderr=subprocess.PIPE, text=True)
            res[name + "_s"] = round(time.perf_counter() - t0, 3)
            if r.returncode != 0:
                raise RuntimeError(f"{name} failed: {r.stderr[-500:]}")
        res["bat_bytes"] = bat.stat().st_size
        res["par_bytes"] = par.stat().st_size
        res["mie_bytes"] = (d / "mie.txt").stat().st_size
        res["mist_lines"] = sum(1 for _ in open(d / "mist.txt"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    print(json.dumps({"metric": "drop-in pipeline wall clock (run.sh sequence)", "results": res,
                      "config": {"workload": args.workload, "n_atoms": n_atoms, "frames": F, "bins": args.bins,
                                 "input": "fp64" if prec else "fp32"}}), flush=True)
    return 0


def main():
    args = parse()
    if args.ingest:
        return run_ingest(args)
    if args.pipeline:
        return run_pipeline(args)
    if args.mie:
        return run_mie(args)
    if args.batconv:
        return run_batconv(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
