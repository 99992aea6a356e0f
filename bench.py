#!/usr/bin/env python
"""Benchmark of the force-model SGD embedding step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--form F]

Default line (the metric: edge-updates/s of the BF16 batched form against the
FP32 plain form on one GB300, final loss against the FP64 oracle, job p50/p99):

  workload  512 independent graphs, vertex counts log-uniform in [500, 50,000]
            (seed 3); even positions kNN graphs (k=10 of 32-D 10-component Gaussian
            mixtures), odd positions R-MAT (edge factor 8); dim 64, minibatch 256,
            5 shared negatives per minibatch, lr 0.02, 20 epochs per graph,
            U[-0.5, 0.5] initial embeddings (seed 1000 + graph).  Synthetic data.
  step      one persistent launch (a CUDA graph) that trains every graph for its
            20 epochs with BF16 storage, FP32 master copy and FP32 arithmetic; the
            embeddings are reset to their start values before every step (untimed).
  value     edge-updates/s (attractive CSR entries plus repulsive (row, valid
            negative) pairs, counted exactly) with everything resident in HBM.
  e2e       the same job through the public call with the host FP32 embeddings
            copied in and out (pinned), the host sampler and graph capture inside.
  compare   the same 512 graphs with FP32 storage in the same launch; the FP32 plain
            form graph by graph; the FP32 plain form on its own workload (R-MAT
            scale 20, ef 16, dim 128, minibatch 4096, 10-epoch job).
  loss      every graph's final-epoch loss against the FP64 oracle (the reference's
            algorithm in FP64) run on the same graph.
  served    the served form on a Poisson stream (200 jobs/s, the configuration's
            rate) and at half the measured capacity: p50/p99 job latency.
  cpu_baseline  the FP64 port (-O3) on every host core, one graph per thread.

--impl reference times the reference's CPU algorithm (the FP64 port in oracle/,
-O3, every host core, one graph per thread) on the same 512 graphs; one step is
one epoch of every graph.  --form plain|bf16|batched|served|spmm|sparse prints the
line of one form alone (plain: R-MAT scale 20; knn20k: the CPU-runnable 20,000-point kNN
workload; bf16: R-MAT scale 22, dim 256, 1024
shared negatives; batched: the default workload without the other forms; served:
the arrival stream; spmm and sparse: the "next" steps on R-MAT scale 20).

For N > 1 (torchrun) every rank runs an independent replica on its own GPU
(the path does not shard: each job is one resident partition); value sums over
ranks, time is the slowest rank's.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "edge-updates/s BF16 batched vs FP32 plain on 1 GB300 at ≤1% loss gap; job p50/p99"
UNIT = "edge-updates/s"
W = dict(scale=20, edge_factor=16, seed=1, dim=128, batch=4096, ns=5, lr=0.02, epochs=10, init_seed=0)
WORKLOAD = "rmat20_ef16_d128_b4096_ns5_fp32_plain"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--pdl", type=int, default=1, help="plain form: overlap consecutive minibatch launches")
    p.add_argument("--edge-cap", type=int, default=0, help="plain form: max CSR entries per work item (0: automatic)")
    p.add_argument("--stage-negs", type=int, default=0,
                   help="plain form: 1 copies the negative rows into shared memory (bulk copies) per CTA")
    p.add_argument("--form", default="headline",
                   choices=["headline", "plain", "knn20k", "bf16", "batched", "served", "spmm", "sparse"],
                   help="headline (default): the metric's comparison on the batched workload with every other "
                        "form beside it; the others print one form alone")
    p.add_argument("--graphs", type=int, default=512, help="batched workload: number of graphs")
    p.add_argument("--jobs", type=int, default=256, help="served form: jobs in the arrival stream")
    p.add_argument("--scale", type=int, default=0, help="bf16 form: R-MAT scale instead of 22 (small profiling cases)")
    p.add_argument("--slots", type=int, default=16, help="served form: jobs in flight at most")
    p.add_argument("--served-precision", default="fp32", choices=["bf16", "fp32"],
                   help="served form: storage of the jobs (dim 32 jobs run FP32: the BF16 form takes 64-256); "
                        "FP32 serves this stream faster (5 negatives: the BF16 form's GEMMs do not pay)")
    p.add_argument("--no-plain-compare", action="store_true", help="batched form: skip the FP32 plain comparison")
    p.add_argument("--no-served", action="store_true", help="headline: skip the served legs")
    p.add_argument("--no-gap", action="store_true", help="skip the FP64 oracle runs (loss gaps)")
    p.add_argument("--shape", default="", help="batched form: team shape instead of the autotuner, "
                                               "staged|rows:W:cap:steps:stages[:ctas] or register:vpw:W:cap")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(seconds: float, world: int) -> float:
    """The slowest rank's time (the whole job ends when the last replica does)."""
    if world <= 1:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t[0])


def whole_job_rate(units_per_rank: int, seconds: float, world: int) -> float:
    """Replicas: every rank does the same units; value = all ranks' units / slowest time."""
    return units_per_rank * world / max_over_ranks(seconds, world)


def workload():
    from distembed_gb300 import graphgen as gg
    n, rowptr, col = gg.rmat_csr(W["scale"], W["edge_factor"], seed=W["seed"])
    x0 = gg.init_embedding(n, W["dim"], seed=W["init_seed"])
    return n, rowptr, col, x0


def algorithmic_bytes_per_epoch(n, nnz_eff, batches, dim, ns, s=4):
    """Gathers with no reuse credited: per CSR entry its column id and the
    neighbour row; per vertex its rowptr entry, its own row read and written;
    per minibatch the negative rows."""
    return nnz_eff * (4 + dim * s) + n * (8 + 2 * dim * s) + batches * ns * dim * s


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(name="plain_batch_kernel_rmat20.txt"):
    """DRAM bytes per launch of a kernel from its committed ncu summary (the line
    `dram_bytes_per_launch_scaled: <bytes>`), or None."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch_scaled:"):
                return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def spmm_roofline(alg, compulsory, step_s, peak, peak_kind):
    """SpMM step on the DRAM side: the ncu DRAM bytes of one launch (committed
    summary) over the step time; the gathered-row figure (every neighbour row
    counted, hub rows hit in L2, so it can pass the peak) beside it."""
    dram = profile_traffic("spmm_kernel_rmat20.txt")
    basis = "ncu DRAM bytes of one launch (profiles/spmm_kernel_rmat20.txt) / step time"
    if dram is None:
        dram, basis = compulsory, "compulsory bytes (every row once) / step time: no committed capture"
    return {"bound": "hbm", "kernel": "spmm_kernel<128>", "achieved": dram / step_s / 1e9, "peak": peak,
            "unit": "GB/s", "frac": dram / step_s / 1e9 / peak, "peak_source": peak_kind, "traffic": dram,
            "basis": basis, "algorithmic_bytes_per_step": alg, "achieved_gathered": alg / step_s / 1e9,
            "frac_gathered": alg / step_s / 1e9 / peak, "compulsory_bytes_per_step": compulsory,
            "note": "frac is DRAM-side; frac_gathered counts every neighbour row gathered (hub rows come from "
                    "L2, so it exceeds what DRAM moves and can pass 1)"}


def sparse_roofline(alg, step_s, peak, peak_kind):
    """Sparse-embedding step on the DRAM side: the ncu DRAM bytes of the step's
    captured kernels (committed summary: five attractive passes and the prune,
    0.91 of the step's device time) over the step time; the gathered-row figure
    beside it."""
    dram = profile_traffic("sparse_embedding_rmat20.txt")
    return {"bound": "hbm", "kernel": "sparse step (sparse_attract_kernel<128> 5x, collect 5x, count + prune, "
            "mirror, finalize)", "achieved": None if dram is None else dram / step_s / 1e9, "peak": peak,
            "unit": "GB/s", "frac": None if dram is None else dram / step_s / 1e9 / peak,
            "peak_source": peak_kind, "traffic": dram,
            "basis": "ncu DRAM bytes of the captured kernels of a step (profiles/sparse_embedding_rmat20.txt; "
                     "the uncaptured 0.09 of the step's device time not counted) / step time",
            "algorithmic_bytes_per_step": alg, "achieved_gathered": alg / step_s / 1e9,
            "frac_gathered": alg / step_s / 1e9 / peak,
            "note": "frac is DRAM-side; frac_gathered counts every neighbour row gathered, no reuse credited (hub "
                    "rows hit in L2, so it can pass 1)"}


class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [t.strip() for t in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def cpu_sample(rowptr, col, x0, seconds):
    """The FP64 port (the reference's algorithm and its OpenMP structure, -O3
    build, no loss) on every host core: stride-sampled minibatches of epoch 0
    until `seconds` have passed."""
    import oracle
    n = len(rowptr) - 1
    batches = (n + W["batch"] - 1) // W["batch"]
    order = [j for s in (0, 4, 2, 6, 1, 5, 3, 7) for j in range(s, batches, 8)]
    x = np.array(x0, dtype=np.float64, copy=True)
    threads = os.cpu_count() or 1
    updates, done, t0 = 0, 0, time.perf_counter()
    for j in order:
        updates += oracle.run_batches(rowptr, col, x, 0, W["batch"], W["ns"], W["lr"], [j], quirks=True,
                                      threads=threads, fast=True)
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": updates / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "build": "g++ -O3 -ffp-contract=fast -fopenmp (oracle/liboracle_fast.so)",
            "sample": f"{done} of {batches} minibatches of epoch 0 (stride-8 order), FP64, {updates} edge-updates "
                      f"in {dt:.1f} s, OpenMP over the rows of a minibatch as the reference"}

def plain_leg(args, rank, world, local, with_cpu, with_gap):
    """The FP32 plain form on R-MAT scale 20 (dim 128, minibatch 4096, 10-epoch
    job): one step = one epoch.  Returns the line of this form (the keys of the
    bench contract) or None on ranks other than 0."""
    import torch

    import distembed_gb300 as de
    n, rowptr, col, x0 = workload()
    dim, B, ns, lr, E = W["dim"], W["batch"], W["ns"], W["lr"], W["epochs"]
    batches = (n + B - 1) // B

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    h = de.Handle(rowptr, col, dim, device=local, quirks=True, compute_loss=True, pdl=bool(args.pdl),
                  edge_cap=args.edge_cap, stage_negatives=bool(args.stage_negs))
    stream = torch.cuda.ExternalStream(h.stream, device=local)
    h.set_embeddings(x0)
    upd = [h.edge_updates(1, B, ns, first_epoch=e) for e in range(E)]

    for k in range(args.warmup):
        h.run(1, B, ns, lr, want_loss=False, first_epoch=k % E)
    h.sync()
    clocks = Clocks(local)
    events = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    events[0].record(stream)
    for k in range(args.steps):
        h.run(1, B, ns, lr, want_loss=False, first_epoch=k % E)
        events[k + 1].record(stream)
    h.sync()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    step_ms = [events[k].elapsed_time(events[k + 1]) for k in range(args.steps)]
    total_s = max_over_ranks(sum(step_ms) / 1e3, world)
    value = whole_job_rate(sum(upd[k % E] for k in range(args.steps)), total_s, world)

    # roofline of the dominant kernel (the per-minibatch kernel: all but one
    # launch of an epoch); per launch = epoch time / launches, gaps included
    nnz_eff = len(col) - int(np.sum(col == n - 1))
    alg_epoch = algorithmic_bytes_per_epoch(n, nnz_eff, batches, dim, ns)
    mean_epoch_s = statistics.mean(step_ms) / 1e3
    achieved = alg_epoch / mean_epoch_s / 1e9
    # one extra epoch with an event around every launch (no overlap between launches)
    pms, kind = h.profile_epoch(B, ns, lr, first_epoch=0)
    launch_us = float(pms[kind == 0].mean()) * 1e3
    serial_achieved = alg_epoch / (float(pms[kind == 0].sum()) / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = profile_traffic()
    dram_gbs = traffic * batches / mean_epoch_s / 1e9 if traffic else None

    # end to end: the reference-facing call on pinned host FP64 buffers
    e2e = None
    if args.e2e_steps > 0:
        x_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
        x_host[:] = x0
        out_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
        e2e_times = []
        for k in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            h.set_embeddings(x_host)
            loss = h.run(E, B, ns, lr, want_loss=True)
            h.get_embeddings(out=out_host)
            t1 = time.perf_counter()
            if k > 0:
                e2e_times.append(t1 - t0)
        e2e_units = sum(upd) * world
        e2e_s = max_over_ranks(statistics.mean(e2e_times), world)
        h2d = n * dim * 8 + E * batches * ns * 4 + E * 4 + 8
        d2h = n * dim * 8 + E * 8
        e2e = {"value": e2e_units / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "step": "EmbeddingAlgo call: host FP64 x in, 10 epochs, host FP64 x out (pinned)",
               "ms_per_step": 1e3 * e2e_s, "final_loss": float(loss[-1])}

    gap = None
    if rank == 0 and world == 1 and with_gap:
        # the whole 10-epoch job against the FP64 oracle at full size, from the
        # same (FP32-rounded) start
        import oracle
        xs = x0.astype(np.float32).astype(np.float64)
        h.set_embeddings(xs)
        gloss = h.run(E, B, ns, lr, want_loss=True)
        gx = h.get_embeddings()
        t1 = time.perf_counter()
        ox, oloss = oracle.run(rowptr, col, xs, E, B, ns, lr, quirks=True, threads=os.cpu_count() or 1)
        gap = {"loss_rel_per_epoch": [float(v) for v in np.abs(gloss - oloss) / oloss],
               "loss_rel_max": float(np.max(np.abs(gloss - oloss) / oloss)),
               "final_loss_rel": float(abs(gloss[-1] - oloss[-1]) / oloss[-1]),
               "x_rel_l2": float(np.linalg.norm(gx - ox) / np.linalg.norm(ox)),
               "oracle_s": round(time.perf_counter() - t1, 1),
               "bound": "per-epoch loss within 1e-3, embedding within 1e-4 relative L2 (tests/test_gpu_cfg2.py)"}

    cpu = None
    if rank == 0 and world == 1 and with_cpu:
        cpu = cpu_sample(rowptr, col, x0, args.cpu_seconds)
    h.close()
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: R-MAT scale 20 (ef 16, a.57 b.19 c.19, seed 1), U[-0.5,0.5] init (seed 0)",
        "config": {"workload": WORKLOAD, "n": n, "nnz": int(len(col)), "dim": dim, "batch": B, "ns": ns,
                   "lr": lr, "epochs_per_job": E, "step": "one epoch (256 minibatches, CUDA graph)",
                   "l2": "inputs larger than L2 (512 MiB FP32 embedding); no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU", "ref_quirks": True,
                   "pdl": bool(args.pdl), "edge_cap": args.edge_cap, "stage_negatives": bool(args.stage_negs)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "kernel": "plain_batch_kernel<128>",
                     "algorithmic_bytes_per_epoch": alg_epoch,
                     "dram_gbs": dram_gbs, "dram_frac": dram_gbs / peak if dram_gbs else None,
                     "note": "achieved = algorithmic bytes / epoch time over 256 launches (gaps included); "
                             "dram_gbs = ncu DRAM bytes per launch (profiles/plain_batch_kernel_rmat20.txt) x "
                             "launches / epoch time",
                     "launch_us_serial": launch_us, "achieved_serial_launches": serial_achieved},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gap_vs_fp64_oracle": gap,
        "gpu_launches": args.steps * (batches + 1),
        "clocks": clk,
    }


def run_plain_form(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        torch.distributed.init_process_group("gloo")
    torch.cuda.set_device(local)
    line = plain_leg(args, rank, world, local, with_cpu=not args.no_cpu_baseline, with_gap=not args.no_gap)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


W1 = dict(n=20000, pts_dim=64, k=15, components=10, seed=0, dim=128, batch=256, ns=5, lr=0.02, epochs=30, init_seed=0)


def l2_copy_peak(device=0):
    """Copy bandwidth of buffers that stay in L2 (24 MiB read + 24 MiB written per
    copy, 20 copies between two CUDA events, best of 10): the measured L2-side peak."""
    import torch
    a = torch.empty(6 << 20, dtype=torch.float32, device=device)
    b = torch.empty_like(a)
    b.copy_(a)
    best = None
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(20):
            b.copy_(a)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 20
        best = t if best is None else min(best, t)
    return 2 * a.numel() * 4 / (best / 1e3) / 1e9


def run_knn20k_form(args):
    """The CPU-runnable workload on the GPU: 20,000-point 64-D Gaussian-mixture kNN
    graph (k=15, symmetrised), dim 128, minibatch 256, 5 negatives, lr 0.02 decayed
    linearly over 30 epochs.  One step = one epoch (79 minibatches, CUDA graph).
    The embedding (10 MB) stays in L2, so the step is latency-bound, not HBM-bound."""
    import torch

    import distembed_gb300 as de
    import oracle
    from distembed_gb300 import graphgen as gg
    torch.cuda.set_device(0)
    n, rowptr, col = gg.knn_csr(W1["n"], W1["pts_dim"], W1["k"], W1["components"], seed=W1["seed"])
    x0 = gg.init_embedding(n, W1["dim"], seed=W1["init_seed"]).astype(np.float32).astype(np.float64)
    dim, B, ns, E = W1["dim"], W1["batch"], W1["ns"], W1["epochs"]
    lrs = [W1["lr"] * (1 - e / E) for e in range(E)]
    batches = (n + B - 1) // B
    h = de.Handle(rowptr, col, dim, quirks=True, compute_loss=False, pdl=bool(args.pdl))
    stream = torch.cuda.ExternalStream(h.stream, device=0)
    h.set_embeddings(x0)
    upd = [h.edge_updates(1, B, ns, first_epoch=e) for e in range(E)]
    for k in range(args.warmup):
        h.run(1, B, ns, lrs[k % E], want_loss=False, first_epoch=k % E)
    h.sync()
    clocks = Clocks(0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev[0].record(stream)
    for k in range(args.steps):
        h.run(1, B, ns, lrs[k % E], want_loss=False, first_epoch=k % E)
        ev[k + 1].record(stream)
    h.sync()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    value = sum(upd[k % E] for k in range(args.steps)) / (sum(step_ms) / 1e3)
    nnz_eff = len(col) - int(np.sum(col == n - 1))
    alg = algorithmic_bytes_per_epoch(n, nnz_eff, batches, dim, ns)
    achieved = alg / (statistics.mean(step_ms) / 1e3) / 1e9
    l2 = l2_copy_peak(0)
    pms, kind = h.profile_epoch(B, ns, lrs[0], first_epoch=0)
    launch_us = float(pms[kind == 0].mean()) * 1e3
    # end to end: the reference-facing call, host FP64 in, the 30-epoch job, host FP64 out
    x_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
    x_host[:] = x0
    out_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
    ts = []
    for k in range(max(args.e2e_steps, 1) + 1):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        h.set_embeddings(x_host)
        h.run(E, B, ns, lrs, want_loss=False)
        h.get_embeddings(out=out_host)
        if k > 0:
            ts.append(time.perf_counter() - t1)
    h.close()
    e2e = {"value": sum(upd) / statistics.mean(ts), "unit": UNIT, "h2d_bytes_per_step": n * dim * 8 + E * batches * ns * 4,
           "d2h_bytes_per_step": n * dim * 8, "ms_per_step": 1e3 * statistics.mean(ts),
           "step": "EmbeddingAlgo call: host FP64 x in (pinned), 30 epochs, host FP64 x out"}
    # the whole job against the FP64 oracle, and the CPU baseline on the same job
    with de.Handle(rowptr, col, dim, quirks=True) as hl:
        hl.set_embeddings(x0)
        lg = hl.run(E, B, ns, lrs)
        xg = hl.get_embeddings()
    threads = os.cpu_count() or 1
    xo, lo = oracle.run(rowptr, col, x0, E, B, ns, lrs, quirks=True, threads=threads)
    t1 = time.perf_counter()
    oracle.run(rowptr, col, x0, E, B, ns, lrs, quirks=True, threads=threads, want_loss=False, fast=True)
    cs = time.perf_counter() - t1
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic: 20,000 points of a 10-component 64-D Gaussian mixture (seed 0, means ~N(0,4I)), exact "
                    "kNN k=15 symmetrised; U[-0.5,0.5] init (seed 0)",
            "config": {"workload": "knn20k_d128_b256_ns5_e30_fp32_plain", "n": n, "nnz": int(len(col)), "dim": dim,
                       "batch": B, "ns": ns, "lr": "0.02 (1 - e/30)", "epochs_per_job": E,
                       "step": f"one epoch ({batches} minibatches, CUDA graph)",
                       "l2": "L2-resident (10 MB FP32 embedding): latency-bound; no flush"},
            "roofline": {"bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
                         "peak_source": "measured here: L2-resident copy (24 MiB), 20 per event pair, best of 10",
                         "kernel": "plain_batch_kernel<128>", "algorithmic_bytes_per_epoch": alg,
                         "launch_us_serial": launch_us, "launches_per_epoch": batches + 1,
                         "note": "79 dependent minibatch launches per epoch of 256 rows each: one launch is a few "
                                 "microseconds of work, so launch latency and the minibatch chain bound it"},
            "cpu_baseline": {"value": sum(upd) / cs, "unit": UNIT, "cores": threads, "kind": "port",
                             "build": "g++ -O3 -ffp-contract=fast -fopenmp (oracle/liboracle_fast.so)",
                             "sample": f"the whole 30-epoch job, FP64, OpenMP over the rows of a minibatch, {cs:.2f} s"},
            "e2e": e2e,
            "gap_vs_fp64_oracle": {"loss_rel_max": float(np.max(np.abs(lg - lo) / lo)),
                                   "final_loss_rel": float(abs(lg[-1] - lo[-1]) / lo[-1]),
                                   "x_rel_l2_final": float(np.linalg.norm(xg - xo) / np.linalg.norm(xo))},
            "gpu_launches": args.steps * (batches + 1), "clocks": clk}
    print(json.dumps(line), flush=True)


W3 = dict(scale=22, edge_factor=16, seed=2, dim=256, batch=8192, ns=1024, lr=0.02, epochs=10, init_seed=0)
WORKLOAD3 = "rmat22_ef16_d256_b8192_ns1024"


def timed_job(h, E, B, ns, lr, stream, warmup):
    """Runs `warmup` epochs, then one E-epoch job with CUDA events around each
    epoch; returns (per-epoch ms, per-epoch FP64 loss of the job)."""
    import torch
    for k in range(warmup):
        h.run(1, B, ns, lr, want_loss=False, first_epoch=k % E)
    h.sync()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(E + 1)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for e in range(E):
        h.run(1, B, ns, lr, want_loss=False, first_epoch=e)
        ev[e + 1].record(stream)
    h.sync()
    torch.cuda.synchronize()
    ms = [ev[e].elapsed_time(ev[e + 1]) for e in range(E)]
    return ms


def run_bf16_form(args):
    """BF16 precision form against the FP32 plain form on the same 10-epoch job."""
    import torch

    import distembed_gb300 as de
    from distembed_gb300 import graphgen as gg
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    scale = args.scale or W3["scale"]
    n, rowptr, col = gg.rmat_csr(scale, W3["edge_factor"], seed=W3["seed"])
    x0 = gg.init_embedding(n, W3["dim"], seed=W3["init_seed"]).astype(np.float32)
    gen_s = time.perf_counter() - t0
    dim, B, ns, lr, E = W3["dim"], W3["batch"], W3["ns"], W3["lr"], W3["epochs"]
    batches = -(-n // B)
    out, clk, e2e = {}, None, None
    names = {0: "minibatch/attractive", 1: "repulsion_gemm", 2: "update_exact_rows", 3: "flush", 4: "negative_gather"}
    final_x = {}
    for form in ("fp32", "bf16"):
        # the same job twice: timed on a handle that computes no loss (the
        # reference computes none), then again on one that does, for the losses
        with de.Handle(rowptr, col, dim, precision=form, quirks=True, compute_loss=True, pdl=bool(args.pdl)) as hl:
            hl.set_embeddings(x0)
            loss = hl.run(E, B, ns, lr, want_loss=True)
            final_x[form] = hl.get_embeddings()
        h = de.Handle(rowptr, col, dim, precision=form, quirks=True, compute_loss=False, pdl=bool(args.pdl))
        stream = torch.cuda.ExternalStream(h.stream, device=0)
        h.set_embeddings(x0)
        upd = [h.edge_updates(1, B, ns, first_epoch=e) for e in range(E)]
        clocks = Clocks(0)
        if form == "bf16":
            clocks.start()
        ms = timed_job(h, E, B, ns, lr, stream, warmup=1)
        if form == "bf16":
            clk = clocks.stop()
        pms, kind = h.profile_epoch(B, ns, lr)      # one more epoch, an event around every launch
        out[form] = {"edge_updates_per_s": sum(upd) / (sum(ms) / 1e3), "ms_per_epoch": statistics.mean(ms),
                     "loss_per_epoch": [float(v) for v in loss],
                     "profiled_epoch_ms": {names[k]: round(float(pms[kind == k].sum()), 3) for k in sorted(set(kind.tolist()))}}
        if form == "bf16" and args.e2e_steps > 0:
            # end to end through the public API: pinned host FP32 in, the 10-epoch job, host FP32 out
            x_host = torch.empty((n, dim), dtype=torch.float32, pin_memory=True).numpy()
            x_host[:] = x0
            o_host = torch.empty((n, dim), dtype=torch.float32, pin_memory=True).numpy()
            ts = []
            for k in range(args.e2e_steps + 1):
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                h.set_embeddings(x_host)
                h.run(E, B, ns, lr, want_loss=False)
                h.get_embeddings(out=o_host)
                if k > 0:
                    ts.append(time.perf_counter() - t1)
            e2e = {"value": sum(upd) / statistics.mean(ts), "unit": UNIT, "h2d_bytes_per_step": n * dim * 4,
                   "d2h_bytes_per_step": n * dim * 4, "ms_per_step": 1e3 * statistics.mean(ts),
                   "step": "host FP32 embedding in (pinned), the 10-epoch job, host FP32 embedding out"}
        h.close()
    # rooflines from the per-launch event times of the profiled BF16 epoch
    prof = out["bf16"]["profiled_epoch_ms"]
    rows_total = n  # every vertex is a GEMM row once per epoch (quirks: the repulsive rows of
    #                 the last minibatch are last_batch_size, the same count)
    kpad = max(64, -(-ns // 64) * 64)
    gemm_flops = 4.0 * rows_total * kpad * dim
    tflops = gemm_flops / (prof["repulsion_gemm"] / 1e3) / 1e12
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        tpeak, tsrc = float(peaks["bf16_tflops"]), "measured (burst)"
    except Exception:
        tpeak, tsrc = 1900.0, "fallback"
    nnz_eff = int(len(col))
    attr_bytes = nnz_eff * (4 + 2 * dim) + n * (8 + 2 * dim + 4 * dim)
    hpeak, hsrc = measured_peak()
    attr_gbs = attr_bytes / (prof["minibatch/attractive"] / 1e3) / 1e9
    roof_gemm = {"bound": "tensor", "kernel": "bf16_repulse_kernel<256>", "achieved": tflops, "peak": tpeak,
                 "unit": "TFLOP/s", "frac": tflops / tpeak, "peak_source": tsrc, "traffic": None,
                 "algorithmic_flops_per_epoch": gemm_flops,
                 "note": "4 x rows x kpad x dim per epoch (two GEMMs) / summed event time of the GEMM launches"}
    roof_attr = {"bound": "hbm", "kernel": "bf16_attract_kernel<256>", "achieved": attr_gbs, "peak": hpeak,
                 "unit": "GB/s", "frac": attr_gbs / hpeak, "peak_source": hsrc,
                 "algorithmic_bytes_per_epoch": attr_bytes,
                 "note": "per CSR entry: column id + BF16 neighbour row; per vertex: rowptr, own BF16 row, FP32 update row"}
    dominant_gemm = prof["repulsion_gemm"] >= prof["minibatch/attractive"]
    gap = abs(out["bf16"]["loss_per_epoch"][-1] - out["fp32"]["loss_per_epoch"][-1]) / out["fp32"]["loss_per_epoch"][-1]
    # every epoch against the FP64 oracle: the GPU restatement (bitwise the CPU
    # oracle's arithmetic, tests/test_gpu_oracle64.py), same FP32-rounded start
    fp64 = None
    if not args.no_gap:
        import oracle
        t1 = time.perf_counter()
        xo, lo = oracle.gpu_run(rowptr, col, x0.astype(np.float64), E, B, ns, lr, quirks=True)
        fp64 = {"oracle": "oracle/liboracle_gpu.so (FP64, bitwise the CPU oracle on small graphs)",
                "oracle_s": round(time.perf_counter() - t1, 1), "loss_per_epoch": [float(v) for v in lo]}
        for form in ("bf16", "fp32"):
            lg = np.asarray(out[form]["loss_per_epoch"])
            fp64[form] = {"loss_rel_per_epoch": [float(v) for v in np.abs(lg - lo) / lo],
                          "loss_rel_max": float(np.max(np.abs(lg - lo) / lo)),
                          "x_rel_l2_final": float(np.linalg.norm(final_x[form] - xo) / np.linalg.norm(xo))}
    line = {"metric": METRIC, "value": out["bf16"]["edge_updates_per_s"], "unit": UNIT, "n_gpus": 1, "steps": E,
            "warmup": 1, "ms_per_step": out["bf16"]["ms_per_epoch"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16",
            "data": f"synthetic: R-MAT scale {scale} (ef 16, a.57 b.19 c.19, seed 2), U[-0.5,0.5] init (seed 0)",
            "config": {"workload": (WORKLOAD3 if scale == W3["scale"] else f"rmat{scale}_ef16_d256_b8192_ns1024") + "_bf16", "n": n, "nnz": int(len(col)), "dim": dim, "batch": B,
                       "ns": ns, "lr": lr, "epochs_per_job": E, "step": f"one epoch ({-(-n // B)} minibatches)",
                       "generate_s": round(gen_s, 1)},
            "roofline": roof_gemm if dominant_gemm else roof_attr,
            "roofline_other": roof_attr if dominant_gemm else roof_gemm,
            "e2e": e2e, "clocks": clk, "gpu_launches": E * (4 * batches + 1),
            "compare": {"fp32_plain": {k: v for k, v in out["fp32"].items()}, "bf16": out["bf16"],
                        "bf16_over_fp32": out["bf16"]["edge_updates_per_s"] / out["fp32"]["edge_updates_per_s"],
                        "final_loss_gap_vs_fp32": gap},
            "gap_vs_fp64_oracle": fp64}
    print(json.dumps(line), flush=True)

W4 = dict(n_lo=500, n_hi=50000, seed=3, dim=64, batch=256, ns=5, lr=0.02, epochs=20, init_seed=1000,
          knn_k=10, knn_dim=32, rmat_ef=8)


def batched_workload(count, device):
    from distembed_gb300 import graphgen as gg
    graphs = gg.graph_suite(count, W4["n_lo"], W4["n_hi"], W4["seed"], knn_k=W4["knn_k"], knn_dim=W4["knn_dim"],
                            rmat_ef=W4["rmat_ef"], device=device)
    x0 = [gg.init_embedding(n, W4["dim"], seed=W4["init_seed"] + i).astype(np.float32)
          for i, (_, n, _, _) in enumerate(graphs)]
    return graphs, x0


def batched_config(graphs):
    """The workload of the default line (the same dict in both arms)."""
    return {"workload": f"batched{len(graphs)}_knn_rmat_d64_b256_ns5_e20", "graphs": len(graphs),
            "vertices": int(sum(n for _, n, _, _ in graphs)), "nnz": int(sum(len(c) for _, _, _, c in graphs)),
            "dim": W4["dim"], "batch": W4["batch"], "ns": W4["ns"], "lr": W4["lr"], "epochs_per_job": W4["epochs"],
            "kinds": "even graphs kNN (k=10, 32-D 10-component mixtures), odd graphs R-MAT (ef 8)",
            "ref_quirks": True}


BATCHED_DATA = ("synthetic: {g} graphs, n log-uniform [500, 50000] (seed 3), even: kNN k=10 of 32-D 10-component "
                "mixtures (FP32 kNN on the GPU), odd: R-MAT ef 8; U[-0.5,0.5] init (seed 1000+i)")


def batched_bytes_per_epoch(graphs, dim, B, ns, s=2):
    """Algorithmic bytes of one epoch of every graph (no reuse credited): per CSR
    entry its column id and the neighbour row (s bytes per component); per vertex
    its rowptr entry, its own row read, the FP32 master read and written and (BF16)
    the BF16 copy written; per minibatch the ns negative rows."""
    tot = 0
    for _, n, rp, c in graphs:
        nnz_eff = len(c) - int(np.sum(c == n - 1))
        batches = (n + B - 1) // B
        copy = dim * s if s == 2 else 0
        tot += nnz_eff * (4 + dim * s) + n * (8 + dim * s + 2 * dim * 4 + copy) + batches * ns * dim * s
    return tot


def parse_shape(text):
    f = text.split(":")
    if f[0] in ("staged", "rows"):
        return dict(kernel=f[0], team_warps=int(f[1]), edge_cap=int(f[2]), pairs=int(f[3]), stages=int(f[4]),
                    team_ctas=int(f[5]) if len(f) > 5 else 1)
    return dict(kernel="register", vertices_per_warp=int(f[1]), team_warps=int(f[2]), edge_cap=int(f[3]))


def batched_leg(graphs, x0_all, precision, local, steps, warmup, e2e_steps=0, shape=None, clocks=False):
    """The batched form on `graphs`: autotuned (or the given shape), then `warmup`
    untimed and `steps` timed launches of the whole 20-epoch job, the embeddings
    reset to x0_all before each (untimed).  Returns a dict of measurements."""
    import torch

    import distembed_gb300 as de
    dim, B, ns, lr, E = W4["dim"], W4["batch"], W4["ns"], W4["lr"], W4["epochs"]
    total_n = int(sum(n for _, n, _, _ in graphs))
    b = de.Batch([(rp, c) for _, _, rp, c in graphs], dim, precision=precision, device=local)
    stream = torch.cuda.ExternalStream(b.stream, device=local)
    x_start = torch.empty((total_n, dim), dtype=torch.float32, pin_memory=True).numpy()
    x_start[:] = x0_all
    b.set_embeddings(-1, x_start)
    t0 = time.perf_counter()
    tuned = []
    if shape:
        try:
            b.set_shape(**shape)
            b.prepare(E, B, ns, lr)
        except de.DEError:  # the shape does not fit this precision: tune
            shape = None
    if not shape:
        shape, tuned = b.autotune(1, B, ns, lr)
    tune_s = time.perf_counter() - t0
    upd = b.edge_updates(E, B, ns)
    b.prepare(E, B, ns, lr)
    b.set_embeddings(-1, x_start)
    b.launch()
    loss = b.wait()            # the job's loss, every epoch (for the oracle comparison)
    trace = b.trace()
    # the timed launches compute the loss of the job's last epoch only (the one
    # the metric's loss gap is taken on); the other epochs take no logarithm
    b.set_loss("last")
    b.prepare(E, B, ns, lr)
    for _ in range(warmup):
        b.set_embeddings(-1, x_start)
        b.launch()
        b.wait()
    clk_rec = Clocks(local) if clocks else None
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * steps)]
    torch.cuda.synchronize()
    if clk_rec:
        clk_rec.start()
        time.sleep(0.3)
    for k in range(steps):
        b.set_embeddings(-1, x_start)
        ev[2 * k].record(stream)
        b.launch()
        ev[2 * k + 1].record(stream)
        b.wait()
    torch.cuda.synchronize()
    clk = clk_rec.stop() if clk_rec else None
    step_ms = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(steps)]
    e2e = None
    if e2e_steps > 0:
        # the public call: host FP32 embeddings in, de_batch_run (host sampler,
        # upload of the draws, graph capture, the launch, the losses back), host out
        x_host = torch.empty((total_n, dim), dtype=torch.float32, pin_memory=True).numpy()
        x_host[:] = x0_all
        out_host = torch.empty((total_n, dim), dtype=torch.float32, pin_memory=True).numpy()
        ts = []
        for k in range(e2e_steps + 1):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            b.set_embeddings(-1, x_host)
            e2e_loss = b.run(E, B, ns, lr)
            b.get_embeddings(-1, out=out_host)
            if k > 0:
                ts.append(time.perf_counter() - t1)
        negs = sum(((n + B - 1) // B) * E * ns for _, n, _, _ in graphs)
        e2e = {"value": upd / statistics.mean(ts), "unit": UNIT,
               "h2d_bytes_per_step": total_n * dim * 4 + negs * 4 + E * 4,
               "d2h_bytes_per_step": total_n * dim * 4 + len(graphs) * E * 8,
               "ms_per_step": 1e3 * statistics.mean(ts),
               "step": "host FP32 embeddings of every graph in (pinned), de_batch_run (host sampler, draws "
                       "uploaded, graph captured, the 20-epoch launch, final-epoch losses back), host FP32 out",
               "final_loss_equal_to_timed_job": bool(np.array_equal(e2e_loss[:, -1], loss[:, -1]))}
        b.prepare(E, B, ns, lr)
    b.close()
    span = trace[:, 1] - trace[:, 0]
    ends = {}
    for t, e in zip(trace[:, 2].tolist(), trace[:, 1].tolist()):
        ends[t] = max(ends.get(t, 0), e)
    ends = np.array(sorted(ends.values()), dtype=np.float64) / 1e6
    return {"edge_updates": upd, "step_ms": step_ms, "value": upd * len(step_ms) / (sum(step_ms) / 1e3), "loss": loss,
            "shape": shape, "tuned": tuned, "tune_s": tune_s, "e2e": e2e, "clocks": clk,
            "trace": {"makespan_ms": float(trace[:, 1].max()) / 1e6, "longest_graph_ms": float(span.max()) / 1e6,
                      "graph_ms_sum": float(span.sum()) / 1e6, "teams": int(len(np.unique(trace[:, 2]))),
                      "team_end_ms_p10_p50_p90": [float(np.percentile(ends, q)) for q in (10, 50, 90)],
                      "note": "the launch that computes every epoch's loss (the timed ones compute the last "
                              "epoch's only)"}}


def plain_same_graphs(graphs, x0, local):
    """The FP32 plain form on the same graphs, one graph after another: device
    time of each 20-epoch job summed (the graph capture of each job untimed)."""
    import torch

    import distembed_gb300 as de
    B, ns, lr, E, dim = W4["batch"], W4["ns"], W4["lr"], W4["epochs"], W4["dim"]
    plain_ms, plain_upd = 0.0, 0
    for i, (_, n, rp, c) in enumerate(graphs):
        with de.Handle(rp, c, dim, quirks=True, compute_loss=True, device=local) as h:
            st = torch.cuda.ExternalStream(h.stream, device=local)
            h.set_embeddings(x0[i])
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            h.run(1, B, ns, lr, want_loss=False)            # capture outside the timed region
            h.set_embeddings(x0[i])
            h.sync()
            e0.record(st)
            h.run(E, B, ns, lr, want_loss=False)
            e1.record(st)
            h.sync()
            plain_ms += e0.elapsed_time(e1)
            plain_upd += h.edge_updates(E, B, ns)
    return {"edge_updates_per_s": plain_upd / (plain_ms / 1e3), "job_ms": plain_ms,
            "note": "FP32 plain form, one graph after another, device time of each 20-epoch job summed"}


def gap_stats(loss, ref, kinds):
    """Per-graph final-epoch relative gaps of `loss` against `ref` ([graphs, epochs])."""
    g = np.abs(loss[:, -1] - ref[:, -1]) / ref[:, -1]

    def st(sel):
        v = g[sel]
        return {"graphs": int(len(v)), "p50": float(np.percentile(v, 50)), "p90": float(np.percentile(v, 90)),
                "max": float(v.max()), "within_1pct": int(np.sum(v <= 0.01))}

    kinds = np.asarray(kinds)
    job = np.abs(loss.sum(0) - ref.sum(0)) / ref.sum(0)
    return {"job_sum_final": float(job[-1]), "job_sum_max_over_epochs": float(job.max()),
            "all": st(np.ones(len(g), bool)), "knn": st(kinds == "knn"), "rmat": st(kinds == "rmat")}


def fp64_oracle_losses(graphs, x0):
    """Every graph's 20-epoch job in the FP64 oracle (bit-exact build, one graph
    per host thread): loss [graphs, epochs]."""
    import oracle
    xs = [np.ascontiguousarray(x, dtype=np.float64) for x in x0]
    _, loss = oracle.run_many([(rp, c) for _, _, rp, c in graphs], xs, W4["epochs"], W4["batch"], W4["ns"],
                              W4["lr"], threads=os.cpu_count() or 1)
    return loss


def batched_cpu_baseline(graphs, x0, seconds):
    """The FP64 port (-O3 build, no loss) on every host core, one graph per
    thread: whole epochs of every graph until `seconds` have passed."""
    import oracle
    xs = [np.ascontiguousarray(x, dtype=np.float64) for x in x0]
    threads = os.cpu_count() or 1
    csr = [(rp, c) for _, _, rp, c in graphs]
    u, e, t0 = 0, 0, time.perf_counter()
    while e < W4["epochs"]:
        du, _ = oracle.run_many(csr, xs, 1, W4["batch"], W4["ns"], W4["lr"], first_epoch=e, want_loss=False,
                                threads=threads, fast=True)
        u += du
        e += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": u / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "build": "g++ -O3 -ffp-contract=fast -fopenmp (oracle/liboracle_fast.so)",
            "sample": f"epochs 0..{e - 1} of all {len(graphs)} graphs, FP64, one graph per thread, {u} edge-updates "
                      f"in {dt:.1f} s"}


def roofline_batched(graphs, step_ms, precision="bf16"):
    alg = batched_bytes_per_epoch(graphs, W4["dim"], W4["batch"], W4["ns"], s=2 if precision == "bf16" else 4) \
        * W4["epochs"]
    mean_s = statistics.mean(step_ms) / 1e3
    peak, peak_kind = measured_peak()
    traffic = profile_traffic("staged_kernel_batched512.txt")
    achieved = alg / mean_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind, "traffic": traffic, "kernel": "staged_kernel (batched, persistent)",
            "algorithmic_bytes_per_launch": alg,
            "dram_gbs": traffic / mean_s / 1e9 if traffic else None,
            "dram_frac": traffic / mean_s / 1e9 / peak if traffic else None,
            "note": "one launch per step; achieved = algorithmic bytes (no reuse credited) / launch time"}


def run_batched_form(args):
    """The batched form alone: BF16 batched against FP32 storage in the same launch,
    the FP32 plain form on the same graphs, and the FP64 oracle on every graph."""
    import torch
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    graphs, x0 = batched_workload(args.graphs, "cuda")
    gen_s = time.perf_counter() - t0
    x0_all = np.concatenate(x0)
    kinds = [k for k, _, _, _ in graphs]
    shape = parse_shape(args.shape) if args.shape else None
    bf = batched_leg(graphs, x0_all, "bf16", 0, args.steps, args.warmup, args.e2e_steps, shape=shape, clocks=True)
    f32 = batched_leg(graphs, x0_all, "fp32", 0, max(1, args.steps // 4), 1, 0, shape=bf["shape"])
    plain = None if args.no_plain_compare else plain_same_graphs(graphs, x0, 0)
    loss = None
    if not args.no_gap:
        lo = fp64_oracle_losses(graphs, x0)
        loss = {"bf16_vs_fp64_oracle": gap_stats(bf["loss"], lo, kinds),
                "fp32_storage_vs_fp64_oracle": gap_stats(f32["loss"], lo, kinds)}
    cpu = None if args.no_cpu_baseline else batched_cpu_baseline(graphs, x0, args.cpu_seconds)
    line = {"metric": METRIC, "value": bf["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(bf["step_ms"]), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": BATCHED_DATA.format(g=len(graphs)),
            "config": batched_config(graphs),
            "impl_detail": {"team_shape": bf["shape"], "autotune_s": round(bf["tune_s"], 2),
                            "autotune_shapes": len(bf["tuned"]), "trace": bf["trace"], "generate_s": round(gen_s, 1),
                            "reset": "embeddings reset to the start values before every step (untimed)",
                            "l2": "inputs larger than L2 (embeddings of every graph); no flush"},
            "roofline": roofline_batched(graphs, bf["step_ms"]),
            "loss": loss,
            "compare": {"fp32_storage_batched": {"edge_updates_per_s": f32["value"],
                                                 "ms_per_step": statistics.mean(f32["step_ms"]), "shape": f32["shape"]},
                        "fp32_plain_same_graphs": plain},
            "cpu_baseline": cpu, "e2e": bf["e2e"], "gpu_launches": args.steps, "clocks": bf["clocks"]}
    print(json.dumps(line), flush=True)


W5 = dict(rate=200.0, seed=4, n_lo=1000, n_hi=2_000_000, dims=(32, 64, 128), epochs=(10, 50), batch=16384, ns=5,
          lr=0.02, knn_max_n=100_000, rmat_ef=8, knn_k=10, knn_dim=32)


def served_workload(count, device):
    """The arrival stream: Poisson arrivals (mean W5['rate'] jobs/s), n log-uniform,
    R-MAT or kNN (kNN only up to knn_max_n vertices: exact kNN of millions of
    points is not generated here), dim and epochs uniform.  Every job uses the
    reference driver's defaults for the rest (minibatch 16384, 5 negatives,
    lr 0.02, cpp/dist_embed.cpp:46-51)."""
    from distembed_gb300 import graphgen as gg
    rng = np.random.Generator(np.random.PCG64(W5["seed"]))
    arrivals = np.cumsum(rng.exponential(1.0 / W5["rate"], size=count))
    arrivals -= arrivals[0]
    ns_ = np.rint(np.exp(rng.uniform(np.log(W5["n_lo"]), np.log(W5["n_hi"]), size=count))).astype(np.int64)
    kinds = rng.integers(0, 2, size=count)
    dims = rng.choice(W5["dims"], size=count)
    epochs = rng.integers(W5["epochs"][0], W5["epochs"][1] + 1, size=count)
    jobs = []
    for i in range(count):
        n = int(ns_[i])
        if kinds[i] == 1 and n <= W5["knn_max_n"]:
            _, rp, col = gg.knn_csr(n, W5["knn_dim"], W5["knn_k"], 10, seed=W5["seed"] * 100003 + i, device=device)
            kind = "knn"
        else:
            _, rp, col = gg.rmat_csr_torch(n, W5["rmat_ef"], seed=W5["seed"] * 100003 + i, device=device)
            kind = "rmat"
        jobs.append(dict(arrival=float(arrivals[i]), kind=kind, n=n, rowptr=rp, col=col, dim=int(dims[i]),
                         epochs=int(epochs[i])))
    return jobs


class ServedStart:
    """Every job starts from a slice of one seeded U[-0.5, 0.5) pool."""

    def __init__(self, jobs):
        nmax = max(j["n"] for j in jobs)
        self.pool = np.random.Generator(np.random.PCG64(1)).uniform(-0.5, 0.5, size=nmax * 128).astype(np.float32)

    def __call__(self, j):
        return self.pool[: j["n"] * j["dim"]].reshape(j["n"], j["dim"])


def job_precision(j, precision):
    """BF16 storage for the jobs the BF16 form takes (dim 64-256), FP32 otherwise."""
    return "bf16" if precision == "bf16" and j["dim"] >= 64 else "fp32"


def served_leg(jobs, x0_of, slots, precision, time_scale, local, clocks=False):
    """The arrival stream through de_server with arrival times scaled by
    `time_scale` (1: the configuration's 200 jobs/s): jobs overlap on the GPU as
    slots and memory allow.  Returns latency percentiles and throughput."""
    import threading

    import distembed_gb300 as de
    B, ns, lr = W5["batch"], W5["ns"], W5["lr"]
    srv = de.Server(slots=slots, hbm_fraction=0.85, device=local)
    for j in sorted(jobs, key=lambda j: j["n"])[:4]:  # warm-up: module load, first launches
        srv.wait(srv.submit(j["rowptr"], j["col"], x0_of(j), 2, B, ns, lr, precision=job_precision(j, precision)))
    results = [None] * len(jobs)
    ids = [None] * len(jobs)
    ready = threading.Semaphore(0)

    def waiter():
        for i in range(len(jobs)):
            ready.acquire()
            x, loss, info = srv.wait(ids[i])
            results[i] = (float(loss[-1]), info)

    th = threading.Thread(target=waiter)
    clk_rec = Clocks(local) if clocks else None
    if clk_rec:
        clk_rec.start()
    th.start()
    start = srv.clock() + 0.05
    for i, j in enumerate(jobs):
        delay = start + j["arrival"] * time_scale - srv.clock()
        if delay > 0:
            time.sleep(delay)
        ids[i] = srv.submit(j["rowptr"], j["col"], x0_of(j), j["epochs"], B, ns, lr,
                            precision=job_precision(j, precision))
        ready.release()
    th.join()
    clk = clk_rec.stop() if clk_rec else None
    st = srv.stats()
    srv.close()
    lat = np.array([r[1]["end_s"] - (start + j["arrival"] * time_scale) for r, j in zip(results, jobs)])
    queue_wait = np.array([r[1]["start_s"] - r[1]["submit_s"] for r in results])
    service = np.array([r[1]["end_s"] - r[1]["start_s"] for r in results])
    upd = sum(r[1]["edge_updates"] for r in results)
    makespan = max(r[1]["end_s"] for r in results) - start
    span = jobs[-1]["arrival"] * time_scale
    return {"jobs": len(jobs), "rate_jobs_per_s": len(jobs) / span if span > 0 else None,
            "offered_edge_updates_per_s": upd / span if span > 0 else None,
            "edge_updates_per_s": upd / makespan, "makespan_s": makespan, "edge_updates": int(upd),
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max()), "queue_wait_p50": float(np.percentile(queue_wait, 50)),
                          "queue_wait_p99": float(np.percentile(queue_wait, 99)),
                          "service_p50": float(np.percentile(service, 50)),
                          "service_p99": float(np.percentile(service, 99))},
            "precision": {p: sum(job_precision(j, precision) == p for j in jobs) for p in ("bf16", "fp32")},
            "slots": slots, "server": st, "clocks": clk, "final_loss": [r[0] for r in results]}


def served_pair(jobs, x0_of, slots, precision, local):
    """The stream at the configuration's rate and at half of the capacity that
    rate measured (so that latency is service, not queueing)."""
    full = served_leg(jobs, x0_of, slots, precision, 1.0, local, clocks=True)
    scale = max(1.0, full["offered_edge_updates_per_s"] / (0.5 * full["edge_updates_per_s"]))
    half = served_leg(jobs, x0_of, slots, precision, scale, local)
    return full, half


def served_oracle_gaps(jobs, x0_of, final_loss, count=3):
    """FP64 oracle on the `count` smallest kNN jobs (kNN training converges; small
    R-MAT jobs are chaotic, FP32 and FP64 trajectories part within tens of epochs)."""
    import oracle
    B, ns, lr = W5["batch"], W5["ns"], W5["lr"]
    small = sorted((i for i in range(len(jobs)) if jobs[i]["kind"] == "knn"), key=lambda i: jobs[i]["n"])[:count]
    out = []
    for i in small:
        j = jobs[i]
        _, lo = oracle.run(j["rowptr"], j["col"], x0_of(j).astype(np.float64), j["epochs"], B, ns, lr, quirks=True,
                           threads=os.cpu_count() or 1)
        out.append({"job": i, "n": j["n"], "dim": j["dim"], "gap": float(abs(final_loss[i] - lo[-1]) / lo[-1])})
    return out


def run_served_form(args):
    """Served form: the arrival stream through de_server at the configuration's
    rate and at half the measured capacity, against the FP32 plain form running
    the same jobs one after another."""
    import torch

    import distembed_gb300 as de
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    jobs = served_workload(args.jobs, "cuda")
    gen_s = time.perf_counter() - t0
    B, ns, lr = W5["batch"], W5["ns"], W5["lr"]
    x0_of = ServedStart(jobs)
    full, half = served_pair(jobs, x0_of, args.slots, args.served_precision, 0)

    # the same jobs through the FP32 plain form, one after another (no overlap)
    plain_s, plain_upd = 0.0, 0
    if not args.no_plain_compare:
        for j in jobs:
            with de.Handle(j["rowptr"], j["col"], j["dim"], quirks=True) as h:
                h.set_embeddings(x0_of(j))
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                h.run(j["epochs"], B, ns, lr, want_loss=True)
                plain_s += time.perf_counter() - t1
                plain_upd += h.edge_updates(j["epochs"], B, ns)
    gaps = [] if args.no_gap else served_oracle_gaps(jobs, x0_of, full["final_loss"])
    for leg in (full, half):
        leg.pop("final_loss")
    value = full["edge_updates_per_s"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 4,
            "ms_per_step": 1e3 * full["makespan_s"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.served_precision,
            "data": f"synthetic: {len(jobs)} jobs, Poisson arrivals {W5['rate']:.0f}/s (seed 4), n log-uniform "
                    "[1000, 2e6], R-MAT ef 8 or kNN k=10 (kNN up to 1e5 vertices), dim in {32, 64, 128}, "
                    "10-50 epochs; minibatch 16384, 5 negatives, lr 0.02",
            "config": {"workload": f"served{len(jobs)}_poisson200", "jobs": len(jobs), "slots": args.slots,
                       "step": "the whole arrival stream", "kinds": {k: sum(jj['kind'] == k for jj in jobs)
                                                                     for k in ("knn", "rmat")},
                       "vertices": int(sum(jj["n"] for jj in jobs)), "nnz": int(sum(len(jj["col"]) for jj in jobs)),
                       "generate_s": round(gen_s, 1)},
            "served_at_config_rate": full, "served_at_half_capacity": half,
            "compare": {"fp32_plain_serial": {"edge_updates_per_s": plain_upd / plain_s if plain_s else None,
                                              "busy_s": plain_s},
                        "served_over_plain": value / (plain_upd / plain_s) if plain_s else None},
            "loss": {"final_gap_vs_fp64_oracle_smallest_knn_jobs": gaps,
                     "served_vs_alone": "bitwise equal (tests/test_gpu_served.py)"},
            "e2e": {"value": value, "unit": UNIT,
                    "h2d_bytes_per_step": int(sum(jj["n"] * jj["dim"] * 4 + len(jj["col"]) * 8 for jj in jobs)),
                    "d2h_bytes_per_step": int(sum(jj["n"] * jj["dim"] * 4 for jj in jobs)),
                    "note": "jobs submitted from host memory and results returned to host memory by the server"},
            "gpu_launches": None, "clocks": full["clocks"]}
    print(json.dumps(line), flush=True)


def run_spmm_form(args):
    """The SpMM step (SpMMAlgo::algo_spmm at one rank) on the plain workload's graph:
    y = lr * A x, one step = the whole matrix, minibatch by minibatch."""
    import torch

    import distembed_gb300 as de
    import oracle
    torch.cuda.set_device(0)
    n, rowptr, col, x0 = workload()
    dim, B, lr = W["dim"], W["batch"], W["lr"]
    x0 = x0.astype(np.float32).astype(np.float64)
    h = de.Handle(rowptr, col, dim, quirks=True)
    stream = torch.cuda.ExternalStream(h.stream, device=0)
    h.set_embeddings(x0)
    y_dev = torch.empty((n, dim), dtype=torch.float32, device="cuda")
    nnz_eff = len(col) - int(np.sum(col == n - 1))
    for _ in range(args.warmup):
        h.spmm(B, lr, out=y_dev)
    clocks = Clocks(0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev[0].record(stream)
    for k in range(args.steps):
        h.spmm(B, lr, out=y_dev)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    step_s = statistics.mean(ms) / 1e3
    value = nnz_eff / step_s
    # per step: per CSR entry its column id and neighbour row; per row its rowptr
    # entry and the output row written (and the device copy of y into the caller's
    # buffer: a read and a write of n x dim)
    alg = nnz_eff * (4 + 4 * dim) + n * (8 + 4 * dim) + 2 * n * dim * 4
    compulsory = nnz_eff * 4 + n * 8 + n * dim * 4 + n * dim * 4 + 2 * n * dim * 4  # ids, rowptr, x once, y, copy
    peak, peak_kind = measured_peak()
    # end to end: host FP64 x in, the SpMM, host FP64 y out
    e2e = None
    if args.e2e_steps > 0:
        x_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
        x_host[:] = x0
        y_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
        ts = []
        for k in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            h.set_embeddings(x_host)
            h.spmm(B, lr, out=y_host)
            if k > 0:
                ts.append(time.perf_counter() - t1)
        e2e = {"value": nnz_eff / statistics.mean(ts), "unit": UNIT, "h2d_bytes_per_step": n * dim * 8,
               "d2h_bytes_per_step": n * dim * 8, "ms_per_step": 1e3 * statistics.mean(ts),
               "step": "host FP64 x in (pinned), the SpMM, host FP64 y out"}
        gap = float(np.linalg.norm(y_host - oracle.spmm(rowptr, col, x0, lr)) / np.linalg.norm(y_host))
    h.close()
    cpu = None
    if not args.no_cpu_baseline:
        t1 = time.perf_counter()
        oracle.spmm(rowptr, col, x0, lr)
        cs = time.perf_counter() - t1
        cpu = {"value": nnz_eff / cs, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"the whole matrix once, FP64, {nnz_eff} CSR entries in {cs:.2f} s"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: R-MAT scale 20 (ef 16, a.57 b.19 c.19, seed 1), U[-0.5,0.5] init (seed 0)",
            "config": {"workload": "rmat20_ef16_d128_b4096_spmm", "n": n, "nnz": int(len(col)), "dim": dim,
                       "batch": B, "lr": lr, "step": "y = lr A x over every minibatch (SpMMAlgo::algo_spmm)",
                       "unit_note": "edge-updates here: CSR entries accumulated (edges into n-1 skipped)",
                       "l2": "inputs larger than L2 (512 MiB x); no flush"},
            "roofline": spmm_roofline(alg, compulsory, step_s, peak, peak_kind),
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": args.steps,
            "parity": {"rel_l2_vs_fp64_oracle": gap if e2e else None}}
    print(json.dumps(line), flush=True)


def run_sparse_form(args):
    """The sparse embedding (SparseEmbedding::algo_sparse_embedding at one rank, the
    reference's one-rank branch) on the plain workload's graph: one step = one run of
    5 iterations at density 0.5 from the same FP64 rows, copied in on the device."""
    import torch

    import distembed_gb300 as de
    import oracle
    torch.cuda.set_device(0)
    n, rowptr, col, x0 = workload()
    dim, B, lr, ns = W["dim"], W["batch"], W["lr"], W["ns"]
    iters, density = 5, 0.5
    keep = int(dim * density)
    x0 = x0.astype(np.float32).astype(np.float64)
    nnz = int(len(col))
    h = de.Handle(rowptr, col, dim, quirks=True)
    stream = torch.cuda.ExternalStream(h.stream, device=0)
    x_dev = torch.from_numpy(x0).to("cuda")
    torch.cuda.synchronize()

    def step():
        h.sparse_set(x_dev)
        h.sparse_run(iters, B, ns, lr, density)

    for _ in range(args.warmup):
        step()
    clocks = Clocks(0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev[0].record(stream)
    for k in range(args.steps):
        step()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    step_s = statistics.mean(ms) / 1e3
    value = nnz * iters / step_s
    # Algorithmic bytes of a step.  Per iteration the attractive pass reads every
    # CSR entry's column id and FP32 neighbour row, each row's own row and work
    # item, and writes its FP32 update; the collector pass reads the updates and
    # reads and writes the FP64 collector.  Once per step: the FP64 rows read in
    # once and written with their FP32 mirror; after the first iteration
    # the present entries are counted (read FP64) and the pruning reads FP64 and
    # writes the dim - k dropped entries in FP64 and FP32 (the rows do not change
    # after it, so the later checks cannot prune); the final pass reads FP64 and
    # writes the absent entries.
    row32, row64 = 4 * dim, 8 * dim
    per_iter = nnz * (4 + row32) + n * (row32 + 32 + row32) + n * row32 + 2 * B * row64
    once = 2 * n * row64 + n * row32 + n * row64 + n * row64 + n * (dim - keep) * 12 \
        + n * row64 + n * (dim - keep) * 8
    alg = iters * per_iter + once
    peak, peak_kind = measured_peak()
    # end to end: host FP64 rows in, the run, host FP64 rows and collector out
    e2e = None
    if args.e2e_steps > 0:
        x_host = torch.empty((n, dim), dtype=torch.float64, pin_memory=True).numpy()
        c_host = torch.empty((B, dim), dtype=torch.float64, pin_memory=True).numpy()
        ts = []
        for k in range(args.e2e_steps + 1):
            x_host[:] = x0
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            h.sparse_embedding(x_host, iters, B, ns, lr, density, inplace=True, coll=c_host)
            if k > 0:
                ts.append(time.perf_counter() - t1)
        e2e = {"value": nnz * iters / statistics.mean(ts), "unit": UNIT, "h2d_bytes_per_step": n * row64,
               "d2h_bytes_per_step": n * row64 + B * row64, "ms_per_step": 1e3 * statistics.mean(ts),
               "step": "host FP64 rows in, 5 iterations, host FP64 rows and batch collector out"}
    # parity and the CPU baseline: 2 iterations (one pruning) on the GPU and in the
    # FP64 oracle (OpenMP over the host cores)
    parity, cpu = None, None
    if not args.no_cpu_baseline:
        gx, gc = h.sparse_embedding(x0, 2, B, ns, lr, density)
        t1 = time.perf_counter()
        ox, oc = oracle.sparse_embedding(rowptr, col, x0, 2, B, ns, lr, density)
        cs = time.perf_counter() - t1
        cpu = {"value": nnz * 2 / cs, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"2 iterations of the same run, FP64, {nnz} CSR entries each, in {cs:.2f} s"}
        parity = {"rows_bitwise_equal_fp64_oracle": bool(np.array_equal(gx, ox)),
                  "collector_rel_l2_vs_fp64_oracle": float(np.linalg.norm(gc - oc) / np.linalg.norm(oc))}
    h.close()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 arithmetic on f64 rows",
            "data": "synthetic: R-MAT scale 20 (ef 16, a.57 b.19 c.19, seed 1), U[-0.5,0.5] init (seed 0)",
            "config": {"workload": "rmat20_ef16_d128_b4096_sparse_embedding", "n": n, "nnz": nnz, "dim": dim,
                       "batch": B, "lr": lr, "iterations_per_step": iters, "density": density,
                       "step": "SparseEmbedding::algo_sparse_embedding, one-rank branch: rows copied in on the "
                               "device, 5 iterations (attractive pass into the batch collector, top-k pruning "
                               "after the first), absent entries cleared",
                       "unit_note": "edge-updates here: attractive pair terms (CSR entries x iterations)",
                       "l2": "inputs larger than L2 (1 GiB FP64 rows, 512 MiB mirror); no flush"},
            "roofline": sparse_roofline(alg, step_s, peak, peak_kind),
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": args.steps * (1 + 2 * iters + 2 + 1),
            "parity": parity}
    print(json.dumps(line), flush=True)



def run_reference(args):
    """The reference's CPU algorithm (the FP64 port, -O3, every host core) on the
    default line's workload: one step = one epoch of every graph (epoch k mod 20
    of the job, state carried from step to step), one graph per thread.  The
    graphs are generated as in the GPU arm (torch on the GPU when one is
    present, so that both arms train the same graphs); nothing of this package
    runs in the timed region."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.form == "plain":
        return run_reference_plain(args)
    import oracle
    try:
        import torch
        device = "cuda" if torch.cuda.is_available() else "cpu"
    except ImportError:
        device = None
    graphs, x0 = batched_workload(args.graphs, device)
    xs = [np.ascontiguousarray(x, dtype=np.float64) for x in x0]
    csr = [(rp, c) for _, _, rp, c in graphs]
    threads = os.cpu_count() or 1
    E = W4["epochs"]

    def step(k):
        u, _ = oracle.run_many(csr, xs, 1, W4["batch"], W4["ns"], W4["lr"], first_epoch=k % E, want_loss=False,
                               threads=threads, fast=True)
        return u

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    updates = sum(step(args.warmup + k) for k in range(args.steps))
    dt = time.perf_counter() - t0
    v = updates / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": BATCHED_DATA.format(g=len(graphs)), "config": batched_config(graphs),
            "impl_detail": {"step": "one epoch of every graph (epoch k mod 20 of the job)",
                            "parallelism": "1 process x all host cores, one graph per thread",
                            "graphs_generated_on": device},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "build": "g++ -O3 -ffp-contract=fast -fopenmp (oracle/liboracle_fast.so)",
                             "sample": f"{args.steps} epochs of all {len(graphs)} graphs, FP64, {updates} edge-updates"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_plain(args):
    """The FP64 port on the plain form's workload (R-MAT scale 20): one step =
    one minibatch of epoch 0, OpenMP over its rows as the reference."""
    import oracle
    n, rowptr, col, x0 = workload()
    batches = (n + W["batch"] - 1) // W["batch"]
    x = np.array(x0, dtype=np.float64, copy=True)
    threads = os.cpu_count() or 1

    def step(k):
        j = (37 * k) % batches
        return oracle.run_batches(rowptr, col, x, 0, W["batch"], W["ns"], W["lr"], [j], quirks=True, threads=threads,
                                  fast=True)

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    updates = sum(step(args.warmup + k) for k in range(args.steps))
    dt = time.perf_counter() - t0
    v = updates / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: R-MAT scale 20 (ef 16, a.57 b.19 c.19, seed 1), U[-0.5,0.5] init (seed 0)",
            "config": {"workload": WORKLOAD, "n": n, "nnz": int(len(col)), "dim": W["dim"], "batch": W["batch"],
                       "ns": W["ns"], "lr": W["lr"], "epochs_per_job": W["epochs"],
                       "step": "one minibatch of epoch 0 (j = 37k mod 256)",
                       "parallelism": "1 process x all host cores (OpenMP)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "build": "g++ -O3 -ffp-contract=fast -fopenmp (oracle/liboracle_fast.so)",
                             "sample": f"{args.steps} minibatches, FP64, {updates} edge-updates"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_headline(args):
    """The default line: the metric's comparison on the batched workload, the
    other forms beside it (on rank 0 of a one-GPU run)."""
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("gloo")
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    graphs, x0 = batched_workload(args.graphs, f"cuda:{local}")
    gen_s = time.perf_counter() - t0
    x0_all = np.concatenate(x0)
    kinds = [k for k, _, _, _ in graphs]
    shape = parse_shape(args.shape) if args.shape else None
    if world > 1:
        torch.distributed.barrier()
    bf = batched_leg(graphs, x0_all, "bf16", local, args.steps, args.warmup, args.e2e_steps, shape=shape,
                     clocks=True)
    total_s = max_over_ranks(sum(bf["step_ms"]) / 1e3, world)
    value = whole_job_rate(bf["edge_updates"] * args.steps, total_s, world)
    e2e = bf["e2e"]
    if e2e is not None and world > 1:
        e2e_s = max_over_ranks(e2e["ms_per_step"] / 1e3, world)
        e2e = dict(e2e, value=bf["edge_updates"] * world / e2e_s, ms_per_step=1e3 * e2e_s)
    extras = rank == 0 and world == 1
    compare, loss, cpu, served = {}, None, None, None
    if extras:
        f32 = batched_leg(graphs, x0_all, "fp32", local, max(1, args.steps // 4), 1, shape=bf["shape"])
        compare["fp32_storage_batched"] = {"edge_updates_per_s": f32["value"],
                                           "ms_per_step": statistics.mean(f32["step_ms"]), "shape": f32["shape"],
                                           "note": "the same 512 graphs in the same persistent launch, FP32 storage"}
        if not args.no_plain_compare:
            compare["fp32_plain_same_graphs"] = plain_same_graphs(graphs, x0, local)
        plain = plain_leg(args, rank, world, local, with_cpu=not args.no_cpu_baseline, with_gap=not args.no_gap)
        for k in ("metric", "unit", "higher_is_better", "scaling", "vs_baseline", "n_gpus"):
            plain.pop(k, None)
        compare["fp32_plain_rmat20"] = plain
        compare["bf16_batched_over_fp32_plain_same_graphs"] = (
            value / compare["fp32_plain_same_graphs"]["edge_updates_per_s"]
            if "fp32_plain_same_graphs" in compare else None)
        compare["bf16_batched_over_fp32_plain_rmat20"] = value / plain["value"]
        compare["bf16_batched_over_fp32_storage_batched"] = value / f32["value"]
        if not args.no_gap:
            lo = fp64_oracle_losses(graphs, x0)
            loss = {"bf16_vs_fp64_oracle": gap_stats(bf["loss"], lo, kinds),
                    "fp32_storage_vs_fp64_oracle": gap_stats(f32["loss"], lo, kinds),
                    "oracle": "oracle/liboracle.so (bit-exact with the reference's own code), every graph's "
                              "20-epoch job, loss of every epoch"}
        if not args.no_cpu_baseline:
            cpu = batched_cpu_baseline(graphs, x0, args.cpu_seconds)
        if not args.no_served:
            jobs = served_workload(args.jobs, f"cuda:{local}")
            x0_of = ServedStart(jobs)
            full, half = served_pair(jobs, x0_of, args.slots, args.served_precision, local)
            other = "fp32" if args.served_precision == "bf16" else "bf16"
            full_other = served_leg(jobs, x0_of, args.slots, other, 1.0, local)
            gaps = [] if args.no_gap else served_oracle_gaps(jobs, x0_of, full["final_loss"])
            for leg in (full, half, full_other):
                leg.pop("final_loss")
                leg.pop("clocks", None)
            served = {"workload": f"served{len(jobs)}_poisson200: Poisson arrivals 200 jobs/s (seed 4), n "
                                  "log-uniform [1000, 2e6], R-MAT ef 8 or kNN k=10 (kNN up to 1e5 vertices), dim in "
                                  "{32, 64, 128}, 10-50 epochs, minibatch 16384, 5 negatives, lr 0.02",
                      "storage": f"{args.served_precision} (BF16 only for jobs of dim 64-256; dim 32 jobs FP32)",
                      "at_config_rate": full, "at_half_capacity": half,
                      f"at_config_rate_{other}": full_other,
                      "final_gap_vs_fp64_oracle_smallest_knn_jobs": gaps,
                      "served_vs_alone": "bitwise equal (tests/test_gpu_served.py)"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": BATCHED_DATA.format(g=len(graphs)),
                "config": batched_config(graphs),
                "impl_detail": {"storage": "BF16 rows read, FP32 master, FP32 arithmetic, FP64 loss sums",
                                "team_shape": bf["shape"], "autotune_s": round(bf["tune_s"], 2),
                                "autotune_shapes": len(bf["tuned"]),
                                "autotune_top3_ms": [[sh, round(t, 2)] for sh, t in
                                                     sorted(bf["tuned"], key=lambda x: x[1])[:3]],
                                "trace": bf["trace"], "generate_s": round(gen_s, 1),
                                "step": "one launch: every graph, 20 epochs (CUDA graph)",
                                "reset": "embeddings reset to the start values before every step (untimed)",
                                "l2": "inputs larger than L2 (embeddings of every graph); no flush",
                                "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": roofline_batched(graphs, bf["step_ms"]),
                "loss": loss, "compare": compare or None, "served": served,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps, "clocks": bf["clocks"]}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.form == "plain":
        run_plain_form(args)
    elif args.form == "knn20k":
        run_knn20k_form(args)
    elif args.form == "bf16":
        run_bf16_form(args)
    elif args.form == "batched":
        run_batched_form(args)
    elif args.form == "served":
        run_served_form(args)
    elif args.form == "spmm":
        run_spmm_form(args)
    elif args.form == "sparse":
        run_sparse_form(args)
    else:
        run_headline(args)


if __name__ == "__main__":
    main()
