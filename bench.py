#!/usr/bin/env python
"""Benchmark of the network-likelihood hot path on GB300.

Workload (one "step"): one log-likelihood + gradient evaluation - forward
sweep over every displayed-tree variant, per-(tree, partition) site sums,
AVERAGE mixture, adjoint sweep, gradient reduction - of the 100 taxa /
8 reticulations / 100k DNA sites network (GTR+G4, seeded synthetic data, the
configuration the differentiation target is quoted on), FP32 CLVs with
per-site power-of-two scaling. Branch lengths change every step (a new
optimizer iterate), so P-matrices are recomputed every step too.

value: whole-job evals/s with inputs resident in HBM (device-resident branch
lengths, CUDA events on the library's stream, max over ranks).
e2e: the same through the C ABI with host buffers (host branch lengths in,
logL + gradient out), wall clock.
Multi-GPU: every rank evaluates its own replica (independent optimizer
iterates) - weak scaling, no collective on the data path.

``--impl reference`` times the oracle's FP64 CPU restatement of the path
(``oracle/``: the reference's schedule and pruning arithmetic plus an adjoint
sweep for the gradient, all host cores) on the full workload, logL + gradient
per step, with the same --steps / --warmup.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "logL+grad evals/s & site-CLV updates/s, FP32 vs FP64 GPU at ≤1e-6 rel ΔlogL"
UNIT = "logL+grad evals/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="netlk", choices=["netlk", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--variant", default="AVERAGE", choices=["AVERAGE", "BEST"])
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-checkpoint-arm", action="store_true",
                    help="skip timing the same workload with 4 CLV checkpoint segments")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0, help="site-count scale (1.0 = full workload)")
    ap.add_argument("--checkpoint-segments", type=int, default=0,
                    help="CLV checkpointing: 0 automatic (every CLV stored while they fit), 1 store every CLV, "
                         "k >= 2: k level segments, the adjoint recomputes each segment's non-permanent CLVs")
    ap.add_argument("--op", default="eval", choices=["eval", "edge"],
                    help="eval: logL + gradient evaluations (the headline); edge: the branch-length "
                         "optimizer's per-edge calls (incremental edge logL, edge derivatives)")
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3, 4],
                    help="1: 50 taxa / 4 reticulations / 10 uneven DNA partitions (75.5k sites); "
                         "2: 100 taxa / 8 reticulations / 100k DNA sites (the headline workload); "
                         "3: 40 taxa / 3 reticulations / 50k protein sites; "
                         "4: a batch of 64 candidate networks scored in one CUDA graph")
    return ap.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes per site-CLV update of each sweep (DNA: 4 states) from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum of the 100-taxon /
# 8-reticulation network at 0.3 of its sites, scaled by updates; writes still dirty in L2 at a launch's end are not
# counted). Keyed by sweep, schedule (level: one launch per DAG level; walk:
# one warp walks the whole DAG), precision and states. The level figures were
# captured before the adjoint dropped read messages from L2, so they are an
# upper bound for the current level adjoint.
TRAFFIC_PER_UPDATE = {"forward_level_fp32_4": 102.3, "backward_level_fp32_4": 295.9,
                      "forward_walk_fp32_4": 85.8, "backward_walk_fp32_4": 213.3}


def cpu_rate(w, steps, warmup, variant, seed=123):
    """The oracle's FP64 CPU sweeps on the FULL workload, one thread per host
    core: per step, new branch lengths, the forward pruning of every
    displayed-tree variant (the reference's schedule and libpll arithmetic,
    threads as the reference's MPI ranks over pattern slices), the mixture, and
    an adjoint sweep for d logL / d every branch length and reticulation
    probability. Returns (evals/s, info)."""
    from oracle import improved, newick, pllmath, sweep
    net = newick.parse_newick(w.newick)
    parts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch, pllmath.gamma_rates_mean(p.alpha, 4))
             for p in w.partitions]
    orc = improved.ImprovedOracle(net, parts, variant=variant)
    orc.loglikelihood()  # the reference's displayed-tree enumeration (host-side, untimed)
    so = sweep.SweepOracle(orc)
    rng = np.random.default_rng(seed)
    base = np.array(orc.brlen, np.float64)

    def lengths():
        return np.clip(base * np.exp(0.05 * rng.standard_normal(base.size)), 1e-6, 100.0)

    for _ in range(warmup):  # the first step also faults in the CLV and adjoint buffers
        so.evaluate(lengths())
    times = []
    for _ in range(steps):
        b = lengths()
        t = time.perf_counter()
        so.evaluate(b)
        times.append(time.perf_counter() - t)
    evals = steps / sum(times)
    patterns = sum(p.n for p in parts)
    info = {"value": evals, "unit": UNIT, "cores": sweep.threads(), "kind": "port",
            "sample": "full workload: all %d patterns, logL + gradient per step (forward pruning of all %d "
                      "variants with per-site scaling, mixture, adjoint sweep), FP64, %d timed steps after "
                      "%d warm-up, new branch lengths every step" % (patterns, so.n_var, steps, warmup),
            "ms_per_step": 1000.0 / evals,
            "site_clv_updates_per_s": so.site_updates * evals,
            "median_ms": statistics.median(times) * 1000.0}
    return evals, info


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from netrax_gb300 import synth
    w = synth.config(args.config, scale=args.scale)
    steps, warmup = args.steps, max(1, args.warmup)
    evals, info = cpu_rate(w, steps, warmup, args.variant)
    line = {"impl": "reference", "metric": METRIC, "value": evals, "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 / evals,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": w.name, "patterns": w.n_patterns, "variant": args.variant,
                       "l2": "no flush: every step streams tens of GB of CLVs, far above the CPU caches"},
            "cpu_baseline": info,
            "e2e": {"value": evals, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_netlk(args, ws, rank, local):
    import torch
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = synth.config(args.config, scale=args.scale)
    lik = NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision=args.precision,
                            device=local, checkpoint_segments=args.checkpoint_segments)
    st = lik.stats
    E = lik.n_edges
    K, W = args.steps, max(3, args.warmup)
    rng = np.random.default_rng(1000 + rank)
    base = w.network.branch_lengths
    host_bl = np.clip(base[None, :] * np.exp(0.05 * rng.standard_normal((K + W, E))), 1e-6, 100.0)
    dev_bl = torch.from_numpy(host_bl).to(dev)
    stream = torch.cuda.ExternalStream(lik.stream(), device=dev)

    # ---------------------------------------------------- device-timed loop
    for k in range(W):
        lik.set_branch_lengths_device(dev_bl[k].data_ptr())
        lik.enqueue(True)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(ws)
    torch.cuda.synchronize()
    l0 = lik.launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(K):
        lik.set_branch_lengths_device(dev_bl[W + k].data_ptr())
        lik.enqueue(True)
    t1.record(stream)
    t1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    clocks = sampler.stop()
    launches = lik.launch_count() - l0
    ms_local = t0.elapsed_time(t1) / K
    ms = allreduce_max(ms_local, ws, dev)
    value = ws * 1000.0 / ms

    # ------------------------------------------- end to end through the C ABI
    K2 = max(3, min(K, 100))
    lik.set_branch_lengths(host_bl[0])
    lik.loglikelihood_gradient()
    barrier(ws)
    t = time.perf_counter()
    for k in range(K2):
        lik.set_branch_lengths(host_bl[W + k % K])
        lik.loglikelihood_gradient()
    e2e_s = allreduce_max((time.perf_counter() - t) / K2, ws, dev)
    h2d = E * 8
    d2h = (2 + lik.n_parts + lik.n_ret) * 8 + E * 8

    # --------------------------------------------- per-kernel event timings
    lik.set_profiling(True)
    for k in range(min(K, 20)):
        lik.set_branch_lengths_device(dev_bl[W + k].data_ptr())
        lik.enqueue(True)
    kt = lik.kernel_times()
    lik.set_profiling(False)
    kavg = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in kt.items()}

    # ----------------------------------------------- accuracy vs FP64 plain
    lik.set_branch_lengths(base)
    l32, g32, r32 = lik.loglikelihood_gradient()
    fp64 = None
    if not args.no_fp64 and args.precision == "fp32":
        lik64 = NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision="fp64",
                                  device=local)
        l64, g64, r64 = lik64.loglikelihood_gradient()
        s64 = torch.cuda.ExternalStream(lik64.stream(), device=dev)
        for k in range(3):
            lik64.set_branch_lengths_device(dev_bl[k].data_ptr())
            lik64.enqueue(True)
        torch.cuda.synchronize()
        Kf = max(3, args.fp64_steps)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s64)
        for k in range(Kf):
            lik64.set_branch_lengths_device(dev_bl[W + k % K].data_ptr())
            lik64.enqueue(True)
        b.record(s64)
        b.synchronize()
        ms64 = a.elapsed_time(b) / Kf
        lik64.set_profiling(True)
        lik64.set_branch_lengths_device(dev_bl[W].data_ptr())
        lik64.enqueue(True)
        kt64 = lik64.kernel_times()
        lik64.close()
        gscale = max(1.0, float(np.abs(g64).max()))
        fp64 = {"evals_per_s": 1000.0 / ms64, "ms_per_step": ms64,
                "speedup_fp32_over_fp64": ms64 / ms_local,
                "rel_dlogl": abs(l32 - l64) / abs(l64),
                "max_rel_grad_err": float(np.abs(g32 - g64).max() / gscale),
                "max_abs_retprob_grad_err": float(np.abs(r32 - r64).max()) if len(r64) else 0.0,
                "kernel_ms": {k: (v[0] / v[1] if v[1] else 0.0) for k, v in kt64.items()}}

    # ----------------------------------- the same workload with 4 CLV checkpoints
    ckpt = None
    if not args.no_checkpoint_arm and args.precision == "fp32" and args.checkpoint_segments == 0:
        likc = NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision="fp32",
                                 device=local, checkpoint_segments=4)
        lc, gc, rc = likc.loglikelihood_gradient()
        sc = torch.cuda.ExternalStream(likc.stream(), device=dev)
        for k in range(3):
            likc.set_branch_lengths_device(dev_bl[k].data_ptr())
            likc.enqueue(True)
        torch.cuda.synchronize()
        Kc = max(3, args.fp64_steps)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(sc)
        for k in range(Kc):
            likc.set_branch_lengths_device(dev_bl[W + k % K].data_ptr())
            likc.enqueue(True)
        b.record(sc)
        b.synchronize()
        msc = a.elapsed_time(b) / Kc
        stc = likc.stats
        likc.close()
        ckpt = {"checkpoint_segments": stc["checkpoint_segments"], "evals_per_s": 1000.0 / msc,
                "ms_per_step": msc, "clv_buffers": stc["clv_slots"], "dag_variants": stc["n_variants"],
                "recompute_site_updates_per_eval": stc["recompute_site_updates"],
                "logl_and_gradient_bit_identical_to_unsegmented": bool(lc == l32 and np.array_equal(gc, g32)
                                                                       and np.array_equal(rc, r32))}

    # ------------------------------------------------------------- roofline
    peak, peak_kind = measured_peak()
    st = lik.stats  # after tuning: launch counts of the chosen shapes
    # the adjoint's time includes the checkpoint recomputes, so its bytes do too
    fwd_b, bwd_b = st["forward_bytes"], st["backward_bytes"] + st["recompute_bytes"]
    dom = "backward" if kavg["backward"] >= kavg["forward"] else "forward"
    dom_bytes = bwd_b if dom == "backward" else fwd_b
    achieved = dom_bytes / (kavg[dom] * 1e-3) / 1e9 if kavg[dom] > 0 else 0.0
    tuning = lik.tuning()
    sched = "walk" if tuning.get(dom + "_walk") else "level"
    traffic = None
    tt = TRAFFIC_PER_UPDATE.get("%s_%s_%s_%d" % (dom, sched, args.precision, lik.states))
    if tt and st["checkpoint_segments"] == 1:  # captured without checkpointing
        traffic = tt * st["site_clv_updates"]
    if lik.states == 20:  # FP32 with 4 rates runs the tensor-core (tcgen05) sweeps
        kname = dom + ("20_tc_kernel" if args.precision == "fp32" and lik.rate_cats == 4 else "20_kernel")
    else:
        kname = dom + ("_walk" if sched == "walk" else "") + "_kernel"
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": dom_bytes,
                "algorithmic_bytes_per_site_update": dom_bytes / st["site_clv_updates"],
                "forward": {"ms": kavg["forward"], "bytes": fwd_b,
                            "GBps": fwd_b / (kavg["forward"] * 1e-3) / 1e9 if kavg["forward"] else 0.0},
                "backward": {"ms": kavg["backward"], "bytes": bwd_b,
                             "GBps": bwd_b / (kavg["backward"] * 1e-3) / 1e9 if kavg["backward"] else 0.0}}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        _, cpu = cpu_rate(w, 3, 1, args.variant)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": w.name, "taxa": w.network.n_tips, "reticulations": w.network.n_reticulations,
                       "sites": w.n_sites, "patterns": w.n_patterns, "partitions": len(w.partitions),
                       "substitution_model": "GTR+G4" if lik.states == 4 else "20-state GTR (LG-like)+G4",
                       "variant": args.variant, "precision": args.precision,
                       "displayed_trees": lik.n_roots, "dag_variants": st["n_variants"],
                       "site_clv_updates_per_eval": st["site_clv_updates"],
                       "checkpoint_segments": st["checkpoint_segments"], "clv_buffers": st["clv_slots"],
                       "recompute_site_updates_per_eval": st["recompute_site_updates"],
                       "device_bytes": st["device_bytes"],
                       "l2": "no flush: every eval streams %.1f GB of CLVs, far above the 129 MB L2"
                             % ((fwd_b + bwd_b) / 1e9),
                       "parallelism": "replica per GPU" if ws > 1 else "1 GPU", "seed": w.seed},
            "site_clv_updates_per_s": value * st["site_clv_updates"],
            "gpu_launches": int(launches),
            "kernel_ms": kavg,
            "autotune": tuning,
            "e2e": {"value": ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_s * 1000.0},
            "roofline": roofline,
            "fp64_plain": fp64,
            "checkpointed": ckpt,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "logl": l32,
        }
        print(json.dumps(line), flush=True)
    lik.close()


def run_batch(args, ws, rank, local):
    """64 candidate networks (taxa U{30..120}, reticulations U{0..6}, 1-8
    DNA partitions of U{1k..30k} sites) scored per call as one CUDA graph of
    persistent launches (warps take (candidate, pattern unit) items; walk
    shapes timed on the batch); every call uploads new host branch lengths
    and downloads every candidate's logL and gradient. Reports candidates/s,
    the p50 / p99 latency of a batch call (when every candidate's result is
    ready), the p50 / p99 latency of one candidate scored alone, and the same
    batch as a graph of per-context launch sequences and one by one."""
    from netrax_gb300 import synth
    n_workers = max(1, min(16, os.cpu_count() or 1))
    cands = synth.candidate_batch(64, scale=args.scale, workers=n_workers)  # spawned pool, before GPU use
    import torch
    from netrax_gb300.likelihood import NetworkBatch, NetworkLikelihood
    torch.cuda.set_device(local)
    liks = [NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision=args.precision,
                              device=local) for w in cands]
    updates = sum(lk.stats["site_clv_updates"] for lk in liks)
    K, W = args.steps, max(3, args.warmup)
    rng = np.random.default_rng(2000 + rank)
    lens = [[np.clip(w.network.branch_lengths * np.exp(0.05 * rng.standard_normal(w.network.n_edges)), 1e-6, 100.0)
             for w in cands] for _ in range(K + W)]
    batch = NetworkBatch(liks)
    per_ctx = NetworkBatch(liks, per_context=True)

    def set_lengths(k):
        for lk, b in zip(liks, lens[k]):
            lk.set_branch_lengths(b)

    for k in range(W):
        set_lengths(k)
        batch.loglikelihood_gradient()
        per_ctx.loglikelihood_gradient()
    info = batch.info()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(ws)
    lat = []
    for k in range(K):
        set_lengths(W + k)
        t = time.perf_counter()
        tot, gb, gr = batch.loglikelihood_gradient()
        lat.append(time.perf_counter() - t)
    clocks = sampler.stop()
    graph = []
    for k in range(min(K, 10)):
        set_lengths(W + k)
        t = time.perf_counter()
        per_ctx.loglikelihood_gradient()
        graph.append(time.perf_counter() - t)
    seq = []
    for k in range(min(K, 5)):
        set_lengths(W + k)
        t = time.perf_counter()
        for lk in liks:
            lk.loglikelihood_gradient()
        seq.append(time.perf_counter() - t)
    alone = []  # one candidate scored by itself, host in and out
    for lk in liks:
        lk.loglikelihood_gradient()
        t = time.perf_counter()
        lk.loglikelihood_gradient()
        alone.append(time.perf_counter() - t)
    lat_ms = np.array(lat) * 1e3
    alone_ms = np.array(alone) * 1e3
    total_s = allreduce_max(float(np.sum(lat)), ws, torch.device("cuda", local))
    value = ws * 64 * K / total_s
    h2d = sum(lk.n_edges * 8 for lk in liks)
    d2h = sum((3 + lk.n_parts + lk.n_ret) * 8 + lk.n_edges * 8 for lk in liks)
    if rank == 0:
        line = {
            "metric": "candidate logL+grad evals/s (64-candidate batch, persistent launches in one CUDA graph)",
            "value": value, "unit": "candidate evals/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": float(np.mean(lat_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": "64 candidate networks: taxa U{30..120}, reticulations U{0..6}, "
                                   "1-8 DNA partitions of U{1k..30k} sites, GTR+G4",
                       "sites": sum(w.n_sites for w in cands), "patterns": sum(w.n_patterns for w in cands),
                       "site_clv_updates_per_batch": updates, "variant": args.variant,
                       "precision": args.precision,
                       "l2": "no flush: every batch streams the CLVs of 64 networks, far above the 129 MB L2",
                       "parallelism": "replica per GPU" if ws > 1 else "1 GPU"},
            "batch_latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                                 "min": float(lat_ms.min()), "max": float(lat_ms.max())},
            "candidate_alone_latency_ms": {"p50": float(np.percentile(alone_ms, 50)),
                                           "p99": float(np.percentile(alone_ms, 99))},
            "persistent": info,
            "per_context_graph_ms_per_batch": float(np.median(graph) * 1e3),
            "speedup_over_per_context_graph": float(np.median(graph) / np.median(lat)),
            "sequential_ms_per_batch": float(np.median(seq) * 1e3),
            "batch_speedup_over_sequential": float(np.median(seq) / np.median(lat)),
            "site_clv_updates_per_s": value / 64 * updates,
            "gpu_launches": int(info["launches_per_call"]) * K,
            "e2e": {"value": value, "unit": "candidate evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "clocks": clocks,
            "device_bytes": int(sum(lk.stats["device_bytes"] for lk in liks)),
        }
        print(json.dumps(line), flush=True)
    batch.close()
    per_ctx.close()
    for lk in liks:
        lk.close()


def run_edge(args, ws, rank, local):
    """The branch-length optimizer's per-edge calls on one context, host
    synchronous like its Newton-Raphson loop (BranchLengthOptimization.cpp:
    171-200, VirtualRerooting.cpp:348-585): a full logL after every length
    changed, netlk_edge_loglikelihood (only the variants above the edge are
    recomputed), netlk_edge_derivatives (analytic d1 and d2; timed on a new
    edge each call, so each call builds that edge's sumtables), and the
    sumtable route of the
    Newton-Raphson loop: netlk_edge_sumtable (the per-tree outside vectors at
    the edge, once per edge) and netlk_edge_sumtable_derivatives (logL, d1, d2
    at a proposed length: one pass over the tables) - against one iteration
    of the tangent route (netlk_edge_loglikelihood at the proposal, then
    netlk_edge_derivatives)."""
    import torch
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    torch.cuda.set_device(local)
    w = synth.config(args.config, scale=args.scale)
    lik = NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision=args.precision,
                            device=local)
    E = lik.n_edges
    base = np.array(w.network.branch_lengths, np.float64)
    rng = np.random.default_rng(2000 + rank)
    lik.loglikelihood_gradient()  # launch-shape autotuning and a full sweep
    K, W = args.steps, max(3, args.warmup)

    def full_once(k):
        lik.set_branch_lengths(np.clip(base * np.exp(0.05 * rng.standard_normal(E)), 1e-6, 100.0))
        return lik.loglikelihood()

    for k in range(W):
        full_once(k)
    t = time.perf_counter()
    nf = max(3, K // 10)
    for k in range(nf):
        full_once(k)
    full_s = (time.perf_counter() - t) / nf
    full_updates = lik.last_site_updates()

    edges = [(k * 37) % E for k in range(K + W)]
    for k in range(W):
        lik.edge_loglikelihood(edges[k], base[edges[k]] * 1.01)
    t = time.perf_counter()
    upd = 0
    for k in range(K):
        e = edges[W + k]
        lik.edge_loglikelihood(e, base[e] * (1.0 + 0.02 * ((k % 5) - 2)))
        upd += lik.last_site_updates()
    edge_s = (time.perf_counter() - t) / K

    nd = max(3, K // 10)
    lik.edge_derivatives(edges[0])
    t = time.perf_counter()
    for k in range(nd):
        lik.edge_derivatives(edges[k])
    der_s = (time.perf_counter() - t) / nd

    # sumtables: build once per edge, then evaluations at proposed lengths
    sedges = [edges[k] for k in range(nd)]
    lik.edge_sumtable(sedges[0])
    t = time.perf_counter()
    built = [lik.edge_sumtable(e) for e in sedges]
    build_s = (time.perf_counter() - t) / nd
    n_tab = built[-1][1]
    table_bytes = (n_tab * lik.stats["n_patterns_total"] * lik.rate_cats * lik.states
                   * (4 if args.precision == "fp32" else 8))
    n_eval = 0
    t = time.perf_counter()
    for e in sedges[-1:]:
        for j in range(max(10, K)):
            lik.edge_sumtable_derivatives(e, base[e] * (0.5 + 0.05 * (j % 20)))
            n_eval += 1
    eval_s = (time.perf_counter() - t) / n_eval
    # one Newton-Raphson iteration the reference's way on an edge whose
    # tables are current: set the proposal (incremental logL), then d1, d2
    e = sedges[-1]
    t = time.perf_counter()
    for j in range(max(10, K)):
        lik.edge_loglikelihood(e, base[e] * (0.5 + 0.05 * (j % 20)))
        lik.edge_derivatives(e)
    nr_iter_s = (time.perf_counter() - t) / max(10, K)
    lik.edge_loglikelihood(e, base[e])
    lik.close()
    # the tangent sweep: a context without sumtables takes it on every call
    likt = NetworkLikelihood(w.network, w.partitions, variant=args.variant, precision=args.precision,
                             device=local, sumtables=False)
    likt.loglikelihood_gradient()
    likt.edge_derivatives(sedges[0])
    t = time.perf_counter()
    for k in range(nd):
        likt.edge_derivatives(sedges[k])
    tangent_s = (time.perf_counter() - t) / nd
    likt.close()
    if rank == 0:
        line = {
            "metric": "edge logL evals/s (incremental) & edge derivative evals/s",
            "value": 1.0 / edge_s, "unit": "edge logL evals/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": edge_s * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": w.name, "taxa": w.network.n_tips, "reticulations": w.network.n_reticulations,
                       "sites": w.n_sites, "patterns": w.n_patterns, "edges": E, "variant": args.variant,
                       "precision": args.precision, "timing": "host wall clock around synchronous calls"},
            "edge_logl_ms": edge_s * 1000.0,
            "mean_site_updates_per_edge_eval": upd / K,
            "full_logl_ms": full_s * 1000.0, "full_site_updates": full_updates,
            "edge_derivatives_ms": der_s * 1000.0, "edge_derivatives_per_s": 1.0 / der_s,
            "edge_derivatives_note": "a new edge each call (its sumtables built on the way)",
            "sumtable": {"applies": all(b for b, _ in built), "build_ms": build_s * 1000.0,
                         "eval_ms": eval_s * 1000.0, "tables_of_evaluated_edge": n_tab,
                         "table_bytes_of_evaluated_edge": table_bytes,
                         "eval_table_GBps_wall": table_bytes / eval_s / 1e9,
                         "set_and_derive_iteration_ms": nr_iter_s * 1000.0,
                         "tangent_sweep_ms": tangent_s * 1000.0,
                         "note": "eval: logL, d1, d2 at a proposed length from the tables; set-and-derive: "
                                 "netlk_edge_loglikelihood at the proposal + netlk_edge_derivatives (tables "
                                 "current); tangent sweep: netlk_edge_derivatives on a context created with sumtables = 0"},
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.op == "edge":
        run_edge(args, ws, rank, local)
    elif args.config == 4:
        run_batch(args, ws, rank, local)
    else:
        run_netlk(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
