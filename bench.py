#!/usr/bin/env python
"""Benchmark of the B-ADMM centroid update on GB300.

One step = one full centroid update (maxIters=200, i.e. 201 B-ADMM
iterations) over the batched uneven-size Euclidean workload: n=200000 D2
instances in d=3, support sizes log-uniform 8..128 from a 64-component
Gaussian mixture, Dirichlet(0.5) weights, k=64 centroids with m=32 supports,
rhoCoeff=2, updatePerLoops=10.  Seeded synthetic data (no dataset download).

Prints one JSON line:
  value      plan-updates/s of the batched FP32 form, inputs resident in HBM,
             CUDA events on the library's stream around K steps
  e2e        the same metric through the reference-facing C entry point
             d2_centroid_sphBregman with host buffers (inputs from pinned host
             memory, results back to the caller's arrays) inside the timing
  plain_gpu  the plain FP64 one-kernel-per-step GPU form on the same inputs
  roofline   the plan-update pass against the measured HBM copy bandwidth (a pass
             runs two B-ADMM iterations where that is exact, plan_pair.cuh)
  cpu_baseline  the C restatement of the reference (oracle port) on the host
  workloads  the word-embedding, 256-bin histogram and two-phase Euclidean
             workloads: plan-updates/s and the plan kernel against the HBM peak
  tuning     the launch shape the autotuner picked for the headline phase
  io         d2 text input: d2g_read MB/s against the reference's fscanf reader
  assign     the assignment step (d2_labeling, exact transport on the GPU):
             transport problems/s, the pruned labeling, a sample checked
             against the oracle's exact solver, which is also timed

--impl reference times the reference algorithm's CPU implementation (the
oracle port; the reference tree itself is not on the GPU host) with every
host core: all 200 000 instances of the same inputs, one process per core on
its shard, 21 of the 201 iterations per step.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "B-ADMM plan-updates/sec (batched vs plain GPU) at obj err ≤1e-5; serve p50/p99"
UNIT = "plan-updates/s"
WORKLOAD = ("batched uneven sizes: n=200000 Euclidean D2 instances, d=3, m_i log-uniform 8-128, "
            "64-component GMM supports, Dirichlet(0.5) weights; k=64 centroids, m=32; "
            "rhoCoeff=2, updatePerLoops=10, maxIters=200 (201 iterations)")
HBM_FALLBACK_GBS = 6800.0
SKIP = set()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU legs
def _cpu_shard(args):
    """One process: the oracle port on a shard of the workload."""
    scale, seed, shard, nshard, iters = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np  # noqa: F401
    import oracle
    from d2_kmeans_gb300 import synth
    ph, c, opts = synth.workload("batched", seed=seed + shard, scale=scale)
    opts = dict(opts, maxIters=iters - 1)
    t = time.perf_counter()
    r = oracle.badmm(ph, c, opts, "port", want=())
    el = time.perf_counter() - t
    assert r["rc"] == 0, r["rc"]
    return len(ph["p_str"]) * r["iters"], el


def cpu_baseline(procs: int, scale: float, iters: int, seed: int = 100):
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_shard, [(scale, seed, s, procs, iters) for s in range(procs)])
    units = sum(u for u, _ in res)
    wall = max(t for _, t in res)
    return units / wall, units, wall


_SHARD = {}


def _shard_init(path, lo, hi):
    """Worker set-up (untimed): this process's instances [lo, hi) of the
    workload written by the parent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    z = np.load(path)
    p_str = z["p_str"]
    cum = np.concatenate([[0], np.cumsum(p_str, dtype=np.int64)])
    a, b = int(cum[lo]), int(cum[hi])
    ph = dict(metric=0, dim=3, str=int(z["str"]), p_str=p_str[lo:hi].copy(), p_w=z["p_w"][a:b].copy(),
              p_supp=z["p_supp"][3 * a:3 * b].copy(), label=z["label"][lo:hi].copy(),
              num_of_labels=int(z["k"]), label_switch=np.ones(hi - lo, np.int8))
    _SHARD.update(ph=ph, c=dict(c_w=z["c_w"], c_supp=z["c_supp"]))


def _shard_step(args):
    import oracle
    shard, iters = args
    opts = dict(maxIters=iters - 1, rhoCoeff=2.0, updatePerLoops=10)
    t = time.perf_counter()
    r = oracle.badmm(_SHARD["ph"], _SHARD["c"], opts, "port", want=())
    el = time.perf_counter() - t
    assert r["rc"] == 0, r["rc"]
    return len(_SHARD["ph"]["p_str"]) * r["iters"], el


def ensure_oracle():
    import oracle
    if not oracle.available("port"):
        oracle.build(reference=False)


REF_ITERS = 21


def run_reference(args, rank):
    """The reference's algorithm on the host cores: the oracle port (the C
    restatement, bit-identical to the reference's FP64 update) over all
    200 000 instances of the headline workload (seed 0, the GPU arm's inputs),
    cut into one shard per core; each shard runs its own update for 21
    iterations (the reference's MPI build would allreduce the cluster sums
    across shards; that exchange is not timed here)."""
    if rank != 0:
        return
    import numpy as np
    from d2_kmeans_gb300 import synth
    ensure_oracle()
    procs = os.cpu_count() or 1
    ph, c, _ = synth.workload("batched", seed=0)
    n = len(ph["p_str"])
    bounds = [(n * s // procs, n * (s + 1) // procs) for s in range(procs)]
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "workload.npz")
        np.savez(path, p_str=ph["p_str"], p_w=ph["p_w"], p_supp=ph["p_supp"], label=ph["label"],
                 c_w=c["c_w"], c_supp=c["c_supp"], str=ph["str"], k=ph["num_of_labels"])
        ctx = mp.get_context("spawn")
        pools = [ctx.Pool(1, initializer=_shard_init, initargs=(path, lo, hi)) for lo, hi in bounds]
        try:
            vals = []
            for i in range(args.warmup + args.steps):
                jobs = [pl.apply_async(_shard_step, ((s, REF_ITERS),)) for s, pl in enumerate(pools)]
                res = [j.get() for j in jobs]
                units = sum(u for u, _ in res)
                wall = max(t for _, t in res)
                if i >= args.warmup:
                    vals.append((units / wall, wall))
        finally:
            for pl in pools:
                pl.close()
                pl.join()
    value = statistics.mean(v for v, _ in vals)
    ms = 1e3 * statistics.mean(w for _, w in vals)
    sample = (f"per step, all {n} instances of the workload (seed 0, the GPU arm's inputs) in {procs} "
              f"shards of about {n // procs}, one process per host core, each running the oracle port "
              f"(the reference's FP64 update restated bit for bit) for {REF_ITERS} of the 201 "
              f"iterations; no cross-shard reduction")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD, "sample": sample},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ GPU legs
def replica_throughput(local_ms: float, units_per_rank: float, device: str = "cuda"):
    """Whole-job throughput of N independent replicas (one process per GPU, no
    collective on the data path): every rank processes units_per_rank units in
    local_ms; the job takes as long as its slowest rank (MAX over ranks).
    Returns (units per second over all ranks, the job's ms)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return world * units_per_rank / (ms / 1e3), ms


def time_steps(P, c, opts, steps):
    import torch
    st = torch.cuda.ExternalStream(P.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(steps):
        r = P.run(c, opts)
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, r


def e2e_steps(ph, c, opts, steps, warmup):
    """Through d2_centroid_sphBregman with host buffers: pinned inputs,
    results into the caller's arrays (c->p_w, c->p_supp, work Z)."""
    import numpy as np
    import torch
    from d2_kmeans_gb300 import badmm

    def pinned(a):
        if a is None:
            return None
        t = torch.empty(a.size, dtype=getattr(torch, str(a.dtype)) if a.dtype != np.int8 else torch.int8,
                        pin_memory=True)
        v = t.numpy()
        v[:] = a.reshape(-1)
        return v
    php = {k: (pinned(v) if isinstance(v, np.ndarray) else v) for k, v in ph.items()}
    d = badmm.DropIn(php, c)
    h2d = sum(php[k].nbytes for k in ("p_str", "p_w", "p_supp", "label", "label_switch")) + \
        d.c_w.nbytes + d.c_supp.nbytes
    d2h = d.c_w.nbytes + d.c_supp.nbytes + 8 * d.m * d.col
    times = []
    for i in range(warmup + steps):
        d.c_w[:] = c["c_w"]
        d.c_supp[:] = c["c_supp"]
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = d.call(opts)
        el = time.perf_counter() - t
        assert rc == 0, rc
        if i >= warmup:
            times.append(el)
    d.close()
    e2e_steps.step_ms = [round(1e3 * t, 2) for t in times]
    return statistics.mean(times), h2d, d2h


OTHER_WORKLOADS = {
    "embed": "word embeddings: vocabulary 20000 x d=300, n=20000 documents of 20-400 Zipf(1.1) tokens, "
             "k=20, m=64, 101 iterations (tensor-core 3xTF32 cost table)",
    "hist": "two-phase set, phase 1: n=100000 dense 256-bin (16x16) histograms, Dirichlet(0.1), "
            "squared grid-distance costs, k=32, m=256, 101 iterations",
    "twophase_euclid": "two-phase set, phase 2: n=100000 Euclidean D2, d=3, m_i 4-32, k=32, m=16, "
                       "101 iterations",
    "ngram": "n-gram phase: n=20000 sequences (log-uniform lengths 30-400 over 20 symbols) as "
             "distributions of their distinct 3-grams, k=64, m=32, 101 iterations, symbol update "
             "every 10",
}


# the FP64 check of the 256-bin histogram phase runs on a 5 000-instance subset
# (its FP64 form moves 136 B per plan entry per iteration: 890 GB at full size)
ERROR_CHECK_SCALE = {"embed": 1.0, "hist": 0.05, "twophase_euclid": 1.0, "ngram": 1.0}


def fp64_errors(name, seed=0):
    """Objective trace and centroid errors of the batched form against the FP64
    form on the same inputs and iterations (both on the GPU)."""
    import numpy as np
    from d2_kmeans_gb300 import badmm, synth
    ph, c, opts = synth.workload(name, seed=seed, scale=ERROR_CHECK_SCALE[name])
    k, m = int(ph["num_of_labels"]), int(ph["str"])
    out = []
    for precision in (0, 1):
        P = badmm.Phase(ph, precision)
        out.append(P.run(c, opts))
        P.close()
    b, f = out
    res = {"n": len(ph["p_str"]),
           "obj_rel_err": float(np.max(np.abs(b["trace"][:, 1] - f["trace"][:, 1]) / np.abs(f["trace"][:, 1]))),
           "c_w_l1": float(np.abs(b["c_w"].reshape(k, m) - f["c_w"].reshape(k, m)).sum(1).max())}
    if b.get("c_sym") is not None:
        res["c_sym_mismatches"] = int(np.sum(b["c_sym"] != f["c_sym"]))
    if b.get("c_supp") is not None:
        s0 = np.asarray(b["c_supp"]).reshape(k * m, -1)
        s1 = np.asarray(f["c_supp"]).reshape(k * m, -1)
        nrm = np.linalg.norm(s1, axis=1)
        res["supp_rel_err"] = float((np.linalg.norm(s0 - s1, axis=1) / np.maximum(nrm, 1e-3 * nrm.max())).max())
    return res


# bounded CPU samples of the secondary workloads (oracle port, 1 core):
# instances kept, iterations run
CPU_SAMPLE = {"embed": (100, 20), "hist": (100, 20), "twophase_euclid": (5000, 20), "ngram": (1000, 20)}


def workload_cpu(name):
    """The oracle port (the reference's algorithm in FP64, bit-identical to
    it) on the first instances of the workload, timed on one host core."""
    import oracle
    from d2_kmeans_gb300 import synth
    ensure_oracle()
    keep, iters = CPU_SAMPLE[name]
    full = {"embed": 20000, "hist": 100000, "twophase_euclid": 100000, "ngram": 20000}[name]
    ph, c, opts = synth.workload(name, seed=0, scale=keep / full)
    t = time.perf_counter()
    r = oracle.badmm(ph, c, dict(opts, maxIters=iters - 1), "port", want=())
    el = time.perf_counter() - t
    n = len(ph["p_str"])
    return {"value": n * r["iters"] / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} instances of the workload, {r['iters']} iterations, {el:.1f} s"}


def workload_leg(name, steps, hbm, tf32_peak):
    """One secondary workload: autotuned, timed over whole centroid updates,
    then the plan-update (and cost-table) launches timed alone (profile mode),
    and its error against the FP64 form."""
    from d2_kmeans_gb300 import badmm, synth
    ph, c, opts = synth.workload(name, seed=0)
    n = len(ph["p_str"])
    P = badmm.Phase(ph, 0)
    if name == "ngram":  # the autotuner starts an n-gram phase from its last run's symbols
        P.run(c, dict(opts, maxIters=0))
    tune = P.autotune(c, dict(opts, maxIters=20))
    P.run(c, opts)
    ms, r = time_steps(P, c, opts, steps)
    st = P.stats()
    badmm.set_config(profile=1)
    P.run(c, opts)
    ps = P.stats()
    badmm.set_config(profile=0)
    P.close()
    achieved = ps["plan_bytes"] / (ps["plan_ms_avg"] / 1e3) / 1e9
    # profile mode times every pass over the plans: one iteration, or two in a pair pass
    ipp = ps["iterations"] / max(ps["plan_launches"], 1)
    out = {"workload": OTHER_WORKLOADS[name], "value": n * st["iterations"] / (ms / 1e3), "unit": UNIT,
           "ms_per_step": ms, "iterations_per_step": st["iterations"],
           "plan_entries": int(st["plan_entries"]), "tuning": tune["best"],
           "plan_update": {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                           "algo_bytes_per_pass": ps["plan_bytes"], "ms_per_pass": ps["plan_ms_avg"],
                           "passes": ps["plan_launches"], "iterations_per_pass": ipp,
                           "plan_update_equiv_frac": achieved * ipp / hbm}}
    if ps["table_launches"]:
        useful = ps["table_flops"] / (ps["table_ms_avg"] / 1e3) / 1e12
        out["cost_table"] = {"kernel": "cost_table_tc_kernel (tcgen05 kind::tf32, 3xTF32)",
                             "ms_per_launch": ps["table_ms_avg"], "flops_per_launch": ps["table_flops"],
                             "achieved_tflops": useful, "tf32_mma_tflops_issued": 3 * useful,
                             "peak_tf32_tflops": tf32_peak, "frac_issued": 3 * useful / tf32_peak,
                             "peak_kind": "half the measured bf16 cuBLAS rate (TF32 MMA runs at half "
                                          "the BF16 rate)"}
    if "fp64" not in SKIP:
        out["error_vs_fp64"] = fp64_errors(name)
    if "cpu" not in SKIP:
        out["cpu_baseline"] = workload_cpu(name)
    return out


IO_WORKLOAD = ("d2 text file of 20 000 instances of the batched workload (d = 3, m_i log-uniform 8-128), "
               "parsed into the reference's mph")


def io_leg():
    """d2g_read (parallel, every host core) against the oracle's restatement of
    the reference's fscanf reader (one core) on the same file; the arrays must
    be identical."""
    import numpy as np
    import oracle
    from d2_kmeans_gb300 import d2io, synth
    ph, _, _ = synth.workload("batched", seed=0, scale=0.1)
    n = len(ph["p_str"])
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "batched.d2")
        d2io.write(f, [dict(metric=d2io.EUCLIDEAN, dim=3, p_str=ph["p_str"], p_w=ph["p_w"],
                            p_supp=ph["p_supp"])])
        mb = os.path.getsize(f) / 1e6
        d2io.read(f, n, [3], [0], avg_strides=[43])  # page cache warm
        t = time.perf_counter()
        ours = d2io.read(f, n, [3], [0], avg_strides=[43])
        t_ours = time.perf_counter() - t
        ensure_oracle()
        t = time.perf_counter()
        rc, port = oracle.read("port", f, n, [3], [0], avg_strides=[43])
        t_port = time.perf_counter() - t
    same = rc == 0 and all(np.array_equal(ours["phases"][0][k], port["phases"][0][k])
                           for k in ("p_str", "p_str_cum", "p_w", "p_supp"))
    return {"workload": IO_WORKLOAD, "file_mb": mb, "value": mb / t_ours, "unit": "MB/s",
            "threads": os.cpu_count(), "seconds": t_ours,
            "cpu_baseline": {"value": mb / t_port, "unit": "MB/s", "cores": 1, "kind": "port",
                             "sample": "the oracle's restatement of d2_read (fscanf per token)"},
            "identical_arrays": bool(same)}


ASSIGN_WORKLOAD = ("assignment step: exact transport distances of the batched workload's n=200000 "
                   "instances (d=3, m_i 8-128) to its k=64 centroids (m=32), 12.8 M transport "
                   "problems per d2_labeling; d2_labeling_prep (Elkan) after a small centroid move")


def assign_leg():
    """d2_labeling / d2_labeling_prep / d2_labeling_post on the GPU (exact
    transport, transportation simplex) over the headline workload, its
    distances checked against the oracle's exact solver on a sample, and the
    oracle timed on that sample as the CPU baseline."""
    import numpy as np
    import oracle
    from d2_kmeans_gb300 import assign, synth
    from d2_kmeans_gb300.assign import Mph, Work
    ph, c, _ = synth.workload("batched", seed=0)
    n, k, m = len(ph["p_str"]), int(ph["num_of_labels"]), int(ph["str"])

    def data_mph(cnt):
        col = int(ph["p_str"][:cnt].sum())
        return Mph([dict(metric=0, dim=3, str=m, p_str=ph["p_str"][:cnt], p_w=ph["p_w"][:col],
                         p_supp=ph["p_supp"][:col * 3])], cnt, label=ph["label"][:cnt].copy(),
                   num_of_labels=k)

    def cent_mph(c_w, c_supp):
        return Mph([dict(metric=0, dim=3, str=m, p_w=c_w, p_supp=c_supp)], k, num_of_labels=k)

    data = data_mph(n)
    cents = cent_mph(c["c_w"], c["c_supp"])
    w = Work(n, k, 1)
    t = time.perf_counter()
    assign.labeling(data, cents, w)  # uploads the instances (kept for later calls)
    first = time.perf_counter() - t
    data.label[:] = ph["label"]
    t = time.perf_counter()
    changed, cost = assign.labeling(data, cents, w)
    t_lab = time.perf_counter() - t
    # pruned labeling, the steady state of the k-means rounds: bounds from a
    # first round, centroids moved a little, bounds updated, labeling again
    w2 = Work(n, k, 1)
    data.label[:] = ph["label"]
    assign.labeling_prep(data, cents, w2)
    rng = np.random.default_rng(7)
    cw2 = c["c_w"].reshape(k, m) * np.exp(rng.normal(size=(k, m)) * 0.02)
    cw2 = (cw2 / cw2.sum(1, keepdims=True)).reshape(-1)
    cents2 = cent_mph(cw2, c["c_supp"] + rng.normal(size=c["c_supp"].size) * 0.02)
    assign.labeling_post(data, cents, cents2, w2)
    t = time.perf_counter()
    changed2, dist2 = assign.labeling_prep(data, cents2, w2)
    t_prep = time.perf_counter() - t
    # distances of a sample against the oracle; the oracle timed on it
    sample = 200
    ds = data_mph(sample)
    ia, jb = np.meshgrid(np.arange(sample), np.arange(k), indexing="ij")
    ours = assign.compute_distances(ds, cents, ia.reshape(-1), jb.reshape(-1))
    ensure_oracle()
    lab = oracle.Labeling("port")
    t = time.perf_counter()
    ref = np.array([lab.distance(ds, i, cents, j) for i, j in zip(ia.reshape(-1), jb.reshape(-1))])
    t_cpu = time.perf_counter() - t
    rel = float(np.max(np.abs(ours - ref) / np.maximum(np.abs(ref), 1e-300)))
    # word embeddings: the embedding workload's shape at 1/10 (2 000 documents
    # of 20-400 words x 20 centroids of m = 64 in R^300)
    pe, ce, _ = synth.workload("embed", seed=0, scale=0.1)
    ne, ke, me, de, V = len(pe["p_str"]), int(pe["num_of_labels"]), int(pe["str"]), int(pe["dim"]), int(pe["vocab_size"])

    def emb_mph(cnt):
        col = int(pe["p_str"][:cnt].sum())
        return Mph([dict(metric=7, dim=de, str=me, p_str=pe["p_str"][:cnt], p_w=pe["p_w"][:col],
                         p_supp_sym=pe["p_supp_sym"][:col], vocab_vec=pe["vocab_vec"], vocab_size=V)],
                   cnt, label=pe["label"][:cnt].copy(), num_of_labels=ke)

    de_m = emb_mph(ne)
    ce_m = Mph([dict(metric=0, dim=de, str=me, p_w=ce["c_w"], p_supp=ce["c_supp"])], ke, num_of_labels=ke)
    assign.labeling(de_m, ce_m, Work(ne, ke, 1))
    de_m.label[:] = pe["label"]
    t = time.perf_counter()
    assign.labeling(de_m, ce_m, Work(ne, ke, 1))
    t_emb = time.perf_counter() - t
    es = emb_mph(5)
    ia, jb = np.meshgrid(np.arange(5), np.arange(ke), indexing="ij")
    ours_e = assign.compute_distances(es, ce_m, ia.reshape(-1), jb.reshape(-1))
    t = time.perf_counter()
    ref_e = np.array([lab.distance(es, i, ce_m, j) for i, j in zip(ia.reshape(-1), jb.reshape(-1))])
    t_cpu_e = time.perf_counter() - t
    embed = {"workload": "word embeddings: 2000 documents (20-400 Zipf(1.1) words of V=20000 x 300) x "
                         "20 centroids (m=64)",
             "value": ne * ke / t_emb, "unit": "transport problems/s", "seconds": t_emb,
             "check": {"pairs": int(ref_e.size),
                       "max_rel_err_vs_oracle": float(np.max(np.abs(ours_e - ref_e) / np.abs(ref_e)))},
             "cpu_baseline": {"value": ref_e.size / t_cpu_e, "unit": "transport problems/s", "cores": 1,
                              "kind": "port", "sample": f"5 documents x {ke} centroids, oracle exact solver"}}
    # whole k-means rounds (d2g_clustering, pruned labeling + B-ADMM update
    # with the reference's options {100, 2.0, 10}) from the workload's
    # centroids; the update's time budget held fixed
    import ctypes
    from d2_kmeans_gb300 import _lib as L
    from d2_kmeans_gb300 import badmm
    old = badmm.set_config(keep_time_budget=1)
    opt = L.BADMM_options.in_dll(L.load(), "badmm_clu_options")
    opt.maxIters, opt.rhoCoeff, opt.updatePerLoops = 100, 2.0, 10
    ctypes.c_void_p.in_dll(L.load(), "p_badmm_options").value = ctypes.addressof(opt)
    ctypes.c_double.in_dll(L.load(), "time_budget").value = 1e300
    data_r = data_mph(n)
    cents_r = cent_mph(c["c_w"].copy(), c["c_supp"].copy())
    t = time.perf_counter()
    rounds = assign.clustering(data_r, cents_r, k, 3, use_triangle=True)
    t_rounds = time.perf_counter() - t
    badmm.set_config(keep_time_budget=old["keep_time_budget"])
    return {"workload": ASSIGN_WORKLOAD, "value": n * k / t_lab, "unit": "transport problems/s",
            "clustering": {"rounds": rounds, "seconds": t_rounds,
                           "what": "d2g_clustering, use_triangle, max_iter 3: labeling + 101-iteration "
                                   "B-ADMM update per round, final plain labeling"},
            "labeling_s": t_lab, "first_call_s": first, "labels_changed": int(changed),
            "mean_cost": cost / n,
            "prep": {"seconds": t_prep, "distances": int(dist2), "labels_changed": int(changed2),
                     "problems_per_s": dist2 / t_prep},
            "check": {"pairs": int(ours.size), "max_rel_err_vs_oracle": rel},
            "embed": embed,
            "cpu_baseline": {"value": ref.size / t_cpu, "unit": "transport problems/s", "cores": 1,
                             "kind": "port",
                             "sample": f"{sample} instances x {k} centroids with the oracle's exact "
                                       "solver (successive shortest paths, FP64)"}}


SERVE_WORKLOAD = ("serving: k=256 resident centroids, m=64, d=64; queries with m_q log-uniform 4-512, "
                  "GMM supports, Dirichlet(1) weights; 200 B-ADMM iterations per solve against all "
                  "centroids + argmin; Poisson arrivals")


def serve_leg(rates=(2000.0, 5000.0, 10000.0, 20000.0), per_rate=1500):
    from d2_kmeans_gb300 import serve, synth
    c_w, c_supp, means = synth.serving_centroids(k=256, m=64, dim=64, n_comp=32, seed=0)
    S = serve.Server(c_w, c_supp, iters=200, rho_coeff=2.0, hbm_budget_bytes=4 << 30, max_queue=4096)
    warm = synth.serving_queries(64, means, sizes=(4, 512), seed=99)
    serve.poisson_run(S, warm, rate=1e6, seed=0)
    out = []
    for i, rate in enumerate(rates):
        qs = synth.serving_queries(per_rate, means, sizes=(4, 512), seed=100 + i)
        r = serve.poisson_run(S, qs, rate=rate, seed=i)
        r.pop("results")
        out.append(r)
    S.close()
    res = {"workload": SERVE_WORKLOAD, "per_rate": out,
           "capacity_req_per_s": max(r["throughput"] for r in out)}
    if "cpu" not in SKIP:
        # the oracle's fixed-centroid solve (FP64, 1 core) of two queries for
        # 20 iterations, scaled to the 200 iterations of a request (its time
        # is linear in the iterations)
        import oracle
        ensure_oracle()
        qs = synth.serving_queries(2, means, sizes=(4, 512), seed=7)
        t = time.perf_counter()
        for w, sp in qs:
            oracle.serve_query(c_w, c_supp, w, sp, iters=20)
        per_req = (time.perf_counter() - t) / len(qs) * 10
        res["cpu_baseline"] = {"value": 1.0 / per_req, "unit": "requests/s", "cores": 1, "kind": "port",
                               "sample": f"2 queries (m_q {qs[0][0].size}, {qs[1][0].size}) x 20 "
                                         f"iterations, scaled to 200: {per_req:.2f} s per request"}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip", default="",
                    help="comma list of legs to skip: e2e,plain,cpu,profile,serve,workloads,fp64,io,"
                         "assign")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:  # one process per GPU: each rank sees its own GPU as device 0
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        return run_reference(args, rank)
    skip = set(x for x in args.skip.split(",") if x)
    SKIP.update(skip)

    import numpy as np
    import torch
    import torch.distributed as dist
    from d2_kmeans_gb300 import badmm, synth
    from d2_kmeans_gb300.build import build as build_lib

    if not os.path.exists(os.path.join(ROOT, "d2_kmeans_gb300", "libd2g.so")):
        build_lib()
    torch.cuda.set_device(0)
    if world > 1:
        dist.init_process_group("nccl")
    badmm.set_config(verbose=0, precision=0, use_graph=1, profile=0)

    ph, c, opts = synth.workload("batched", seed=0)
    n = len(ph["p_str"])
    P = badmm.Phase(ph, 0)
    tuning = P.autotune(c, dict(opts, maxIters=20))
    for _ in range(args.warmup):
        P.run(c, opts)
    gpu = int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)
    if world > 1:
        dist.barrier()
    with ClockSampler(gpu if world > 1 else 0) as clk:
        ms, r = time_steps(P, c, opts, args.steps)
    clocks = clk.summary()
    stats = P.stats()
    iters = stats["iterations"]
    value, ms = replica_throughput(ms, n * iters)

    # end to end through the reference-facing entry point, right after the
    # device-timed steps (same inputs, same options, same step count)
    e2e = None
    if "e2e" not in skip:
        sec, h2d, d2h = e2e_steps(ph, c, opts, args.steps, max(1, args.warmup))
        e2e_value, e2e_ms = replica_throughput(sec * 1e3, n * iters)
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_ms / 1e3,
               "step_ms": e2e_steps.step_ms,
               "note": "mean of the steps; a host copy of a step occasionally stalls for tens of ms "
                       "on this host (the device time of the update does not change)",
               "api": "d2_centroid_sphBregman (reference structs, host buffers)"}

    hbm, peak_kind = peaks()
    roof = None
    if "profile" not in skip:
        badmm.set_config(profile=1)
        P.run(c, opts)
        ps = P.stats()
        badmm.set_config(profile=0)
        achieved = ps["plan_bytes"] / (ps["plan_ms_avg"] / 1e3) / 1e9
        traffic = None
        tp = os.path.join(ROOT, "profiles", "plan_kernel_traffic.json")
        if os.path.exists(tp):
            with open(tp) as f:
                traffic = json.load(f).get("traffic_bytes_per_launch")
        passes = ps["plan_launches"]  # passes over the plans (profile mode times each one)
        paired = passes < stats["iterations"]
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                "kernel": ("plan_pair_kernel<32, EUCLID3> (two B-ADMM iterations per pass over the plans)"
                           if paired else "plan_kernel_tma<32, EUCLID3>"),
                "passes_per_step": passes, "iterations_per_pass": stats["iterations"] / passes,
                "note": ("a pair pass reads and writes Z and Y once for two iterations (8 B per plan "
                         "entry per iteration); its bound moves from HBM toward issue and latency"
                         if paired else "one iteration per pass: 16 B per plan entry per iteration"),
                "algo_bytes_per_launch": ps["plan_bytes"], "ms_per_launch": ps["plan_ms_avg"]}
        # the same launch against 16 B per plan entry per iteration (Z and Y read
        # and written once per iteration, the one-iteration-per-pass formulation)
        ipp = stats["iterations"] / passes
        ubytes = 16.0 * stats["plan_entries"] * ipp
        roof["plan_update_bytes_per_launch"] = ubytes
        roof["plan_update_equiv_gbs"] = ubytes / (ps["plan_ms_avg"] / 1e3) / 1e9
        roof["plan_update_equiv_frac"] = roof["plan_update_equiv_gbs"] / hbm
    trace_b = r["trace"]
    cw_b = r["c_w"].copy()
    P.close()

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 plans, f64 cross-plan reductions",
           "data": "synthetic (seeded GMM / Dirichlet; no dataset)",
           "config": {"workload": WORKLOAD, "iterations_per_step": iters,
                      "parallelism": "replicas" if world > 1 else "1 GPU",
                      "l2": "inputs larger than L2: Z and Y are 1.1 GB each",
                      "plan_entries": int(stats["plan_entries"])},
           "clocks": clocks, "gpu_launches": int(stats["kernel_launches"]) * args.steps,
           "roofline": roof, "tuning": tuning}

    if "plain" not in skip and rank == 0:
        Q = badmm.Phase(ph, 1)
        Q.run(c, opts)  # warm-up: graph capture
        ms_p, rp = time_steps(Q, c, opts, 3)
        Q.close()
        obj_err = float(np.max(np.abs(trace_b[:, 1] - rp["trace"][:, 1]) / np.abs(rp["trace"][:, 1])))
        cw_l1 = float(np.abs(cw_b.reshape(64, 32) - rp["c_w"].reshape(64, 32)).sum(1).max())
        vp = n * iters / (ms_p / 1e3)
        out["plain_gpu"] = {"value": vp, "unit": UNIT, "ms_per_step": ms_p, "steps": 3,
                            "form": "FP64, one kernel per reference step, C/X/Z0 in HBM",
                            "batched_over_plain": value / world / vp,
                            "obj_rel_err_batched_vs_fp64": obj_err, "c_w_l1_vs_fp64": cw_l1}
    if e2e is not None:
        out["e2e"] = e2e
    if "serve" not in skip and rank == 0:
        out["serve"] = serve_leg()
    if "io" not in skip and rank == 0:
        out["io"] = io_leg()
    if "assign" not in skip and rank == 0:
        out["assign"] = assign_leg()
    if "workloads" not in skip and rank == 0:
        tf32 = bf16_peak() / 2
        out["workloads"] = {w: workload_leg(w, 2, hbm, tf32) for w in OTHER_WORKLOADS}
    if "cpu" not in skip and rank == 0:
        ensure_oracle()
        v, units, wall = cpu_baseline(1, 20000 / 200000, 21, seed=100)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"oracle port (C restatement of the reference, FP64, 1 core) "
                                         f"on 20000 instances of the workload for 21 iterations: "
                                         f"{units} plan-updates in {wall:.1f} s"}
    if world > 1:
        dist.barrier()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
