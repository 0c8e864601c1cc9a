"""Run one B-ADMM centroid update on a seeded synthetic workload.

    python -m d2_kmeans_gb300.run_workload --workload batched --scale 0.1 --iters 3

Workloads (d2_kmeans_gb300.synth.workload): plain, batched, hist,
twophase_euclid, embed, ngram.  --scale shrinks the number of instances only;
--iters sets maxIters (the loop runs maxIters+1 iterations); --precision 1
selects the FP64 form; --cost-gemm 1 computes the word-embedding cost table
on FP32 CUDA cores instead of the tensor cores.  Prints the run statistics
as one JSON line.

    python -m d2_kmeans_gb300.run_workload --workload serve --requests 64

runs that many serving requests (k=256 centroids, m=64, d=64, m_q
log-uniform 4..512, 200 iterations) back to back through the server.

    python -m d2_kmeans_gb300.run_workload --workload labeling --scale 0.0025 --repeat 3

runs the assignment step (d2g_labeling: exact transport of every instance
against every centroid) on the batched workload (or --of embed for the
word-embedding one) at that scale, --repeat times, and prints the time and
problems/s of each call.
"""
from __future__ import annotations

import argparse
import json

from . import badmm, synth


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="batched")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--iters", type=int, default=None)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--cost-gemm", type=int, default=0)
    ap.add_argument("--batch-entries", type=int, default=0,
                    help="serving: plan entries per device batch (0 = library default)")
    ap.add_argument("--of", default="batched", help="labeling: the workload whose instances are labeled")
    args = ap.parse_args(argv)
    badmm.set_config(verbose=0, cost_gemm=args.cost_gemm)
    if args.workload == "labeling":
        import time

        from . import assign
        from .assign import Mph, Work
        ph, c, _ = synth.workload(args.of, seed=args.seed, scale=args.scale)
        n, k, m, d = len(ph["p_str"]), int(ph["num_of_labels"]), int(ph["str"]), int(ph.get("dim", 0))
        fields = {key: ph[key] for key in ("p_str", "p_w", "p_supp", "p_supp_sym", "vocab_vec",
                                           "dist_mat", "vocab_size") if ph.get(key) is not None}
        metric = badmm._metric(ph["metric"])
        data = Mph([dict(fields, metric=metric, dim=d, str=m)], n, label=ph["label"], num_of_labels=k)
        cmetric = metric % 7
        cents = Mph([dict(metric=cmetric, dim=d, str=m, p_w=c["c_w"], p_supp=c.get("c_supp"),
                          dist_mat=ph.get("dist_mat"), vocab_size=ph.get("vocab_size", 0))], k,
                    num_of_labels=k)
        for _ in range(args.repeat):
            data.label[:] = ph["label"]
            t = time.perf_counter()
            changed, cost = assign.labeling(data, cents, Work(n, k, 1))
            dt = time.perf_counter() - t
            print(json.dumps({"workload": args.of, "n": n, "k": k, "pairs": n * k, "seconds": dt,
                              "problems_per_s": n * k / dt, "labels_changed": changed}))
        return
    if args.workload == "serve":
        import time

        from . import serve
        c_w, c_supp, means = synth.serving_centroids(k=256, m=64, dim=64, n_comp=32, seed=args.seed)
        S = serve.Server(c_w, c_supp, iters=args.iters or 200, max_batch_entries=args.batch_entries)
        qs = synth.serving_queries(args.requests, means, sizes=(4, 512), seed=args.seed + 1)
        t = time.perf_counter()
        out = serve.poisson_run(S, qs, rate=1e9, seed=0)
        out.pop("results")
        out["seconds"] = time.perf_counter() - t
        S.close()
        print(json.dumps(out))
        return
    ph, c, opts = synth.workload(args.workload, seed=args.seed, scale=args.scale)
    if args.iters is not None:
        opts = dict(opts, maxIters=args.iters)
    P = badmm.Phase(ph, args.precision)
    for _ in range(args.repeat):
        r = P.run(c, opts)
    st = P.stats()
    P.close()
    st["n"] = len(ph["p_str"])
    st["obj_last"] = float(r["trace"][-1, 1]) if len(r["trace"]) else None
    print(json.dumps(st))


if __name__ == "__main__":
    main()
