"""Generate the golden fixtures of the B-ADMM centroid update.

Runs the reference's own d2_centroid_sphBregman (compiled unmodified from the
reference tree by oracle/Makefile into oracle/_ref/) on small seeded inputs
and stores inputs and outputs as .npz files next to this script.  The
reference publishes no golden vectors and has no unit tests, so these
fixtures are the pin: tests check the C restatement (oracle/liboracle.so,
which also builds on the GPU machine) and the CUDA paths against them.

Run from the repository root where the reference tree is present:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from d2_kmeans_gb300 import synth  # noqa: E402

REF_DATA = os.path.join(oracle.REF_TREE, "data")


def digest(z: np.ndarray) -> np.ndarray:
    """Order-sensitive summary of a plan array: sums, moments, samples."""
    idx = np.arange(0, z.size, max(1, z.size // 64))
    w = np.cos(np.arange(z.size) * 0.001)
    return np.concatenate([[z.sum(), (z * z).sum(), (z * w).sum()], z[idx]])


def read_simple():
    """The reference's 5 three-bin histograms (data/simple.d2, .hist0)."""
    toks = open(os.path.join(REF_DATA, "simple.d2")).read().split()
    vals = list(map(float, toks))
    w = []
    i = 0
    while i < len(vals):
        n = int(vals[i + 1])
        w.extend(vals[i + 2:i + 2 + n])
        i += 2 + n
    h = list(map(float, open(os.path.join(REF_DATA, "simple.d2.hist0")).read().split()))
    nb = int(h[0])
    return np.array(w).reshape(-1, nb), np.array(h[1:1 + nb * nb]).reshape(nb, nb)


def read_protein_1gram(limit):
    """The first `limit` sequences of the reference's protein 1-gram file
    (data/protein_seq/protein_1gram.dat) with its PAM250 symbol cost
    (PAM250_distmat.dat), parsed as data/protein_seq/d2_protein_ngram.cc:71-150
    reads them: letters keyed in the cost file's order, weights re-normalised.
    Sequences holding a gap support ("--") are skipped: the reference's reader
    drops the last weight slot for a gap and leaves the gap's symbol slot
    unwritten, so those sequences have no well-defined input."""
    base = os.path.join(REF_DATA, "protein_seq")
    with open(os.path.join(base, "PAM250_distmat.dat")) as f:
        head = f.readline()
        keys = [ch for ch in head if "A" <= ch <= "Z"]
        D = np.array(f.read().split()[: len(keys) ** 2], dtype=np.float64)
    key = {ch: i for i, ch in enumerate(keys)}
    toks = open(os.path.join(base, "protein_1gram.dat")).read().split()
    pos = 6  # "Seq # N Class # C"
    p_str, w, sym = [], [], []
    while len(p_str) < limit:
        pos += 2  # name, class
        dim, n = int(toks[pos]), int(toks[pos + 1])
        pos += 2
        ww = np.array(toks[pos:pos + n], dtype=np.float64)
        pos += n
        grams = toks[pos:pos + n]
        pos += n
        if any("-" in g for g in grams):
            continue
        assert dim == 1 and all(len(g) == 1 and g in key for g in grams)
        p_str.append(n)
        w.extend(ww / ww.sum())
        sym.extend(key[g] for g in grams)
    return (np.array(p_str, np.int32), np.array(w), np.array(sym, np.int32),
            D.reshape(len(keys), len(keys)))


def read_mountain():
    """Phase 0 of the reference's data/mountaindat.d2 (2000 objects, d = 3,
    11 011 support points) read by the reference's own d2_read, labels i % 10,
    and initial centroids (k = 10, m = 6) from the reference's own
    d2_centroid_rands (src/d2/centroid_rand.c:161-295; srand(0) order), both
    compiled into oracle/_ref: the centroid update of the reference's
    mountaindat example, whose objective trace over 100 iterations runs
    949.94 / 800.13 / 751.01 / 737.56 / 731.14 at iterations 20 ... 100."""
    import ctypes as C
    from d2_kmeans_gb300 import _lib as L
    from d2_kmeans_gb300.assign import Mph
    rc, arr = oracle.read("ref", os.path.join(REF_DATA, "mountaindat.d2"), 2000, [3, 3], [0, 0],
                          avg_strides=[6, 11])
    assert rc == 0 and arr["size"] == 2000
    p0 = arr["phases"][0]
    n, k, m, d = arr["size"], 10, 6, 3
    label = (np.arange(n) % k).astype(np.int32)
    ph = dict(metric=0, dim=d, str=m, p_str=p0["p_str"].astype(np.int32), p_w=p0["p_w"],
              p_supp=p0["p_supp"], label=label, num_of_labels=k, label_switch=np.ones(n, np.int8))
    data = Mph([ph], n, label=label, num_of_labels=k)
    w, supp = np.full(k * m, np.nan), np.full(k * m * d, np.nan)
    p_str, cum = np.zeros(k, np.int32), np.zeros(k, np.uint64)
    c = L.sph()
    c.dim, c.str, c.max_str, c.metric_type = d, m, m, 0
    c.p_str = p_str.ctypes.data_as(C.POINTER(C.c_int))
    c.p_str_cum = cum.ctypes.data_as(C.POINTER(C.c_size_t))
    c.p_w = w.ctypes.data_as(C.POINTER(C.c_double))
    c.p_supp = supp.ctypes.data_as(C.POINTER(C.c_double))
    rands = oracle._lib("ref").d2_centroid_rands
    rands.restype = C.c_int
    assert rands(C.byref(data.mph), 0, C.byref(c)) == 0
    return ph, dict(c_w=w, c_supp=supp)


def cases():
    out = {}
    ph, c = synth.euclidean_phase(300, 6, 16, 3, (4, 16), False, 10, 1.0, seed=11)
    out["euclid_small"] = (ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10))
    ph, c = synth.euclidean_phase(200, 5, 6, 3, (2, 16), False, 10, 1.0, seed=12)
    out["euclid_oddm"] = (ph, c, dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=10))
    ph, c = synth.euclidean_phase(150, 4, 8, 2, (3, 12), False, 6, 1.0, seed=13)
    out["euclid_collide"] = (ph, c, dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=3))
    ph, c = synth.euclidean_phase(12, 3, 32, 5, (129, 520), False, 8, 1.0, seed=15)
    out["euclid_bigplans_d5"] = (ph, c, dict(maxIters=40, rhoCoeff=1.0, updatePerLoops=10))
    ph, c = synth.histogram_phase(120, 4, side=4, alpha=0.1, seed=14)
    out["hist_small"] = (ph, c, dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=10))
    w, D = read_simple()
    n, nb = w.shape
    ph = dict(metric=5, dim=0, str=nb, p_str=np.full(n, nb, np.int32), p_w=w.reshape(-1),
              dist_mat=D.reshape(-1), vocab_size=nb, label=np.array([0, 1, 0, 1, 0], np.int32),
              num_of_labels=2, label_switch=np.ones(n, np.int8))
    c = dict(c_w=np.full(2 * nb, 1.0 / nb), c_supp=None)
    out["simple_kat"] = (ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10))
    # n-gram phases: synthetic 3-grams and 2-grams (support update / check collision)
    ph, c = synth.ngram_phase(150, 5, 12, 3, 20, (20, 80), 6, seed=16)
    out["ngram_small"] = (ph, c, dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=10))
    ph, c = synth.ngram_phase(100, 4, 8, 2, 12, (10, 50), 4, seed=17)
    out["ngram_collide"] = (ph, c, dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=3))
    # the reference's protein 1-gram sequences with PAM250 costs, the protein
    # app's B-ADMM options (d2_protein_ngram.cc:383-386) and centroid size 20
    p_str, w, sym, D = read_protein_1gram(400)
    rng = np.random.default_rng(18)
    k, m = 8, 20
    label = rng.integers(0, k, size=p_str.size).astype(np.int32)
    label[:k] = np.arange(k)
    ph = dict(metric=6, dim=1, str=m, p_str=p_str, p_w=w, p_supp_sym=sym, dist_mat=D.reshape(-1),
              vocab_size=D.shape[0], label=label, num_of_labels=k,
              label_switch=np.ones(p_str.size, np.int8))
    c = dict(c_w=rng.dirichlet(np.ones(m), size=k).reshape(-1), c_supp=None,
             c_sym=sym[rng.integers(0, sym.size, size=k * m)].astype(np.int32))
    out["protein_kat"] = (ph, c, dict(maxIters=60, rhoCoeff=1.0, updatePerLoops=60))
    ph2 = dict(ph)
    out["protein_upd10"] = (ph2, c, dict(maxIters=40, rhoCoeff=1.0, updatePerLoops=10))
    ph, c = read_mountain()
    out["mountain_kat"] = (ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10))
    return out


def pack(name, ph, c, opts, res, extra=None):
    d = {"opts": np.array([opts["maxIters"], opts["rhoCoeff"], opts["updatePerLoops"]])}
    for k, v in ph.items():
        if isinstance(v, np.ndarray):
            d["in_" + k] = v
        else:
            d["meta_" + k] = np.array(v)
    d["c0_w"] = np.asarray(c["c_w"]).reshape(-1)
    if c.get("c_supp") is not None:
        d["c0_supp"] = np.asarray(c["c_supp"]).reshape(-1)
    if c.get("c_sym") is not None:
        d["c0_sym"] = np.asarray(c["c_sym"]).reshape(-1)
    d["out_c_w"] = res["c_w"]
    if c.get("c_supp") is not None:
        d["out_c_supp"] = res["c_supp"]
    if c.get("c_sym") is not None:
        d["out_c_sym"] = res["c_sym"]
    d["out_trace"] = res["trace"]
    d["out_Z_digest"] = digest(res["Z"])
    if extra:
        d.update(extra)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


def main():
    if not oracle.available("reference"):
        oracle.build(reference=True)
    for name, (ph, c, opts) in cases().items():
        res = oracle.badmm(ph, c, opts, "reference", want=())
        port = oracle.badmm(ph, c, opts, "port", want=())
        assert res["rc"] == 0 and port["rc"] == 0
        assert np.array_equal(res["c_w"], port["c_w"]) and np.array_equal(res["Z"], port["Z"])
        if c.get("c_sym") is not None:
            assert np.array_equal(res["c_sym"], port["c_sym"])
        pack(name, ph, c, opts, res)
        print(name, "col", int(np.sum(ph["p_str"])), "trace", res["trace"][:, 1])
    # warm start: second call after a k-means reassignment of ~10% of the instances
    ph, c, opts = cases()["euclid_small"]
    r1 = oracle.badmm(ph, c, opts, "reference", want=())
    rng = np.random.default_rng(99)
    lab2 = ph["label"].copy()
    mv = rng.random(lab2.size) < 0.1
    lab2[mv] = rng.integers(0, ph["num_of_labels"], size=int(mv.sum()))
    lab2[: ph["num_of_labels"]] = np.arange(ph["num_of_labels"])
    ls2 = (lab2 != ph["label"]).astype(np.int8)
    ph2 = dict(ph, label=lab2, label_switch=ls2)
    c2 = dict(c_w=r1["c_w"], c_supp=r1["c_supp"], Z=r1["Z"])
    r2 = oracle.badmm(ph2, c2, opts, "reference", want=())
    p2 = oracle.badmm(ph2, c2, opts, "port", want=())
    assert np.array_equal(r2["c_w"], p2["c_w"])
    pack("euclid_warm", ph2, dict(c_w=r1["c_w"], c_supp=r1["c_supp"]), opts, r2,
         extra={"first_c_w": c["c_w"], "first_c_supp": c["c_supp"], "first_label": ph["label"]})
    print("euclid_warm switched", int(ls2.sum()))


if __name__ == "__main__":
    main()
