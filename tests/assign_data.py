"""Seeded assignment-step problems (instances + centroids in the reference's
structures) shared by the oracle and GPU tests of the assignment step."""
import numpy as np

from d2_kmeans_gb300.assign import EUCLIDEAN, HISTOGRAM, SPARSE_HISTOGRAM, Mph, Work

N_GRAM, WORD_EMBED = 6, 7


def euclid_phase(rng, n, dim, lo, hi, k, m, spread=3.0):
    """instances: supports around k cluster means; centroids: m supports near each mean"""
    means = rng.normal(size=(k, dim)) * spread
    lab = rng.integers(0, k, size=n)
    p_str = rng.integers(lo, hi + 1, size=n).astype(np.int32)
    supp = np.concatenate([means[lab[i]] + rng.normal(size=(s, dim)) for i, s in enumerate(p_str)])
    w = np.concatenate([rng.dirichlet(np.full(s, 0.8)) for s in p_str])
    c_supp = np.concatenate([means[j] + rng.normal(size=(m, dim)) * 0.8 for j in range(k)])
    c_w = np.concatenate([rng.dirichlet(np.ones(m)) for _ in range(k)])
    data = dict(metric=EUCLIDEAN, dim=dim, str=m, p_str=p_str, p_w=w, p_supp=supp.reshape(-1))
    cent = dict(metric=EUCLIDEAN, dim=dim, str=m, p_w=c_w, p_supp=c_supp.reshape(-1))
    return data, cent


def grid_costs(side):
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 2)
    return ((g[:, None, :] - g[None, :, :]) ** 2).sum(-1).astype(float)


def hist_phase(rng, n, k, side, sparse=False, asym=False):
    V = side * side
    dm = grid_costs(side)
    if asym:
        dm = dm * (1.0 + 0.3 * rng.random((V, V)))
    protos = rng.dirichlet(np.full(V, 0.3), size=k)
    lab = rng.integers(0, k, size=n)
    c_w = np.concatenate([rng.dirichlet(protos[j] * 50 + 0.05) for j in range(k)])
    cent = dict(metric=HISTOGRAM, dim=0, str=V, p_w=c_w, dist_mat=dm, vocab_size=V)
    if not sparse:
        w = np.stack([rng.dirichlet(protos[lab[i]] * 40 + 0.05) for i in range(n)])
        w[w < 1e-4] = 0.0
        w /= w.sum(1, keepdims=True)
        data = dict(metric=HISTOGRAM, dim=0, str=V, p_str=np.full(n, V, np.int32),
                    p_w=w.reshape(-1), dist_mat=dm, vocab_size=V)
    else:
        p_str = rng.integers(3, V // 2, size=n).astype(np.int32)
        sym, w = [], []
        for i, s in enumerate(p_str):
            p = protos[lab[i]] + 1e-3
            ids = np.sort(rng.choice(V, s, replace=False, p=p / p.sum()))
            sym.append(ids)
            w.append(rng.dirichlet(np.ones(s)))
        data = dict(metric=SPARSE_HISTOGRAM, dim=0, str=V, p_str=p_str, p_w=np.concatenate(w),
                    p_supp_sym=np.concatenate(sym).astype(np.int32), dist_mat=dm, vocab_size=V)
    return data, cent


def build(data_phases, cent_phases, n, k, label):
    data = Mph(data_phases, n, label=label, num_of_labels=k)
    cents = Mph(cent_phases, k, num_of_labels=k)
    return data, cents


def ref_scratch(data_phases, n, k):
    """The g_var[n].C arrays the reference's d2_compute_distance needs
    (clustering_util.c:178-197): str * (col + k * str) doubles per phase, with
    the sparse-histogram cost blocks precomputed as _dpdist2_submat does."""
    out = []
    for ph in data_phases:
        p_str = np.asarray(ph["p_str"])
        col = int(p_str.sum())
        m = int(ph["str"])
        C = np.zeros(m * (col + k * m))
        if ph["metric"] == SPARSE_HISTOGRAM:
            V = ph["vocab_size"]
            dm = np.asarray(ph["dist_mat"]).reshape(V, V)
            cum = np.concatenate([[0], np.cumsum(p_str)])
            for i in range(p_str.size):
                sym = ph["p_supp_sym"][cum[i]:cum[i + 1]]
                C[m * cum[i]: m * cum[i + 1]] = dm[sym, :].reshape(-1)
        out.append(C)
    return out


def perturb(cent_phases, rng, scale):
    """new centroids near the old ones (weights renormalised)"""
    out = []
    for ph in cent_phases:
        ph = dict(ph)
        w = np.asarray(ph["p_w"]).reshape(-1, ph["str"])
        w = w * np.exp(rng.normal(size=w.shape) * scale)
        ph["p_w"] = (w / w.sum(1, keepdims=True)).reshape(-1)
        if ph.get("p_supp") is not None:
            ph["p_supp"] = np.asarray(ph["p_supp"]) + rng.normal(size=len(ph["p_supp"])) * scale
        out.append(ph)
    return out


def oracle_clustering(oracle_mod, data_phases, cent_phases, n, k, label, max_iter, use_triangle,
                      opts=None):
    """The reference's d2_clustering loop (src/d2/clustering.c:409-525) composed
    from the oracle's labeling restatement and its B-ADMM restatement (both
    bit-identical to the reference's own functions), no time budget.  Returns
    (labels, centroid Mph, rounds)."""
    opts = opts or dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    lab = oracle_mod.Labeling("port")
    data = Mph(data_phases, n, label=np.asarray(label).copy(), num_of_labels=k)
    cents = Mph(cent_phases, k, num_of_labels=k)
    work = Work(n, k, len(data_phases))
    Z = [None] * len(data_phases)
    it = 0
    while it < max_iter:
        if use_triangle:
            changed = lab.labeling_prep(data, cents, work)[0]
        else:
            changed = lab.labeling(data, cents, work)[0]
        if changed < 0.001 * n:
            break
        old = Mph([dict(ph, p_w=cents.arrays[i]["p_w"].copy(),
                        p_supp=None if "p_supp" not in cents.arrays[i] else cents.arrays[i]["p_supp"].copy(),
                        p_supp_sym=(None if "p_supp_sym" not in cents.arrays[i]
                                    else cents.arrays[i]["p_supp_sym"].copy()))
                   for i, ph in enumerate(cent_phases)], k, num_of_labels=k)
        for i, ph in enumerate(data_phases):
            phase = dict(ph, label=data.label.copy(), num_of_labels=k,
                         label_switch=work.label_switch.copy())
            cw = {"c_w": cents.arrays[i]["p_w"], "c_supp": cents.arrays[i].get("p_supp")}
            if ph["metric"] == N_GRAM:
                cw["c_sym"] = cents.arrays[i]["p_supp_sym"]
            if Z[i] is not None:
                cw["Z"] = Z[i]
            r = oracle_mod.badmm(phase, cw, opts, "port", want=())
            assert r["rc"] == 0
            cents.arrays[i]["p_w"][:] = r["c_w"]
            if "p_supp" in cents.arrays[i]:
                cents.arrays[i]["p_supp"][:] = r["c_supp"][:cents.arrays[i]["p_supp"].size]
            if ph["metric"] == N_GRAM:
                cents.arrays[i]["p_supp_sym"][:] = r["c_sym"]
            Z[i] = r["Z"]
        if use_triangle:
            lab.labeling_post(data, old, cents, work)
        it += 1
    if use_triangle:
        lab.labeling(data, cents, work)
    return data.label.copy(), cents, it


def embed_phase(rng, n, k, V, dim, m, lo=3, hi=30):
    """word-embedding instances (distinct word ids, Dirichlet weights) over a
    Gaussian vocabulary; centroids with m supports in R^dim near topic words"""
    vocab = rng.normal(size=(V, dim))
    topics = [rng.choice(V, V // k, replace=False) for _ in range(k)]
    p_str = rng.integers(lo, hi + 1, size=n).astype(np.int32)
    lab = rng.integers(0, k, size=n)
    sym, w = [], []
    for i, s in enumerate(p_str):
        pool = topics[lab[i]] if rng.random() < 0.8 and s <= V // k else np.arange(V)
        sym.append(rng.choice(pool, s, replace=False))
        w.append(rng.dirichlet(np.ones(s)))
    data = dict(metric=WORD_EMBED, dim=dim, str=m, p_str=p_str, p_w=np.concatenate(w),
                p_supp_sym=np.concatenate(sym).astype(np.int32), vocab_vec=vocab.reshape(-1),
                vocab_size=V)
    c_supp = np.concatenate([vocab[rng.choice(topics[j], m, replace=False)] + rng.normal(size=(m, dim)) * 0.3
                             for j in range(k)])
    c_w = np.concatenate([rng.dirichlet(np.ones(m)) for _ in range(k)])
    cent = dict(metric=EUCLIDEAN, dim=dim, str=m, p_w=c_w, p_supp=c_supp.reshape(-1))
    return data, cent


def ngram_phase(rng, n, k, m, dim, V, lo=10, hi=80):
    """sequences over V symbols from k families as distributions of their
    distinct dim-grams; centroids: m n-grams of each family with Dirichlet weights"""
    from d2_kmeans_gb300 import synth
    dist = synth.symbol_cost(V, int(rng.integers(1 << 30)))
    fam = rng.dirichlet(np.full(V, 0.4), size=k)
    lab = rng.integers(0, k, size=n)
    radix = V ** np.arange(dim - 1, -1, -1)
    p_str, sym, w = [], [], []
    for i in range(n):
        seq = rng.choice(V, size=int(rng.integers(lo, hi + 1)), p=fam[lab[i]])
        code, cnt = np.unique(np.lib.stride_tricks.sliding_window_view(seq, dim) @ radix,
                              return_counts=True)
        p_str.append(code.size)
        sym.append(((code[:, None] // radix[None, :]) % V).reshape(-1))
        w.append(cnt / cnt.sum())
    data = dict(metric=N_GRAM, dim=dim, str=m, p_str=np.array(p_str, np.int32), p_w=np.concatenate(w),
                p_supp_sym=np.concatenate(sym).astype(np.int32), dist_mat=dist.reshape(-1), vocab_size=V)
    c_sym = np.concatenate([rng.choice(V, size=m * dim, p=fam[j]) for j in range(k)]).astype(np.int32)
    c_w = np.concatenate([rng.dirichlet(np.ones(m)) for _ in range(k)])
    cent = dict(metric=N_GRAM, dim=dim, str=m, p_w=c_w, p_supp_sym=c_sym, dist_mat=dist.reshape(-1),
                vocab_size=V)
    return data, cent
