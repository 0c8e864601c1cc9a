"""Seeded synthetic D2 phases for the five B-ADMM workloads.

The reference's experiment data (20newsgroups, icip14, USPS, MNIST) is not
available, so each workload is a seeded stand-in with the shapes, sizes and
value distributions of the experiment it replaces.  All draws come from
``numpy.random.default_rng(seed)``.  The returned dictionaries use the
reference's d2 layout (include/d2/clustering.h:14-95): per-instance support
sizes ``p_str``, flat weights ``p_w`` (each instance sums to 1, as
src/d2/clustering_io.c:140-151 re-normalises on read), supports ``p_supp``
(col x dim, one row per support point) or vocabulary ids ``p_supp_sym``.
"""
from __future__ import annotations

import numpy as np

EUCLIDEAN, HISTOGRAM, N_GRAM, WORD_EMBED, SPARSE_HISTOGRAM = 0, 5, 6, 7, 12

# weights below this are lifted before re-normalising; the reference's reader
# asserts w > 1e-9 for non-histogram phases (clustering_io.c:145)
_W_FLOOR = 1e-8


def _segment_normalise(w: np.ndarray, p_str: np.ndarray) -> np.ndarray:
    starts = np.concatenate(([0], np.cumsum(p_str)[:-1]))
    sums = np.add.reduceat(w, starts)
    return w / np.repeat(sums, p_str)


def _dirichlet_segments(rng, p_str, alpha, floor=_W_FLOOR):
    g = rng.gamma(alpha, 1.0, size=int(p_str.sum()))
    w = _segment_normalise(g, p_str)
    if floor:
        w = _segment_normalise(np.maximum(w, floor), p_str)
    return w


def _labels(rng, n, k):
    lab = rng.integers(0, k, size=n).astype(np.int32)
    lab[:k] = rng.permutation(k).astype(np.int32)  # every cluster non-empty
    return lab


def _gmm(rng, n_points, dim, n_comp, mean_scale=3.0):
    means = rng.normal(0.0, mean_scale, size=(n_comp, dim))
    comp = rng.integers(0, n_comp, size=n_points)
    return means[comp] + rng.normal(0.0, 1.0, size=(n_points, dim)), means


def euclidean_phase(n, k, m, dim=3, sizes=(4, 16), log_uniform=False, n_comp=10,
                    alpha=1.0, seed=0):
    """GMM-supported Euclidean D2 phase plus k seeded initial centroids."""
    rng = np.random.default_rng(seed)
    lo, hi = sizes
    if log_uniform:
        p_str = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=n))).astype(np.int32)
        p_str = np.clip(p_str, lo, hi)
    else:
        p_str = rng.integers(lo, hi + 1, size=n).astype(np.int32)
    col = int(p_str.sum())
    supp, means = _gmm(rng, col, dim, n_comp)
    p_w = _dirichlet_segments(rng, p_str, alpha)
    label = _labels(rng, n, k)
    comp = rng.integers(0, n_comp, size=k * m)
    c_supp = means[comp] + rng.normal(0.0, 1.0, size=(k * m, dim))
    c_w = rng.dirichlet(np.ones(m), size=k)
    phase = dict(metric=EUCLIDEAN, dim=dim, str=m, p_str=p_str, p_w=p_w,
                 p_supp=supp.reshape(-1), label=label, num_of_labels=k,
                 label_switch=np.ones(n, np.int8))
    cent = dict(c_w=c_w.reshape(-1), c_supp=c_supp.reshape(-1))
    return phase, cent


def grid_cost(side):
    """Squared grid distance between the bins of a side x side image."""
    r, c = np.divmod(np.arange(side * side), side)
    return ((r[:, None] - r[None, :]) ** 2 + (c[:, None] - c[None, :]) ** 2).astype(np.float64)


def histogram_phase(n, k, side=16, alpha=0.1, seed=0):
    """Dense side*side-bin histograms ~ Dirichlet(alpha) with squared grid cost."""
    rng = np.random.default_rng(seed)
    bins = side * side
    p_str = np.full(n, bins, np.int32)
    g = rng.gamma(alpha, 1.0, size=(n, bins))
    g[np.arange(n), rng.integers(0, bins, size=n)] += 1e-3  # no all-zero histogram
    p_w = (g / g.sum(axis=1, keepdims=True)).reshape(-1)
    label = _labels(rng, n, k)
    c_w = rng.dirichlet(np.ones(bins), size=k)
    phase = dict(metric=HISTOGRAM, dim=0, str=bins, p_str=p_str, p_w=p_w,
                 dist_mat=grid_cost(side).reshape(-1), vocab_size=bins, label=label,
                 num_of_labels=k, label_switch=np.ones(n, np.int8))
    return phase, dict(c_w=c_w.reshape(-1), c_supp=None)


def vocabulary(V, dim, seed=0):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(V, dim))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def embed_phase(n, k, m, V=20000, dim=300, sizes=(20, 400), zipf=1.1, seed=0, vocab=None):
    """Bag-of-word-vectors documents over a unit-normed vocabulary.

    Each document draws m_i distinct token ids without replacement with
    probability proportional to rank^-zipf (Gumbel top-k); weights are
    tf-idf-like (a Gamma(1) term frequency times log(V/rank)) normalised to 1.
    Centroid supports start at m random vocabulary vectors per cluster.
    """
    rng = np.random.default_rng(seed)
    if vocab is None:
        vocab = vocabulary(V, dim, seed + 1000)
    logp = -zipf * np.log(np.arange(1, V + 1, dtype=np.float64))
    idf = np.log(V / np.arange(1, V + 1, dtype=np.float64)) + 1.0
    p_str = rng.integers(sizes[0], sizes[1] + 1, size=n).astype(np.int32)
    syms = []
    ws = []
    chunk = 256
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        keys = logp[None, :] + rng.gumbel(size=(e - s, V))
        for r in range(e - s):
            mi = int(p_str[s + r])
            ids = np.argpartition(-keys[r], mi - 1)[:mi]
            ids.sort()
            syms.append(ids.astype(np.int32))
            ws.append(rng.gamma(1.0, 1.0, size=mi) * idf[ids])
    p_supp_sym = np.concatenate(syms)
    p_w = _segment_normalise(np.concatenate(ws), p_str)
    label = _labels(rng, n, k)
    c_supp = vocab[rng.integers(0, V, size=k * m)]
    c_w = np.full((k, m), 1.0 / m)
    phase = dict(metric=WORD_EMBED, dim=dim, str=m, p_str=p_str, p_w=p_w, p_supp_sym=p_supp_sym,
                 vocab_vec=vocab.reshape(-1), vocab_size=V, label=label, num_of_labels=k,
                 label_switch=np.ones(n, np.int8))
    return phase, dict(c_w=c_w.reshape(-1), c_supp=c_supp.reshape(-1))


def symbol_cost(V=20, seed=0):
    """Symmetric symbol-to-symbol cost with a zero diagonal, in half units like
    a substitution-matrix distance: squared distances of V random points in R^5."""
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(V, 5))
    d = ((p[:, None, :] - p[None, :, :]) ** 2).sum(-1)
    return np.round(2.0 * d) / 2.0


def ngram_phase(n, k, m, dim=3, V=20, lengths=(30, 400), families=16, seed=0, dist=None):
    """Sequences over V symbols as n-gram distributions (D2_N_GRAM).

    Each sequence has a log-uniform length and draws its symbols i.i.d. from
    one of ``families`` symbol distributions (Dirichlet(0.5)); its supports
    are its distinct dim-grams (symbols in [0, V)) weighted by their counts,
    normalised to 1, ordered by decreasing count like the reference's protein
    n-gram files.  Centroid supports start at m n-grams drawn from the data.
    """
    rng = np.random.default_rng(seed)
    if dist is None:
        dist = symbol_cost(V, seed + 500)
    fam = rng.dirichlet(np.full(V, 0.5), size=families)
    lo, hi = lengths
    L = np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=n))), max(lo, dim), hi)
    p_str, syms, ws = [], [], []
    radix = V ** np.arange(dim - 1, -1, -1)
    for i in range(n):
        seq = rng.choice(V, size=int(L[i]), p=fam[rng.integers(families)])
        grams = np.lib.stride_tricks.sliding_window_view(seq, dim)
        code, cnt = np.unique(grams @ radix, return_counts=True)
        order = np.argsort(-cnt, kind="stable")
        code, cnt = code[order], cnt[order]
        tup = (code[:, None] // radix[None, :]) % V
        p_str.append(len(code))
        syms.append(tup.reshape(-1))
        ws.append(cnt / cnt.sum())
    p_str = np.asarray(p_str, np.int32)
    p_supp_sym = np.concatenate(syms).astype(np.int32)
    p_w = np.concatenate(ws)
    label = _labels(rng, n, k)
    pick = rng.integers(0, int(p_str.sum()), size=k * m)
    c_sym = p_supp_sym.reshape(-1, dim)[pick].reshape(-1)
    c_w = rng.dirichlet(np.ones(m), size=k)
    phase = dict(metric=N_GRAM, dim=dim, str=m, p_str=p_str, p_w=p_w, p_supp_sym=p_supp_sym,
                 dist_mat=dist.reshape(-1), vocab_size=V, label=label, num_of_labels=k,
                 label_switch=np.ones(n, np.int8))
    return phase, dict(c_w=c_w.reshape(-1), c_supp=None, c_sym=c_sym.astype(np.int32))


def serving_centroids(k=256, m=64, dim=64, n_comp=32, seed=0):
    rng = np.random.default_rng(seed)
    pts, means = _gmm(rng, k * m, dim, n_comp)
    c_w = rng.dirichlet(np.ones(m), size=k)
    return c_w, pts.reshape(k, m, dim), means


def serving_queries(n_req, means, sizes=(4, 512), alpha=1.0, seed=1):
    """Query distributions: log-uniform support size, GMM supports, Dirichlet weights."""
    rng = np.random.default_rng(seed)
    dim = means.shape[1]
    lo, hi = sizes
    sz = np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=n_req))), lo, hi)
    out = []
    for mq in sz.astype(int):
        comp = rng.integers(0, means.shape[0], size=mq)
        supp = means[comp] + rng.normal(size=(mq, dim))
        w = rng.dirichlet(np.full(mq, alpha))
        w = np.maximum(w, _W_FLOOR)
        out.append((w / w.sum(), supp))
    return out


# The five workloads.  ``scale`` shrinks n (and nothing else) for tests that
# need the oracle to finish in seconds.
def workload(name: str, seed: int = 0, scale: float = 1.0):
    def N(n):
        return max(8, int(round(n * scale)))
    if name == "plain":          # n=2000, d=3, m_i U{4..16}, k=10, m=16, 100 iterations
        ph, c = euclidean_phase(N(2000), 10, 16, 3, (4, 16), False, 10, 1.0, seed)
        return ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    if name == "batched":        # n=200000, m_i log-uniform 8..128, k=64, m=32, 200 iterations
        ph, c = euclidean_phase(N(200000), 64, 32, 3, (8, 128), True, 64, 0.5, seed)
        return ph, c, dict(maxIters=200, rhoCoeff=2.0, updatePerLoops=10)
    if name == "embed":          # V=20000 x 300, n=20000 docs of 20..400 tokens, k=20, m=64
        ph, c = embed_phase(N(20000), 20, 64, 20000, 300, (20, 400), 1.1, seed)
        return ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    if name == "hist":           # phase 1 of the two-phase set: 256-bin histograms, k=32
        ph, c = histogram_phase(N(100000), 32, 16, 0.1, seed)
        return ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    if name == "ngram":          # sequences as 3-grams over 20 symbols, k=64, m=32
        ph, c = ngram_phase(N(20000), 64, 32, 3, 20, (30, 400), 16, seed)
        return ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    if name == "twophase_euclid":  # phase 2: d=3, m_i 4..32, k=32, m=16
        ph, c = euclidean_phase(N(100000), 32, 16, 3, (4, 32), False, 10, 1.0, seed + 7)
        return ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    raise KeyError(name)
