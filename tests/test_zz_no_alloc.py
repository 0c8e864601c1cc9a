"""d2g_distmat_noalloc, the ground-cost entry point for callers that cannot
allocate GPU memory (code running inside another runtime's allocator, or
handed only pre-allocated device buffers, must not call cudaMalloc), against
the allocating calculate_distmat on the same
inputs: two calls in a row (the second smaller and of another metric type, so
anything a call left in the shared fixed scratch array must not show through),
and both against the oracle's cost blocks.  Tolerance: the FP64 path's 1e-9
relative between the two GPU entry points, 1e-12 against the oracle.  Also: a
second call leaves the device's free memory unchanged, and invalid inputs are
refused with the status of the failed check."""
import ctypes as C

import numpy as np
import pytest

from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import synth

pytestmark = pytest.mark.gpu


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def calculate_distmat_host(lib, ph, c):
    """The existing entry point: host buffers in, host C out."""
    p_str = np.ascontiguousarray(ph["p_str"], np.int32)
    col = int(p_str.sum())
    m, dim = int(ph["str"]), int(ph["dim"])
    keep = []

    def k(a, dt):
        a = None if a is None else np.ascontiguousarray(a, dt)
        keep.append(a)
        return a
    data = L.sph()
    data.dim, data.str, data.col = dim, m, col
    data.p_str = _ptr(p_str, C.c_int)
    data.p_w = _ptr(k(ph["p_w"], np.float64), C.c_double)
    data.metric_type = int(ph["metric"])
    data.p_supp = _ptr(k(ph.get("p_supp"), np.float64), C.c_double)
    data.p_supp_sym = _ptr(k(ph.get("p_supp_sym"), np.int32), C.c_int)
    data.vocab_size = int(ph.get("vocab_size", 0))
    data.vocab_vec = _ptr(k(ph.get("vocab_vec"), np.float64), C.c_double)
    cen = L.sph()
    cen.dim, cen.str, cen.col = dim, m, int(ph["num_of_labels"]) * m
    cs = k(c["c_supp"], np.float64)
    cen.p_supp = _ptr(cs, C.c_double)
    label = k(ph["label"], np.int32)
    out = np.zeros(m * col)
    lib.calculate_distmat(C.byref(data), _ptr(label, C.c_int), p_str.size, C.byref(cen),
                          _ptr(out, C.c_double))
    return out


def device_inputs(torch, ph, c, label=None):
    """Every input of d2g_distmat_noalloc as a device tensor the caller owns."""
    dev = torch.device("cuda")
    t = lambda a, dt: None if a is None else torch.tensor(np.asarray(a, dt), device=dev)  # noqa: E731
    col = int(np.sum(ph["p_str"]))
    return dict(p_str=t(ph["p_str"], np.int32), supp=t(ph.get("p_supp"), np.float64),
                sym=t(ph.get("p_supp_sym"), np.int32), vocab=t(ph.get("vocab_vec"), np.float64),
                label=t(ph["label"] if label is None else label, np.int32),
                c_supp=t(c["c_supp"], np.float64),
                out=torch.full((int(ph["str"]) * col,), float("nan"), dtype=torch.float64, device=dev))


def call_noalloc(lib, ph, d):
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    return lib.d2g_distmat_noalloc(int(ph["metric"]), int(ph["dim"]), int(ph["str"]), d["p_str"].numel(),
                                   int(np.sum(ph["p_str"])), p(d["p_str"]), p(d["supp"]), p(d["sym"]),
                                   p(d["vocab"]), int(ph.get("vocab_size", 0)), p(d["label"]),
                                   int(ph["num_of_labels"]), p(d["c_supp"]), p(d["out"]), None)


def distmat_noalloc_device(lib, torch, ph, c):
    """The new entry point: every array is a device buffer the caller owns."""
    dev = torch.device("cuda")
    p_str = torch.tensor(np.asarray(ph["p_str"], np.int32), device=dev)
    col = int(np.sum(ph["p_str"]))
    m, dim = int(ph["str"]), int(ph["dim"])
    supp = None if ph.get("p_supp") is None else torch.tensor(np.asarray(ph["p_supp"]), device=dev)
    sym = (None if ph.get("p_supp_sym") is None
           else torch.tensor(np.asarray(ph["p_supp_sym"], np.int32), device=dev))
    vocab = (None if ph.get("vocab_vec") is None
             else torch.tensor(np.asarray(ph["vocab_vec"]), device=dev))
    label = torch.tensor(np.asarray(ph["label"], np.int32), device=dev)
    c_supp = torch.tensor(np.asarray(c["c_supp"], np.float64), device=dev)
    out = torch.full((m * col,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    rc = lib.d2g_distmat_noalloc(int(ph["metric"]), dim, m, p_str.numel(), col, p(p_str), p(supp),
                                 p(sym), p(vocab), int(ph.get("vocab_size", 0)), p(label),
                                 int(ph["num_of_labels"]), p(c_supp), p(out), None)
    assert rc == 0, lib.d2g_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _bind(lib):
    f = lib.d2g_distmat_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_size_t, C.c_size_t] + [C.c_void_p] * 4 + \
        [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib


def _two_phases():
    ph1, c1 = synth.euclidean_phase(400, 5, 16, 3, (4, 20), False, 8, 1.0, seed=51)
    ph2, c2 = synth.embed_phase(60, 3, 8, V=300, dim=12, sizes=(3, 25), seed=52)
    return (ph1, c1), (ph2, c2)


def test_noalloc_distmat_matches_calculate_distmat_twice(oracle_mod):
    torch = pytest.importorskip("torch")
    lib = _bind(L.load())
    for ph, c in _two_phases():
        ref = calculate_distmat_host(lib, ph, c)
        got = distmat_noalloc_device(lib, torch, ph, c)
        assert np.isfinite(got).all()
        np.testing.assert_allclose(got, ref, rtol=1e-9, atol=0)
        # and both against the oracle's cost blocks (FP64 on the CPU)
        np.testing.assert_allclose(got, oracle_mod.cost_blocks(ph, c), rtol=1e-12, atol=0)


def test_noalloc_second_call_takes_no_device_memory():
    torch = pytest.importorskip("torch")
    lib = _bind(L.load())
    (ph, c), _ = _two_phases()
    d = device_inputs(torch, ph, c)
    assert call_noalloc(lib, ph, d) == 0, lib.d2g_last_error()  # set-up call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert call_noalloc(lib, ph, d) == 0, lib.d2g_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_refuses_a_label_out_of_range():
    torch = pytest.importorskip("torch")
    lib = _bind(L.load())
    (ph, c), _ = _two_phases()
    label = np.array(ph["label"], np.int32)
    label[7] = int(ph["num_of_labels"])  # one past the last cluster
    d = device_inputs(torch, ph, c, label=label)
    assert call_noalloc(lib, ph, d) == L.D2G_E_INVAL
    assert b"status 2" in lib.d2g_last_error()
    # the shared array keeps nothing of the refused call: a good call after it is exact
    d = device_inputs(torch, ph, c)
    assert call_noalloc(lib, ph, d) == 0, lib.d2g_last_error()
    torch.cuda.synchronize()
    np.testing.assert_allclose(d["out"].cpu().numpy(), calculate_distmat_host(lib, ph, c), rtol=1e-9, atol=0)


def test_noalloc_refuses_sizes_beyond_the_fixed_array():
    lib = _bind(L.load())
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    for size, col in ((2_000_000, 20_000_000), (100, 3_000_000), (2 ** 62, 2 ** 62), (2 ** 61 + 1, 8)):
        rc = lib.d2g_distmat_noalloc(0, 3, 16, size, col, dummy, dummy, None, None, 0,
                                     dummy, 4, dummy, dummy, None)
        assert rc == L.D2G_E_INVAL, (size, col)
        assert b"8 MiB" in lib.d2g_last_error()
