"""ctypes bindings of libd2g.so (include/d2g.h).

The structures mirror the reference's d2 data model
(include/d2/clustering.h:14-200, include/d2/param.h:4-8, SCALAR = double) so
that the drop-in entry point d2_centroid_sphBregman can be driven exactly as
the reference's own d2_clustering() drives it.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# D2G_LIB selects another build of the library (e.g. an instrumented one)
LIB_PATH = os.environ.get("D2G_LIB") or os.path.join(HERE, "libd2g.so")

D2_EUCLIDEAN_L2, D2_CITYBLOCK_L1, D2_HISTOGRAM, D2_N_GRAM, D2_WORD_EMBED, D2_SPARSE_HISTOGRAM = (
    0, 1, 5, 6, 7, 12)

D2G_OK, D2G_E_INVAL, D2G_E_CUDA, D2G_E_NOMEM, D2G_E_UNSUPPORTED = 0, -1, -2, -3, -4
D2G_E_EMPTY_CLUSTER, D2G_E_NUMERIC, D2G_E_ADMISSION, D2G_E_NOTFOUND = -5, -6, -7, -8
D2G_SHARD_GLOBAL_RHO = 1

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class sph(C.Structure):
    _fields_ = [("dim", C.c_int), ("str", C.c_int), ("max_str", C.c_int),
                ("col", C.c_size_t), ("max_col", C.c_size_t),
                ("p_str", ip), ("p_str_cum", C.POINTER(C.c_size_t)), ("p_w", dp),
                ("metric_type", C.c_int), ("p_supp", dp), ("p_supp_sym", ip),
                ("dist_mat", dp), ("vocab_size", C.c_int), ("vocab_vec", dp),
                ("is_meta_allocated", C.c_char)]


class trieq(C.Structure):
    _fields_ = [("l", dp), ("u", dp), ("s", dp), ("c", dp), ("r", C.c_char_p)]


class mph(C.Structure):
    _fields_ = [("s_ph", C.c_int), ("size", C.c_size_t), ("global_size", C.c_size_t),
                ("label", ip), ("num_of_labels", C.c_int), ("ph", C.POINTER(sph))]


class var_sph(C.Structure):
    _fields_ = [("C", dp), ("X", dp), ("L", dp)]


class var_sphBregman(C.Structure):
    _fields_ = [("X", dp), ("Z", dp), ("Y", dp), ("Xc", dp), ("Zr", dp)]


class var_mph(C.Structure):
    _fields_ = [("s_ph", C.c_int), ("g_var", C.POINTER(var_sph)),
                ("l_var_sphBregman", C.POINTER(var_sphBregman)),
                ("label_switch", C.POINTER(C.c_char)), ("tr", trieq)]


class BADMM_options(C.Structure):
    _fields_ = [("maxIters", C.c_int), ("rhoCoeff", C.c_double), ("updatePerLoops", C.c_int)]


class d2g_config(C.Structure):
    _fields_ = [("precision", C.c_int), ("verbose", C.c_int), ("use_graph", C.c_int),
                ("sync_scratch", C.c_int), ("profile", C.c_int), ("cost_gemm", C.c_int),
                ("keep_time_budget", C.c_int), ("pair_iterations", C.c_int)]


class d2g_phase_desc(C.Structure):
    _fields_ = [("metric_type", C.c_int), ("dim", C.c_int), ("str", C.c_int),
                ("size", C.c_size_t), ("p_str", C.c_void_p), ("p_w", C.c_void_p),
                ("p_supp", C.c_void_p), ("p_supp_sym", C.c_void_p), ("vocab_vec", C.c_void_p),
                ("dist_mat", C.c_void_p), ("vocab_size", C.c_int), ("label", C.c_void_p),
                ("num_of_labels", C.c_int), ("global_size", C.c_size_t)]


class d2g_badmm_opts(C.Structure):
    _fields_ = [("maxIters", C.c_int), ("rhoCoeff", C.c_double), ("updatePerLoops", C.c_int),
                ("time_budget", C.c_double)]


class d2g_run_stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rho", C.c_double), ("total_ms", C.c_double),
                ("plan_ms_avg", C.c_double), ("plan_launches", C.c_int),
                ("kernel_launches", C.c_longlong), ("plan_bytes", C.c_double),
                ("plan_entries", C.c_size_t), ("path", C.c_int), ("table_ms_avg", C.c_double),
                ("table_launches", C.c_int), ("table_flops", C.c_double)]


class d2g_tuning(C.Structure):
    _fields_ = [("exchange", C.c_int), ("stage_costs", C.c_int), ("ctas_per_sm", C.c_int),
                ("cost_gemm", C.c_int), ("pairs", C.c_int), ("unit_order", C.c_int),
                ("stage_scales", C.c_int)]


class d2g_dists(C.Structure):
    _fields_ = [("size", C.c_size_t), ("str", C.c_int), ("p_str", C.c_void_p), ("p_w", C.c_void_p),
                ("p_supp", C.c_void_p), ("p_supp_sym", C.c_void_p)]


class d2g_server_desc(C.Structure):
    _fields_ = [("num_of_labels", C.c_int), ("str", C.c_int), ("dim", C.c_int),
                ("c_w", C.c_void_p), ("c_supp", C.c_void_p), ("iters", C.c_int),
                ("rhoCoeff", C.c_double), ("hbm_budget_bytes", C.c_size_t),
                ("max_queue", C.c_int), ("max_batch_entries", C.c_int)]


# name -> (restype, argtypes); every function declared in include/d2g.h
SIGNATURES = {
    "d2_allocate_work_sphBregman": (C.c_int, [C.POINTER(sph), C.c_size_t, C.POINTER(var_sphBregman)]),
    "d2_free_work_sphBregman": (C.c_int, [C.POINTER(var_sphBregman)]),
    "d2_centroid_sphBregman": (C.c_int, [C.POINTER(mph), C.POINTER(var_mph), C.c_int,
                                         C.POINTER(sph), C.POINTER(sph)]),
    "calculate_distmat": (None, [C.POINTER(sph), ip, C.c_size_t, C.POINTER(sph), dp]),
    "d2g_distmat_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_size_t, C.c_size_t] +
                            [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                C.c_void_p, C.c_void_p]),
    "d2g_get_config": (C.c_int, [C.POINTER(d2g_config)]),
    "d2g_set_config": (C.c_int, [C.POINTER(d2g_config)]),
    "d2g_error_string": (C.c_char_p, [C.c_int]),
    "d2g_last_error": (C.c_char_p, []),
    "d2g_phase_create": (C.c_int, [C.POINTER(d2g_phase_desc), C.c_int, C.POINTER(C.c_void_p)]),
    "d2g_phase_destroy": (C.c_int, [C.c_void_p]),
    "d2g_phase_refresh": (C.c_int, [C.c_void_p, C.POINTER(d2g_phase_desc)]),
    "d2g_phase_set_labels": (C.c_int, [C.c_void_p, C.c_void_p]),
    "d2g_phase_set_plans": (C.c_int, [C.c_void_p, C.c_void_p]),
    "d2g_phase_get_plans": (C.c_int, [C.c_void_p, C.c_void_p]),
    "d2g_badmm_run": (C.c_int, [C.c_void_p, C.POINTER(d2g_badmm_opts), C.c_void_p, C.c_void_p,
                                C.c_void_p]),
    "d2g_centroid_rands": (C.c_int, [C.POINTER(mph), C.c_int, C.POINTER(sph)]),
    "d2g_write_split": (C.c_int, [C.c_char_p, C.POINTER(mph), C.c_int, C.c_char]),
    "d2g_badmm_run_sym": (C.c_int, [C.c_void_p, C.POINTER(d2g_badmm_opts), C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "d2g_phase_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "d2g_phase_stats": (C.c_int, [C.c_void_p, C.POINTER(d2g_run_stats)]),
    "d2g_phase_get_scratch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "d2g_phase_stream": (C.c_void_p, [C.c_void_p]),
    "d2g_phase_test_wait": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double]),
    "d2g_phase_set_allreduce": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "d2g_badmm_run_shards": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(d2g_badmm_opts), C.c_int,
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "d2g_read": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(mph)]),
    "d2g_mph_alloc": (C.c_int, [C.c_int, C.c_size_t, ip, ip, ip, C.POINTER(C.POINTER(mph))]),
    "d2g_mph_free": (C.c_int, [C.POINTER(mph)]),
    "d2g_emd_pairs": (C.c_int, [C.c_int, C.c_int, C.POINTER(d2g_dists), C.POINTER(d2g_dists),
                                C.c_void_p, C.c_int, C.c_size_t] + [C.c_void_p] * 4),
    "d2g_compute_distances": (C.c_int, [C.POINTER(mph), C.POINTER(mph), C.c_int, C.c_size_t,
                                        C.c_void_p, C.c_void_p, C.c_void_p]),
    "d2g_labeling": (C.c_int, [C.POINTER(mph), C.POINTER(mph), C.POINTER(var_mph), C.c_int,
                               C.POINTER(C.c_size_t), C.POINTER(C.c_double)]),
    "d2g_labeling_prep": (C.c_int, [C.POINTER(mph), C.POINTER(mph), C.POINTER(var_mph), C.c_int,
                                    C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "d2g_labeling_post": (C.c_int, [C.POINTER(mph), C.POINTER(mph), C.POINTER(mph),
                                    C.POINTER(var_mph), C.c_int]),
    "d2_compute_distance": (C.c_double, [C.POINTER(mph), C.c_size_t, C.POINTER(mph), C.c_size_t,
                                         C.c_int, C.POINTER(var_mph), C.c_size_t]),
    "d2_labeling": (C.c_size_t, [C.POINTER(mph), C.POINTER(mph), C.POINTER(var_mph), C.c_int]),
    "d2g_clustering": (C.c_int, [C.c_int, C.c_int, C.POINTER(mph), C.POINTER(mph), C.c_int, C.c_int,
                                 C.c_char_p, C.POINTER(C.c_int)]),
    "d2g_assignment": (C.c_int, [C.c_int, C.POINTER(mph), C.POINTER(mph), C.c_int,
                                 C.POINTER(C.c_size_t)]),
    "d2_clustering": (C.c_int, [C.c_int, C.c_int, C.POINTER(mph), C.POINTER(mph), C.c_int, C.c_char,
                                C.c_char_p]),
    "d2_labeling_prep": (C.c_size_t, [C.POINTER(mph), C.POINTER(mph), C.POINTER(var_mph), C.c_int]),
    "d2_labeling_post": (C.c_size_t, [C.POINTER(mph), C.POINTER(mph), C.POINTER(mph),
                                      C.POINTER(var_mph), C.c_int]),
    "d2g_phase_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(d2g_tuning)]),
    "d2g_phase_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(d2g_tuning)]),
    "d2g_phase_autotune": (C.c_int, [C.c_void_p, C.POINTER(d2g_badmm_opts), C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "d2g_server_create": (C.c_int, [C.POINTER(d2g_server_desc), C.POINTER(C.c_void_p)]),
    "d2g_server_destroy": (C.c_int, [C.c_void_p]),
    "d2g_server_submit": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_longlong)]),
    "d2g_server_progress": (C.c_int, [C.c_void_p, C.c_int]),
    "d2g_server_result": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_int), C.c_void_p,
                                    C.POINTER(C.c_double)]),
}
DATA_SYMBOLS = ("badmm_clu_options", "badmm_cen_options", "p_badmm_options", "time_budget",
                "d2_alg_type")

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libd2g.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with d2_kmeans_gb300.build.build()")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            if hasattr(lib, name):
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
        _lib = lib
    return _lib


class D2GError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = load()
        msg = lib.d2g_last_error().decode()
        super().__init__(f"{where}: {lib.d2g_error_string(code).decode()} ({code}): {msg}")
        self.code = code


def check(code: int, where: str) -> int:
    if code != 0:
        raise D2GError(code, where)
    return code
