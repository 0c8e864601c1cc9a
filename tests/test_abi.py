"""The C ABI on the CPU: libd2g.so loads (no GPU needed), exports every
function and data symbol include/*.h declares, the header compiles as C, and
the reference-compatible structures have the reference's layout."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from d2_kmeans_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
import oracle  # noqa: E402

REF_INCLUDE = os.path.join(oracle.REF_TREE, "include")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        txt = re.sub(r"\btypedef\b[^;{]*;", "", txt)  # function-pointer types are not functions
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", txt, re.M):
            if m.group(1) not in ("if", "while", "for", "return", "sizeof"):
                names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from d2_kmeans_gb300.build import build
    build()
    return L.load()


def test_every_declared_function_is_exported(lib):
    names = declared_functions()
    assert {"d2_centroid_sphBregman", "d2_allocate_work_sphBregman", "d2_free_work_sphBregman",
            "calculate_distmat", "d2g_phase_create", "d2g_badmm_run"} <= names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python bindings cover every declared function
    assert names <= set(L.SIGNATURES), sorted(names - set(L.SIGNATURES))


def test_data_symbols_and_defaults(lib):
    for n in L.DATA_SYMBOLS:
        assert hasattr(lib, n), n
    clu = L.BADMM_options.in_dll(lib, "badmm_clu_options")
    cen = L.BADMM_options.in_dll(lib, "badmm_cen_options")
    # src/d2/centroid_Bregman.c:17-18
    assert (clu.maxIters, clu.rhoCoeff, clu.updatePerLoops) == (100, 2.0, 10)
    assert (cen.maxIters, cen.rhoCoeff, cen.updatePerLoops) == (2000, 1.0, 10)
    assert C.c_double.in_dll(lib, "time_budget").value > 1e200


def test_error_strings_and_config_roundtrip(lib):
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert lib.d2g_error_string(code)
    cfg = L.d2g_config()
    assert lib.d2g_get_config(C.byref(cfg)) == 0
    bad = L.d2g_config(7, 1, 1, 0, 0, 0)
    assert lib.d2g_set_config(C.byref(bad)) == L.D2G_E_INVAL
    assert lib.d2g_set_config(C.byref(cfg)) == 0


def test_invalid_phase_is_rejected_without_a_gpu(lib):
    d = L.d2g_phase_desc()
    h = C.c_void_p()
    assert lib.d2g_phase_create(C.byref(d), 0, C.byref(h)) == L.D2G_E_INVAL
    d.metric_type = L.D2_N_GRAM
    d.size, d.str, d.num_of_labels = 1, 2, 1
    one = (C.c_int * 1)(1)
    w = (C.c_double * 1)(1.0)
    d.p_str, d.p_w, d.label = C.addressof(one), C.addressof(w), C.addressof((C.c_int * 1)(0))
    # an n-gram phase needs its symbols and symbol cost
    assert lib.d2g_phase_create(C.byref(d), 0, C.byref(h)) == L.D2G_E_INVAL
    d.metric_type = 1  # D2_CITYBLOCK_L1: no B-ADMM support update in the reference either
    assert lib.d2g_phase_create(C.byref(d), 0, C.byref(h)) == L.D2G_E_UNSUPPORTED


def test_header_compiles_as_c():
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-x", "c", "-"],
                       input=f'#include "{INCLUDE}/d2g.h"\nint main(void){{return 0;}}\n',
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
%s
#define F(T, f) printf(#T "." #f " %%zu\n", offsetof(T, f));
#define S(T) printf(#T " %%zu\n", sizeof(T));
int main(void) {
  S(sph) F(sph, col) F(sph, p_str) F(sph, p_str_cum) F(sph, p_w) F(sph, metric_type)
  F(sph, p_supp) F(sph, p_supp_sym) F(sph, dist_mat) F(sph, vocab_size) F(sph, vocab_vec)
  F(sph, is_meta_allocated)
  S(mph) F(mph, size) F(mph, global_size) F(mph, label) F(mph, num_of_labels) F(mph, ph)
  S(var_sph) S(var_sphBregman) F(var_sphBregman, Xc) F(var_sphBregman, Zr)
  S(var_mph) F(var_mph, g_var) F(var_mph, l_var_sphBregman) F(var_mph, label_switch) F(var_mph, tr)
  S(trieq) S(BADMM_options) F(BADMM_options, rhoCoeff) F(BADMM_options, updatePerLoops)
  return 0;
}
"""


def _layout(include_line, flags, tmp_path, tag):
    src = tmp_path / f"probe_{tag}.c"
    exe = tmp_path / f"probe_{tag}"
    src.write_text(PROBE % include_line)
    r = subprocess.run(["gcc", "-std=gnu99"] + flags + [str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_struct_layout_matches_the_reference(tmp_path):
    if not os.path.isdir(REF_INCLUDE):
        pytest.skip("reference headers not present on this host")
    ours = _layout(f'#include "{INCLUDE}/d2g.h"', [], tmp_path, "ours")
    ref = _layout('#include "d2/clustering.h"\n#include "d2/param.h"',
                  ["-D_D2_DOUBLE", "-D__BLAS_LEGACY__", f"-I{REF_INCLUDE}"], tmp_path, "ref")
    assert ours == ref


def test_python_struct_mirror_sizes():
    # ctypes mirror of the same structures (used by the Python drop-in path)
    assert C.sizeof(L.BADMM_options) == 24
    assert C.sizeof(L.sph) == C.sizeof(C.c_void_p) * 11 + 16 + 8  # 104 on LP64
    assert C.sizeof(L.mph) == 48
    assert C.sizeof(L.var_sphBregman) == 40


def _small_dropin():
    from d2_kmeans_gb300 import badmm, synth
    ph, c = synth.euclidean_phase(60, 3, 8, 3, (4, 12), False, 5, 1.0, seed=5)
    return ph, badmm.DropIn(ph, c)


def test_random_init_without_rands_uses_the_librarys(lib):
    """c0 == NULL with no d2_centroid_rands in the program: c is filled by
    d2g_centroid_rands (the same result as calling it directly).  Without a
    GPU the update itself then fails with a device error, leaving the
    initialisation in c."""
    import torch
    if hasattr(C.CDLL(None), "d2_centroid_rands"):
        pytest.skip("a d2_centroid_rands is already loaded into this process")
    if torch.cuda.is_available():
        pytest.skip("covered with the update by the GPU tests")
    ph, d = _small_dropin()
    d.c_w[:] = -1.0
    d.c_supp[:] = -1.0
    rc = d.call({}, random_init=True)
    assert rc not in (0, L.D2G_E_UNSUPPORTED, L.D2G_E_INVAL)
    w = np.full(d.c_w.size, np.nan)
    s = np.full(d.c_supp.size, np.nan)
    c = L.sph()
    c.dim, c.str, c.max_str, c.metric_type = d.dim, d.m, d.m, 0
    p_str, cum = np.zeros(d.k, np.int32), np.zeros(d.k, np.uint64)
    c.p_str = p_str.ctypes.data_as(C.POINTER(C.c_int))
    c.p_str_cum = cum.ctypes.data_as(C.POINTER(C.c_size_t))
    c.p_w = w.ctypes.data_as(C.POINTER(C.c_double))
    c.p_supp = s.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.d2g_centroid_rands(C.byref(d.mph), 0, C.byref(c)) == 0
    assert np.array_equal(d.c_w, w) and np.array_equal(d.c_supp, s)
    d.close()


def test_random_init_calls_the_programs_rands(lib, rands_stub):
    """With d2_centroid_rands loaded, c0 == NULL fills c through it first
    (centroid_Bregman.c:95-98).  Without a GPU the update itself then fails
    with a device error, leaving the initialisation in c."""
    import torch
    from conftest import rands_stub_init
    if torch.cuda.is_available():
        pytest.skip("covered with the update by the GPU tests")
    ph, d = _small_dropin()
    d.c_w[:] = -1.0
    d.c_supp[:] = -1.0
    rc = d.call({}, random_init=True)
    assert rc not in (0, L.D2G_E_UNSUPPORTED, L.D2G_E_INVAL)
    exp = rands_stub_init(ph, 3, 8)
    assert np.array_equal(d.c_w, exp["c_w"]) and np.array_equal(d.c_supp, exp["c_supp"])
    d.close()
