import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: runs the CUDA path on a GB300 (libd2g.so)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    if not oracle.available("port") or (
            not oracle.available("reference") and os.path.isdir(oracle.REF_TREE)):
        oracle.build()
    return oracle


@pytest.fixture(scope="session")
def d2g():
    """The product: libd2g.so through its Python mirror (built if missing)."""
    from d2_kmeans_gb300.build import build as build_lib
    from d2_kmeans_gb300 import badmm
    build_lib()
    badmm.set_config(verbose=0, precision=0, use_graph=1, profile=0, sync_scratch=0, cost_gemm=0)
    return badmm


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    """(phase, c0, opts, expected) of one fixture written by make_golden.py."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    ph = {}
    for k in z.files:
        if k.startswith("in_"):
            ph[k[3:]] = z[k]
        elif k.startswith("meta_"):
            ph[k[5:]] = z[k].item()
    c0 = {"c_w": z["c0_w"], "c_supp": z["c0_supp"] if "c0_supp" in z.files else None}
    if "c0_sym" in z.files:
        c0["c_sym"] = z["c0_sym"]
    o = z["opts"]
    opts = dict(maxIters=int(o[0]), rhoCoeff=float(o[1]), updatePerLoops=int(o[2]))
    exp = {k: z[k] for k in z.files if k.startswith("out_") or k.startswith("first_")}
    return ph, c0, opts, exp


def digest(zv):
    from golden.make_golden import digest as d
    return d(zv)


# A stand-in for the reference's d2_centroid_rands (src/d2/centroid_rand.c:161-295)
# with a fixed, easily restated choice: the first num_of_labels instances whose
# support size equals the centroid's, copied in order; like the reference it
# also sets the centroids' strides and column count (:176-182).  The drop-in
# finds it by dlsym once it is loaded into the global scope.
RANDS_STUB = r"""
#include "d2g.h"
int d2_centroid_rands(mph *p, int idx, sph *c) {
  sph *ph = p->ph + idx;
  int K = p->num_of_labels, m = c->str, d = ph->dim, j = 0;
  for (int l = 0; l < K; ++l) {
    c->p_str[l] = m;
    c->p_str_cum[l] = (size_t)l * m;
  }
  c->col = (size_t)m * K;
  for (size_t i = 0; i < p->size && j < K; ++i) {
    if (ph->p_str[i] != m) continue;
    size_t o = ph->p_str_cum[i];
    for (int k = 0; k < m; ++k) {
      c->p_w[j * m + k] = ph->p_w[o + k];
      for (int t = 0; t < d; ++t) c->p_supp[(j * m + k) * d + t] = ph->p_supp[(o + k) * d + t];
    }
    ++j;
  }
  return 0;
}
"""


def rands_stub_init(ph, k, m):
    """What RANDS_STUB writes into c (numpy)."""
    p_str = np.asarray(ph["p_str"])
    cum = np.concatenate([[0], np.cumsum(p_str)])
    d = int(ph["dim"])
    sel = np.nonzero(p_str == m)[0][:k]
    assert sel.size == k
    w = np.concatenate([ph["p_w"][cum[i]:cum[i] + m] for i in sel])
    s = np.concatenate([np.asarray(ph["p_supp"]).reshape(-1, d)[cum[i]:cum[i] + m] for i in sel])
    return {"c_w": w, "c_supp": s.reshape(-1)}


@pytest.fixture(scope="session")
def rands_stub(tmp_path_factory):
    """RANDS_STUB compiled with gcc and loaded with RTLD_GLOBAL."""
    import ctypes
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc is not present")
    d = tmp_path_factory.mktemp("rands")
    src, so = d / "rands.c", d / "librands.so"
    src.write_text(RANDS_STUB)
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"), "-o", str(so),
                    str(src)], check=True)
    return ctypes.CDLL(str(so), mode=ctypes.RTLD_GLOBAL)
