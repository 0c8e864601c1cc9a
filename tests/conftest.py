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
    o = z["opts"]
    opts = dict(maxIters=int(o[0]), rhoCoeff=float(o[1]), updatePerLoops=int(o[2]))
    exp = {k: z[k] for k in z.files if k.startswith("out_") or k.startswith("first_")}
    return ph, c0, opts, exp


def digest(zv):
    from golden.make_golden import digest as d
    return d(zv)
