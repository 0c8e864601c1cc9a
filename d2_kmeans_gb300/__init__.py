"""d2_kmeans_gb300: GB300-native B-ADMM Wasserstein-barycenter centroid update.

The product is ``libd2g.so`` (hand-written sm_103a CUDA behind the C ABI in
``include/d2g.h``); this package builds it, binds it with ctypes and mirrors
the reference's interface (``badmm.DropIn``, ``badmm.Phase``,
``serve.Server``).  There is no CPU fallback: every entry point raises if the
library is missing or the GPU call fails.
"""
from . import synth  # noqa: F401

__all__ = ["synth", "badmm", "build"]
