"""GB300-native implementation of pMSz's topology-correction hot path.

Given an original 3-D scalar field and its error-bounded decompressed copy, the
path labels steepest ascent/descent directions on the 14-neighbour stencil,
detects false or missing extrema and mislabelled vertices, and runs the
eps-bounded edit loop until the corrected field has the original's extrema and
ascending / descending segmentations (reference: pMSz.cu, c_loops and
iscriticle).  The compute runs in hand-written CUDA kernels for sm_103a behind
the C ABI of include/pmsz.h; this package is its Python face.
"""
from . import _build, capi, fields  # noqa: F401

__all__ = ["build", "capi", "fields"]  # the torch-facing API: pmsz_anonymous_gb300.api


def build() -> str:
    """Compile libpmsz_gb300.so (and the pmsz CLI) for sm_103a."""
    return _build.build()

