"""haplo_gb300: GB300 (sm_103a) HaploADMIXTURE fitting path behind a C ABI.

The compute path is libhaplo_gb300.so (hand-written CUDA for sm_103a); this
package is the host-side mirror of the reference's Julia entry points.
"""
from ._lib import load, HxError, HX_KMAX, HX_QMAX, LIB_PATH  # noqa: F401
from .admix import GB300Admix, random_init, run_admixture  # noqa: F401
from . import bed, synth, sweep, skfr  # noqa: F401

__all__ = ["GB300Admix", "random_init", "run_admixture", "bed", "synth", "sweep", "skfr", "load", "HxError"]
