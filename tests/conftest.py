import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "haploadmixture.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def O():
    from oracle import oracle as orc
    orc.load()
    return orc


@pytest.fixture(scope="session")
def built_lib():
    """Builds libhaplo_gb300.so in-tree if needed and returns its path."""
    import build_ext
    return build_ext.build()


@pytest.fixture(scope="session")
def hx(built_lib):
    import haplo_gb300
    haplo_gb300.load()
    return haplo_gb300


def small_cohort(I, J, K, seed=7, alpha=0.5, miss=0.02, pmode="dirichlet", extra_snps=0):
    """Parameters and oracle-generated BED bytes of a small synthetic cohort."""
    from oracle import oracle as orc
    from haplo_gb300 import synth
    Q, P = synth.draw_params(I, J, K, alpha, pmode, seed)
    cq, cp = synth.cumulative(Q, P)
    bed = orc.synth(seed, I, J, cq, cp, miss)
    if extra_snps:
        rng = np.random.default_rng(seed + 99)
        extra = rng.integers(0, 256, size=(extra_snps, bed.shape[1]), dtype=np.uint8)
        if I % 4:
            extra[:, -1] &= (1 << (2 * (I % 4))) - 1
        bed = np.vstack([bed, extra])
    return dict(I=I, J=J, K=K, Q=Q, P=P, bed=bed, seed=seed, miss=miss)
