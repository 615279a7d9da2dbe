"""Synthetic admixed cohorts of the benchmark shapes.

No public dataset is used: seeded synthetic cohorts of the named shapes stand
in.  Parameters are drawn on the host with numpy (PCG64); genotypes are drawn
by a counter-based SplitMix64 stream, either on the GPU
(hx_synth_bed_device) or by the CPU oracle, and the two agree bit for bit.

Generator (per individual i and two-SNP block j): two haplotype copies, each
with ancestry z ~ Categorical(Q_i) and haplotype h ~ Categorical(P_{z,j}) over
{00, 01, 10, 11}; genotypes are the per-SNP allele counts; each (i, SNP) is
set missing (code 0b01) with probability `miss`.
"""
import ctypes as C

import numpy as np

from . import _lib

BASE_SEED = 20261203

# name: I, J (two-SNP blocks), K, Dirichlet alpha of Q, missing rate, P mode
CONFIGS = {
    "C1": dict(I=1000, J=1000, K=3, alpha=0.5, miss=0.005, pmode="dirichlet", seed=BASE_SEED + 1),
    "C2": dict(I=10000, J=50000, K=5, alpha=0.5, miss=0.01, pmode="shared", seed=BASE_SEED + 2),
    "C3": dict(I=100000, J=100000, K=8, alpha=0.3, miss=0.01, pmode="dirichlet", seed=BASE_SEED + 3),
    "C4": dict(I=20000, J=20000, K=6, alpha=0.5, miss=0.01, pmode="dirichlet", seed=BASE_SEED + 4),
    "C5": dict(I=200000, J=100000, K=6, alpha=0.2, miss=0.01, pmode="dirichlet", seed=BASE_SEED + 5),
}

TWO53 = float(2 ** 53)


def draw_params(I, J, K, alpha, pmode="dirichlet", seed=0, mix=0.2):
    """True Q (K x I) and P (K x 4J) of a cohort.

    pmode 'dirichlet': p_kj ~ Dir(1,1,1,1); 'shared': p_kj = (1-mix) pbar_j +
    mix Dir(1,1,1,1) with pbar_j ~ Dir(1,1,1,1) (low differentiation)."""
    rng = np.random.default_rng(seed)
    Q = rng.dirichlet(np.full(K, alpha), size=I).T            # K x I
    if pmode == "dirichlet":
        P = rng.dirichlet(np.ones(4), size=(K, J))             # K x J x 4
    elif pmode == "shared":
        pbar = rng.dirichlet(np.ones(4), size=J)               # J x 4
        noise = rng.dirichlet(np.ones(4), size=(K, J))
        P = (1.0 - mix) * pbar[None, :, :] + mix * noise
    else:
        raise ValueError(pmode)
    return np.asfortranarray(Q), np.asfortranarray(P.reshape(K, 4 * J))


def cumulative(Q, P):
    """Cumulative probabilities in generator order: cumQ (K x I) over k,
    cumP (K x 4J) over the haplotypes of each (k, block) quartet."""
    K, I = Q.shape
    J = P.shape[1] // 4
    cumQ = np.cumsum(Q, axis=0)
    cumP = np.cumsum(P.reshape(K, J, 4), axis=2).reshape(K, 4 * J)
    return np.asfortranarray(cumQ), np.asfortranarray(cumP)


def thresholds(cum):
    """Integer thresholds ceil(cum * 2^53): for a 53-bit draw n,
    n < ceil(c 2^53)  <=>  n 2^-53 < c."""
    return np.asfortranarray(np.ceil(cum * TWO53).astype(np.uint64))


def synth_device(seed, Q, P, miss, d_bed_addr, device=0):
    """Fills device memory at d_bed_addr (ceil(I/4) * 2J bytes) with the BED
    matrix of the cohort."""
    K, I = Q.shape
    J = P.shape[1] // 4
    cumQ, cumP = cumulative(Q, P)
    tQ, tP = thresholds(cumQ), thresholds(cumP)
    _lib.check(_lib.load().hx_synth_bed_device(seed, I, J, K, _lib.ptr(tQ), _lib.ptr(tP), miss,
                                               C.c_void_p(d_bed_addr), device))


def config(name, **sizes):
    """Named synthetic workload; `sizes` (I, J, K) overrides give a smaller
    case of the same generator, used for profiling captures."""
    c = dict(CONFIGS[name])
    c.update({k: int(v) for k, v in sizes.items() if v})
    Q, P = draw_params(c["I"], c["J"], c["K"], c["alpha"], c["pmode"], c["seed"])
    c["Q"], c["P"] = Q, P
    c["bps"] = (c["I"] + 3) // 4
    c["n_snp"] = 2 * c["J"]
    return c
