"""hx_loglikelihood_noalloc: the log-likelihood entry point that allocates no
device memory, for callers that cannot allocate at call time (frameworks that
own the whole device memory pool, latency-critical loops where cudaMalloc
would synchronise the device).  Called through the C ABI on caller-owned
device buffers and checked against the existing entry point
(hx_loglikelihood on a context) to 1e-12 relative in FP64 and 1e-9 in the
mixed method, on two calls in a row with different inputs, so that the
scratch left by the first call cannot leak into the second.

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


def _reference_ll(hx, c, q, p, precision):
    d = hx.GB300Admix(c["bed"], c["I"], c["J"], c["K"], bytes_per_snp=c["bed"].shape[1],
                      n_snp=c["bed"].shape[0], precision=precision)
    try:
        return d.loglikelihood(q, p)
    finally:
        d.close()


def _device_inputs(c, q, p):
    import torch
    dev = torch.device("cuda", 0)
    bed = torch.from_numpy(np.ascontiguousarray(c["bed"])).to(dev)
    dq = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(q).T)).to(dev)      # column-major K x I
    dp = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(p).T)).to(dev)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    return bed, dq, dp, out


def _call(lib, c, bed, dq, dp, out, prec, stream):
    return lib.hx_loglikelihood_noalloc(C.c_void_p(bed.data_ptr()), c["bed"].shape[1], c["I"], c["J"], c["K"],
                                        C.c_void_p(dq.data_ptr()), C.c_void_p(dp.data_ptr()), prec,
                                        C.c_void_p(out.data_ptr()), stream)


def _noalloc_ll(hx, c, q, p, precision, stream=None):
    import torch
    from haplo_gb300 import _lib
    lib = hx.load()
    bed, dq, dp, out = _device_inputs(c, q, p)
    prec = {"fp64": _lib.HX_PREC_FP64, "mixed": _lib.HX_PREC_MIXED}[precision]
    torch.cuda.synchronize()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    st = _call(lib, c, bed, dq, dp, out, prec, handle)
    assert st == _lib.HX_OK, lib.hx_status_string(st)
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return float(out.item())


@pytest.mark.parametrize("precision,rel", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_noalloc_matches_context_entry_point_two_calls(hx, precision, rel):
    from haplo_gb300.admix import random_init
    c1 = small_cohort(777, 301, 4, seed=31, miss=0.03)
    c2 = small_cohort(129, 57, 6, seed=32, miss=0.05)
    for c, seed in ((c1, 1), (c2, 2)):
        q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(seed))
        want = _reference_ll(hx, c, q, p, precision)
        got = _noalloc_ll(hx, c, q, p, precision)
        assert got == pytest.approx(want, rel=rel)


@pytest.mark.parametrize("precision,rel", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_noalloc_on_caller_stream(hx, precision, rel):
    """The kernels are enqueued on the caller's stream (a torch stream here),
    and a call leaves the free device memory unchanged."""
    import torch
    from haplo_gb300 import _lib
    from haplo_gb300.admix import random_init
    c = small_cohort(515, 203, 5, seed=33, miss=0.02)
    q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(3))
    want = _reference_ll(hx, c, q, p, precision)
    s = torch.cuda.Stream()
    assert _noalloc_ll(hx, c, q, p, precision, stream=s) == pytest.approx(want, rel=rel)
    # after a first call (module loaded), further calls allocate nothing
    lib = hx.load()
    bed, dq, dp, out = _device_inputs(c, q, p)
    prec = {"fp64": _lib.HX_PREC_FP64, "mixed": _lib.HX_PREC_MIXED}[precision]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, c, bed, dq, dp, out, prec, C.c_void_p(s.cuda_stream)) == _lib.HX_OK
    s.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert float(out.item()) == pytest.approx(want, rel=rel)


def test_noalloc_mixed_tiny_pair_likelihoods(hx):
    """Q/P entries far below the fit's 1e-5 floor give FP32 pair likelihoods
    below the smallest normal float; the mixed method still matches FP64."""
    from haplo_gb300.admix import random_init
    c = small_cohort(260, 40, 3, seed=34, miss=0.02)
    q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(4))
    p = p.copy()
    # block 0: haplotype 00 nearly impossible in every population
    p[:, 0] = 1e-22
    p[:, 1:4] /= p[:, 1:4].sum(axis=1, keepdims=True) / (1 - 1e-22)
    want = _reference_ll(hx, c, q, p, "fp64")
    got = _noalloc_ll(hx, c, q, p, "mixed")
    assert np.isfinite(got)
    assert got == pytest.approx(want, rel=1e-7)


def test_noalloc_rejects_sizes_beyond_scratch(hx):
    from haplo_gb300 import _lib
    lib = hx.load()
    # I beyond 128 * HX_NOALLOC_SCRATCH individuals is refused before any device work
    big_I = 128 * 32768 + 1
    st = lib.hx_loglikelihood_noalloc(C.c_void_p(1), (big_I + 3) // 4, big_I, 1, 2, C.c_void_p(1), C.c_void_p(1),
                                      _lib.HX_PREC_FP64, C.c_void_p(1), None)
    assert st == _lib.HX_EUNSUPPORTED
