"""Tensor-core (tcgen05) Hessian/gradient passes of the mixed method against
the FP64 oracle, for every supported K, on ragged shapes (I not a multiple of
the 128-row tile, J not a multiple of the 16-block stage) and multi-chunk
splits.  Tolerances (relative to the largest entry): gradient 1e-6 (FP16 hi/lo
operands, 22 significant bits), Hessian 1e-4 (BF16 hi/lo, 16 bits), both
accumulated in FP32.
"""
import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def make(hx, c, **kw):
    return hx.GB300Admix(c["bed"], c["I"], c["J"], c["K"], bytes_per_snp=c["bed"].shape[1],
                         n_snp=c["bed"].shape[0], **kw)


def start(c, seed=3):
    from haplo_gb300.admix import random_init
    return random_init(c["I"], c["J"], c["K"], np.random.default_rng(seed))


@pytest.mark.parametrize("K", list(range(1, 13)))
def test_tc_accumulations_all_K(hx, O, K):
    c = small_cohort(300, 75, K, seed=200 + K, miss=0.05)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = start(c, seed=K)
    d = make(hx, c, precision="mixed")
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = O.accum_q(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = O.accum_p(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4


@pytest.mark.parametrize("I,J,K", [(1, 1, 2), (64, 16, 3), (129, 17, 4), (2000, 3001, 5)])
def test_tc_edge_shapes(hx, O, I, J, K):
    c = small_cohort(I, J, K, seed=I + J, miss=0.03)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = start(c)
    d = make(hx, c, precision="mixed")
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = O.accum_q(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = O.accum_p(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4


def test_tc_matches_cuda_core_mixed_path(hx, coh_tc):
    c = coh_tc
    q, p = start(c)
    a = make(hx, c, precision="mixed")
    b = make(hx, c, precision="mixed", path="cuda_cores")
    for fa, fb in ((a.update_q_accum, b.update_q_accum), (a.update_p_accum, b.update_p_accum)):
        Xa, za = fa(q, p)
        Xb, zb = fb(q, p)
        assert rel_err(za, zb) < 1e-5 and rel_err(Xa, Xb) < 1e-4


def test_tc_passes_are_deterministic(hx, coh_tc):
    c = coh_tc
    q, p = start(c)
    d = make(hx, c, precision="mixed")
    X1, z1 = d.update_p_accum(q, p)
    X2, z2 = d.update_p_accum(q, p)
    assert np.array_equal(X1, X2) and np.array_equal(z1, z2)


def test_tc_fit_reaches_fp64_optimum(hx, O):
    c = small_cohort(400, 300, 3, seed=21, alpha=0.5, miss=0.01)
    q0, p0 = start(c, seed=1)
    out = {}
    for prec in ("fp64", "mixed"):
        d = make(hx, c, precision=prec)
        d.set_qp(q0, p0)
        info = d.fit(n_iter=3000, rtol=1e-14, em_iters=5)
        out[prec] = (info, d.get_qp()[0])
    print("ll mixed %.12g fp64 %.12g  max|dQ| %.3g" % (out["mixed"][0]["ll"], out["fp64"][0]["ll"],
                                                      np.abs(out["mixed"][1] - out["fp64"][1]).max()))
    assert out["mixed"][0]["ll"] == pytest.approx(out["fp64"][0]["ll"], rel=5e-9)
    assert np.abs(out["mixed"][1] - out["fp64"][1]).max() < 2e-5


@pytest.fixture(scope="module")
def coh_tc():
    return small_cohort(1000, 500, 6, seed=77, miss=0.02)


def test_autotune_keeps_the_sums(hx, O):
    """hx_autotune picks grid splits by timing; the sums it leaves behind are
    the tensor-core pass's to the same bounds (gradient 1e-6, Hessian 1e-4,
    log-likelihood 1e-8), and a later context of the same shape runs with
    them (its sums equal the tuned context's bit for bit)."""
    from haplo_gb300.admix import random_init
    c = small_cohort(2304, 901, 5, seed=77)      # a shape no other test uses
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(8))
    d = make(hx, c, precision="mixed")
    d.set_qp(q, p)
    chunks = d.autotune()
    assert len(chunks) == 3 and min(chunks) >= 1
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = O.accum_q(b, c["K"], q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4
    XtXp, Xtzp = d.update_p_accum(q, p)
    oXp, ozp = O.accum_p(b, c["K"], q, p)
    assert rel_err(Xtzp, ozp) < 1e-6 and rel_err(XtXp, oXp) < 1e-4
    assert d.loglikelihood(q, p) == pytest.approx(O.loglik(b, c["K"], q, p), rel=1e-8)
    d2 = make(hx, c, precision="mixed")
    X2, z2 = d2.update_q_accum(q, p)
    np.testing.assert_array_equal(X2, XtX)
    np.testing.assert_array_equal(d2.update_p_accum(q, p)[1], Xtzp)
