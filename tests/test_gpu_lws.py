"""Learned warm start on the GPU: features, network forward and gradient
against the FP64 restatement (weights rounded to FP16 on both sides), the
training kernels, and the warm-started fit against the plain fit."""
import os

import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from oracle import lws_oracle
    return lws_oracle


def test_features_match_oracle(hx, O, L):
    from haplo_gb300 import lws
    from haplo_gb300.admix import random_init
    c = small_cohort(300, 90, 4, seed=23, miss=0.02)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = random_init(c["I"], c["J"], 4, np.random.default_rng(4))
    d = hx.GB300Admix(c["bed"], c["I"], c["J"], 4, precision="mixed")
    d.set_qp(q, p)
    fg = lws.features(d)
    fo = L.features(b, 4, q, p)
    assert np.abs(fg[:, :, 0] - fo[:, :, 0]).max() < 2e-5      # FP32 renormalised products
    # f2 = (g - 1) sqrt(n): the mixed gradient's 1e-5 relative error, times sqrt(n)
    assert np.abs(fg[:, :, 1] - fo[:, :, 1]).max() < 1e-4 * np.sqrt(c["J"])


def test_forward_and_gradient_match_oracle(hx, L):
    from haplo_gb300 import lws
    rng = np.random.default_rng(1)
    for K in (2, 6, 12):
        n = 300
        feat = np.stack([-np.abs(rng.normal(0, 0.3, (n, K))), rng.gamma(2.0, 0.5, (n, K))], axis=2)
        t = rng.dirichlet(np.ones(K) * 0.5, size=n)
        params = lws.init_params(K)
        params[lws._O["b1"][0]:lws._O["b1"][0] + 64] = rng.normal(0, 0.3, 64)
        qg = lws.forward(feat, params)
        qo, _ = L.forward(feat, params)
        assert np.abs(qg - qo).max() < 2e-5
        lg, gg = lws.grad(feat, t, params)
        lo, go = L.loss_grad(feat, t, params)
        assert lg == pytest.approx(lo, rel=1e-5)
        assert np.abs(gg - go).max() < 2e-4 * np.abs(go).max()


def test_training_reduces_the_loss_and_is_reproducible(hx):
    from haplo_gb300 import lws
    rng = np.random.default_rng(2)
    n, K = 20000, 5
    feat = np.stack([-np.abs(rng.normal(0, 0.5, (n, K))), rng.gamma(2.0, 0.5, (n, K))], axis=2).astype(np.float32)
    z = 3.0 * feat[:, :, 0] + feat[:, :, 1]
    t = np.exp(z - z.max(axis=1, keepdims=True))
    t /= t.sum(axis=1, keepdims=True)
    p1, l1 = lws.train(feat, t, steps=300, batch=2048, lr=3e-3, seed=9)
    p2, l2 = lws.train(feat, t, steps=300, batch=2048, lr=3e-3, seed=9)
    np.testing.assert_array_equal(p1, p2)
    # the cross-entropy is bounded below by the targets' entropy: the excess
    # over it must shrink
    ent = -(t * np.log(t)).sum(axis=1).mean()
    assert np.mean(l1[-20:]) - ent < 0.5 * (np.mean(l1[:5]) - ent)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                    "haploadmixture.jl_gb300", "haplo_gb300", "lws_params.npy")),
                    reason="trained parameters not present")
def test_warm_started_fit_reaches_the_plain_optimum(hx):
    """Held-out cohort (seed outside the training set): the chosen fit (with the
    warm start) and the plain mixed fit converge to the same log-likelihood;
    the iteration counts of both are reported."""
    from haplo_gb300 import lws, synth
    from haplo_gb300.admix import random_init
    I, J, K = 6000, 2000, 6
    Q, P = synth.draw_params(I, J, K, 0.2, "dirichlet", 777)
    cq, cp = synth.cumulative(Q, P)
    from oracle import oracle as O
    bed = O.synth(778, I, J, cq, cp, 0.01)
    q0, p0 = random_init(I, J, K, np.random.default_rng(779))
    plain = hx.GB300Admix(bed, I, J, K, precision="mixed")
    plain.set_qp(q0, p0)
    ip = plain.fit(n_iter=500, rtol=1e-9, em_iters=5)
    chosen = hx.GB300Admix(bed, I, J, K, precision="mixed")
    chosen.set_qp(q0, p0)
    ic = lws.fit(chosen, n_iter=500, rtol=1e-9, em_iters=5)
    print("plain iters %d ll %.10e %.3f s | warm start accepted %s iters %d ll %.10e %.3f s"
          % (ip["iters"], ip["ll"], ip["seconds"], ic["warm_start_accepted"], ic["iters"], ic["ll"], ic["seconds"]))
    assert ic["ll"] == pytest.approx(ip["ll"], rel=1e-8)
