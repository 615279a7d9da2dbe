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


PARAMS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "haploadmixture.jl_gb300",
                      "haplo_gb300", "lws_params.npy")


def _xent(pred, target):
    return float(-np.mean(np.sum(target * np.log(np.clip(pred, 1e-12, None)), axis=1)))


@pytest.mark.skipif(not os.path.exists(PARAMS), reason="trained parameters not present")
def test_network_gain_as_a_predictor(hx):
    """What the trained network gains, on held-out cohorts (seeds outside the
    training set), where the warm start applies (after init_em! and one outer
    iteration): its Q is closer to the converged Q (cross-entropy, converged
    rows put in the labelling of that point) than the uniform Q is, by at
    least 0.02 nats.  The cross-entropy of the fit's own Q at that point is
    reported beside it."""
    from haplo_gb300 import lws
    qnow = []
    X, T = lws.training_set(cohorts=3, I=20000, J=5000, K=6, seed=4242, plain_iters=1, q_now_out=qnow)
    pred = lws.forward(X, lws.load_params())
    x_net, x_uni = _xent(pred, T), _xent(np.full_like(T, 1.0 / T.shape[1]), T)
    x_cur, x_floor = _xent(np.concatenate(qnow), T), _xent(T, T)
    print("cross-entropy vs converged Q: network %.4f, uniform %.4f, current Q %.4f, targets' entropy %.4f"
          % (x_net, x_uni, x_cur, x_floor))
    assert x_net < x_uni - 0.02


@pytest.mark.skipif(not os.path.exists(PARAMS), reason="trained parameters not present")
def test_warm_started_fit_reaches_the_plain_optimum(hx):
    """Held-out cohort: the warm-started fit ends at the plain mixed fit's
    log-likelihood or above it (within 1e-8 relative; the fit maximises it);
    the iteration counts and times of both are reported."""
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
    assert ic["ll"] >= ip["ll"] - 1e-8 * abs(ip["ll"])
