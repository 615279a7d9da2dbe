"""CPU checks of the learned warm start's restatement (oracle/lws_oracle.py):
the network gradient against finite differences, and the feature identity
sum_k q_k f2_k = 1."""
import numpy as np
import pytest

from conftest import small_cohort


@pytest.fixture(scope="module")
def L():
    from oracle import lws_oracle
    return lws_oracle


def test_network_gradient_is_finite_difference(L):
    from haplo_gb300 import lws
    rng = np.random.default_rng(0)
    n, K = 7, 5
    feat = rng.normal(size=(n, K, 2))
    t = rng.dirichlet(np.ones(K), size=n)
    params = lws.init_params(3).astype(np.float64)
    params[lws._O["b1"][0]:lws._O["b1"][0] + 64] = rng.normal(0, 0.3, 64)
    loss, g = L.loss_grad(feat, t, params, round16=False)
    for idx in list(rng.choice(8513, 40, replace=False)) + [8512]:
        e = np.zeros_like(params)
        e[idx] = 1e-6
        fd = (L.loss_grad(feat, t, params + e, round16=False)[0]
              - L.loss_grad(feat, t, params - e, round16=False)[0]) / 2e-6
        assert fd == pytest.approx(g[idx], abs=1e-7 + 1e-5 * abs(g[idx]))


def test_features_gradient_identity(O, L):
    c = small_cohort(60, 25, 3, seed=5)
    b = O.Bed(c["bed"], c["I"], c["J"])
    from haplo_gb300.admix import random_init
    q, p = random_init(c["I"], c["J"], 3, np.random.default_rng(2))
    f = L.features(b, 3, q, p)
    assert np.all(f[:, :, 0] <= 0) and np.allclose(f[:, :, 0].max(axis=1), 0)
    n = (c["J"] - O.double_missing(b)).astype(float)
    g = f[:, :, 1] / np.sqrt(n)[:, None] + 1.0
    np.testing.assert_allclose((q.T * g).sum(axis=1), 1.0, rtol=1e-12)
