"""K sweep with restarts (hx_create_shared + hx_fit_many): every fit equals
the same fit run alone (bit-for-bit: fits are deterministic and share only
read-only genotype classes), and AIC follows its formula."""
import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_k_sweep_equals_sequential_fits(hx, precision):
    from haplo_gb300 import sweep
    from haplo_gb300.admix import random_init
    c = small_cohort(1500, 600, 4, seed=44, alpha=0.5, miss=0.01)
    Ks, restarts, seed = [2, 3, 4, 5], 2, 7
    kw = dict(n_iter=150, rtol=1e-7, em_iters=3)
    rows = sweep.k_sweep(c["bed"], c["I"], c["J"], Ks, restarts=restarts, seed=seed, precision=precision,
                         keep=True, **kw)
    assert [(r["K"], r["restart"]) for r in rows] == [(K, r) for K in Ks for r in range(restarts)]
    for row in rows:
        K = row["K"]
        d = hx.GB300Admix(c["bed"], c["I"], c["J"], K, precision=precision)
        d.set_qp(*random_init(c["I"], c["J"], K, np.random.default_rng(seed + 1000 * K + row["restart"])))
        info = d.fit(**kw)
        q, p = d.get_qp()
        assert row["ll"] == info["ll"] and row["iters"] == info["iters"]
        np.testing.assert_array_equal(row["q"], q)
        np.testing.assert_array_equal(row["p"], p)
        assert row["aic"] == pytest.approx(2 * ((K - 1) * c["I"] + 3 * K * c["J"]) - 2 * info["ll"], rel=1e-15)
        d.close()
    best = {K: max(r["ll"] for r in rows if r["K"] == K) for K in Ks}
    assert best[4] > best[2] and best[3] > best[2]


def test_shared_context_survives_parent_handle_order(hx):
    from haplo_gb300 import sweep
    c = small_cohort(300, 100, 3, seed=9)
    parent = hx.GB300Admix(c["bed"], c["I"], c["J"], 3, precision="mixed")
    child = hx.GB300Admix.shared(parent, 5)
    assert child.K == 5 and child.I == parent.I
    np.testing.assert_array_equal(child.census(), parent.census())
    np.testing.assert_array_equal(child.double_missing(), parent.double_missing())
    del parent                      # the child keeps the parent context alive
    from haplo_gb300.admix import random_init
    child.set_qp(*random_init(c["I"], c["J"], 5, np.random.default_rng(1)))
    assert np.isfinite(sweep.fit_many([child], n_iter=5, rtol=0.0, em_iters=1)[0]["ll"])
    child.close()
