"""The two benchmark configurations small enough for the CPU oracle, at their
own shapes (seeded synthetic cohorts; no public dataset is used).

C1, plain method: I = 1,000 individuals x 2,000 SNPs (1,000 blocks), K = 3,
Q ~ Dirichlet(0.5), P ~ Dirichlet(1,1,1,1), 0.5% missing.  The FP64 GPU fit
(init_em! + admixture_qn! at rtol 1e-7) equals the oracle's fit from the
same start: log-likelihood within 1e-9 relative, Q and P within 1e-5,
outer iterations within one.  The mixed method, run to convergence from the
same start, reaches the FP64 optimum within 1e-8 in log-likelihood and 1e-5
in Q (the accuracy bar of the chosen method).

C2, plain method against the FP64 oracle: I = 10,000 x 100,000 SNPs (50,000
blocks), K = 5, P = 0.8 shared ancestral + 0.2 Dirichlet noise, 1% missing,
Q uniform with random jitter.  Census and double-missing counts bit-exact;
log-likelihood, Q and P gradients and Hessians within 1e-10 relative (to the
largest entry) at identical Q, P.  The tensor-core passes of the mixed method
at the same point: Hessian 1e-4, gradient 2e-6.  The gradient bound is the
accumulation bias of the tensor core: each TMEM window takes 16 MMA adds per
column (8 stages x 2 k-steps) before it is folded, and every add rounds the
FP32 accumulator toward zero, up to 2^-23 of it: 16 x 2^-23 = 1.9e-6 (the
measured error here is about 1.1e-6, all of one sign).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _cohort(O, name):
    from haplo_gb300 import synth
    cfg = synth.config(name)
    cq, cp = synth.cumulative(cfg["Q"], cfg["P"])
    bed = O.synth(cfg["seed"], cfg["I"], cfg["J"], cq, cp, cfg["miss"])
    return cfg, bed


def _make(hx, cfg, bed, precision):
    return hx.GB300Admix(bed, cfg["I"], cfg["J"], cfg["K"], bytes_per_snp=bed.shape[1], n_snp=bed.shape[0],
                         precision=precision)


def test_c1_fp64_fit_matches_oracle_fit(hx, O):
    from haplo_gb300.admix import random_init
    cfg, bed = _cohort(O, "C1")
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    assert (I, J, K) == (1000, 1000, 3)
    b = O.Bed(bed, I, J)
    q0, p0 = random_init(I, J, K, np.random.default_rng(cfg["seed"] + 7))
    qo, po, llo, ito, _ = O.fit(b, K, q0, p0, n_iter=1000, rtol=1e-7, em_iters=5)
    d = _make(hx, cfg, bed, "fp64")
    d.set_qp(q0, p0)
    info = d.fit(n_iter=1000, rtol=1e-7, em_iters=5)
    qd, pd = d.get_qp()
    d.close()
    assert info["converged"]
    assert info["ll"] == pytest.approx(llo, rel=1e-9)
    assert abs(info["iters"] - ito) <= 1
    assert np.abs(qd - qo).max() < 1e-5
    assert np.abs(pd - po).max() < 1e-5


def test_c1_mixed_reaches_fp64_optimum(hx, O):
    from haplo_gb300.admix import random_init
    cfg, bed = _cohort(O, "C1")
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    q0, p0 = random_init(I, J, K, np.random.default_rng(cfg["seed"] + 7))
    out = {}
    for prec in ("fp64", "mixed"):
        d = _make(hx, cfg, bed, prec)
        d.set_qp(q0, p0)
        info = d.fit(n_iter=3000, rtol=1e-13, em_iters=5)
        out[prec] = (info["ll"], d.get_qp()[0])
        d.close()
    assert out["mixed"][0] == pytest.approx(out["fp64"][0], rel=1e-8)
    assert np.abs(out["mixed"][1] - out["fp64"][1]).max() < 1e-5


@pytest.fixture(scope="module")
def c2(hx, O):
    cfg, bed = _cohort(O, "C2")
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    assert (I, J, K) == (10000, 50000, 5)
    rng = np.random.default_rng(cfg["seed"] + 11)
    q = np.full((K, I), 1.0 / K) * (1.0 + 0.1 * rng.random((K, I)))        # uniform with random jitter
    q = np.asfortranarray(q / q.sum(axis=0, keepdims=True))
    p = rng.random((K, J, 4))
    p = np.asfortranarray((p / p.sum(axis=2, keepdims=True)).reshape(K, 4 * J))
    b = O.Bed(bed, I, J)
    # the oracle's sums at this point, once for both precisions
    ref = dict(ll=O.loglik(b, K, q, p), q=O.accum_q(b, K, q, p), p=O.accum_p(b, K, q, p))
    return dict(cfg=cfg, bed=bed, b=b, q=q, p=p, ref=ref)


def test_c2_census_and_double_missing_bit_exact(hx, O, c2):
    d = _make(hx, c2["cfg"], c2["bed"], "fp64")
    census = d.census()
    np.testing.assert_array_equal(census, O.census(c2["b"]))
    assert int(census.sum()) == c2["cfg"]["I"] * c2["cfg"]["J"]
    np.testing.assert_array_equal(d.double_missing(), O.double_missing(c2["b"]))
    d.close()


def test_c2_fp64_loglik_gradient_hessian(hx, O, c2):
    q, p, ref = c2["q"], c2["p"], c2["ref"]
    d = _make(hx, c2["cfg"], c2["bed"], "fp64")
    assert d.loglikelihood(q, p) == pytest.approx(ref["ll"], rel=1e-10)
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = ref["q"]
    assert rel_err(Xtz, oz) < 1e-10 and rel_err(XtX, oX) < 1e-10
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = ref["p"]
    assert rel_err(Xtz, oz) < 1e-10 and rel_err(XtX, oX) < 1e-10
    d.close()


def test_c2_mixed_tensor_core_passes(hx, O, c2):
    q, p, ref = c2["q"], c2["p"], c2["ref"]
    d = _make(hx, c2["cfg"], c2["bed"], "mixed")
    assert d.loglikelihood(q, p) == pytest.approx(ref["ll"], rel=1e-8)
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = ref["q"]
    assert rel_err(Xtz, oz) < 2e-6 and rel_err(XtX, oX) < 1e-4
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = ref["p"]
    assert rel_err(Xtz, oz) < 2e-6 and rel_err(XtX, oX) < 1e-4
    d.close()
