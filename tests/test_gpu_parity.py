"""GPU parity: every device pass / solver / step through the C ABI against the
CPU oracle on the same seeded inputs.

Tolerances: integer work (decode, census, double-missing counts, synthetic
genotypes) is bit-exact.  The plain FP64 method agrees with the FP64 oracle to
1e-10 relative (log-likelihood, gradient, Hessian; scale = largest entry).
QP/projection/ZAL results agree to 1e-9 relative.  The mixed method (FP32
per-pair arithmetic, FP64 totals) is held to 1e-5 relative on the gradient,
1e-3 on the Hessian and 1e-8 on the log-likelihood.
"""
import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def make(hx, c, precision="fp64", **kw):
    return hx.GB300Admix(c["bed"], c["I"], c["J"], c["K"], bytes_per_snp=c["bed"].shape[1],
                         n_snp=c["bed"].shape[0], precision=precision, **kw)


def start(c, seed=3):
    from haplo_gb300.admix import random_init
    return random_init(c["I"], c["J"], c["K"], np.random.default_rng(seed))


@pytest.fixture(scope="module")
def coh():
    return small_cohort(333, 203, 3, seed=17, extra_snps=6)


def test_census_and_double_missing_bit_exact(hx, O, coh):
    d = make(hx, coh)
    b = O.Bed(coh["bed"], coh["I"], coh["J"], n_snp=coh["bed"].shape[0])
    np.testing.assert_array_equal(d.census(), O.census(b))
    np.testing.assert_array_equal(d.double_missing(), O.double_missing(b))
    assert int(d.census().sum()) == coh["I"] * coh["J"]


@pytest.mark.parametrize("I,J,K", [(1, 1, 1), (5, 9, 2), (130, 17, 4), (333, 203, 7)])
def test_device_generator_matches_cpu_bytes(hx, O, I, J, K):
    import torch
    from haplo_gb300 import synth
    Q, P = synth.draw_params(I, J, K, 0.4, "dirichlet", seed=I + J + K)
    cq, cp = synth.cumulative(Q, P)
    want = O.synth(99, I, J, cq, cp, 0.03)
    buf = torch.zeros(want.size, dtype=torch.uint8, device="cuda")
    synth.synth_device(99, Q, P, 0.03, buf.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy().reshape(want.shape), want)


@pytest.mark.parametrize("K", list(range(1, 13)))
def test_loglik_and_accumulations_fp64_all_K(hx, O, K):
    c = small_cohort(141, 37, K, seed=100 + K, miss=0.05)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = start(c, seed=K)
    d = make(hx, c)
    assert d.loglikelihood(q, p) == pytest.approx(O.loglik(b, K, q, p), rel=1e-12)
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = O.accum_q(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-12 and rel_err(XtX, oX) < 1e-12
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = O.accum_p(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-12 and rel_err(XtX, oX) < 1e-12
    qn, pn = d.em_accum(q, p)
    oq, op = O.em_accum(b, K, q, p)
    assert rel_err(qn, oq) < 1e-12 and rel_err(pn, op) < 1e-12
    assert rel_err(d.em_p_accum(q, p), op) < 1e-12      # em_p! runner


def test_loglik_formulas_and_injected_state(hx, O, coh):
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    q, p = start(coh)
    d = make(hx, coh)
    d.set_qp(q, p)
    want = O.loglik(b, coh["K"], q, p, formula=1)
    assert d.loglikelihood() == pytest.approx(want, rel=1e-12)
    assert d.loglikelihood(q, p) == pytest.approx(O.loglik(b, coh["K"], q, p, formula=2), rel=1e-12)


def test_qp_and_projection_match_oracle(hx, O, coh):
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    K = coh["K"]
    q, p = start(coh)
    d = make(hx, coh)
    XtX, Xtz = O.accum_q(b, K, q, p)
    dq = d.qp_q(XtX, Xtz, q)
    oq, f = O.qp_q(XtX, Xtz, q)
    assert f == 0 and np.abs(dq - oq).max() < 1e-9
    XtXp, Xtzp = O.accum_p(b, K, q, p)
    dp = d.qp_p(XtXp, Xtzp, p)
    op, f = O.qp_p(XtXp, Xtzp, p)
    assert f == 0 and np.abs(dp - op).max() < 1e-9
    rng = np.random.default_rng(0)
    V = rng.normal(size=(K, 500)) * 0.5 + 1.0 / K
    np.testing.assert_allclose(d.project_q(V), O.project_q(V), atol=1e-15)
    W = rng.normal(size=(K, 400)) * 0.5 + 0.25
    np.testing.assert_allclose(d.project_p(W), O.project_p(W), atol=1e-15)


def test_zal_matches_oracle(hx, O, coh):
    d = make(hx, coh)
    n = coh["K"] * (coh["I"] + 4 * coh["J"])
    rng = np.random.default_rng(4)
    U = np.zeros((n, 3))
    V = np.zeros((n, 3))
    Uo, Vo = U.copy(), V.copy()
    for it in range(1, 6):
        x, xn, xn2 = rng.normal(size=(3, n))
        xt, U, V = d.zal(x, xn, xn2, U, V, it)
        xo, Uo, Vo = O.zal(x, xn, xn2, Uo, Vo, it)
        np.testing.assert_allclose(U, Uo, rtol=0, atol=0)
        assert rel_err(xt, xo) < 1e-9


def test_update_steps_match_oracle(hx, O, coh):
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    K = coh["K"]
    q, p = start(coh)
    d = make(hx, coh)
    d.set_qp(q, p)
    d.update_q(False)
    qn_d = d.get_qp("x_next")[0]
    qn_o, _ = O.update_q(b, K, q, p)
    assert np.abs(qn_d - qn_o).max() < 1e-9
    d.update_p(False)
    pn_d = d.get_qp("x_next")[1]
    pn_o, _ = O.update_p(b, K, qn_o, p)
    assert np.abs(pn_d - pn_o).max() < 1e-9
    d.set_qp(q, p)
    d.em_step()
    qe, pe = d.get_qp("x_next")
    oqe, ope = O.em_step(b, K, q, p)
    assert np.abs(qe - oqe).max() < 1e-12 and np.abs(pe - ope).max() < 1e-12


def test_fit_matches_oracle_fp64(hx, O):
    c = small_cohort(400, 300, 3, seed=21, alpha=0.5, miss=0.01)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q0, p0 = start(c, seed=1)
    qo, po, llo, ito, tro = O.fit(b, 3, q0, p0, n_iter=300, rtol=1e-7)
    d = make(hx, c)
    d.set_qp(q0, p0)
    info = d.fit(n_iter=300, rtol=1e-7, em_iters=5)
    qd, pd = d.get_qp()
    assert info["ll"] == pytest.approx(llo, rel=1e-9)
    assert abs(info["iters"] - ito) <= 1
    assert np.abs(qd - qo).max() < 1e-5
    assert info["ll"] == pytest.approx(d.loglikelihood(qd, pd), rel=1e-12)


def test_mixed_precision_passes(hx, O, coh):
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    K = coh["K"]
    q, p = start(coh)
    d = make(hx, coh, precision="mixed")
    assert d.loglikelihood(q, p) == pytest.approx(O.loglik(b, K, q, p), rel=1e-8)
    XtX, Xtz = d.update_q_accum(q, p)
    oX, oz = O.accum_q(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-5 and rel_err(XtX, oX) < 1e-3
    XtX, Xtz = d.update_p_accum(q, p)
    oX, oz = O.accum_p(b, K, q, p)
    assert rel_err(Xtz, oz) < 1e-5 and rel_err(XtX, oX) < 1e-3


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_loglik_zero_and_nan_likelihoods(hx, O, coh, precision):
    # log of a zero pair likelihood is -inf, of a NaN one NaN, as the
    # reference's FP64 logs (src/loops.jl:236-258)
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    K = coh["K"]
    q, p = start(coh)
    d = make(hx, coh, precision=precision)
    p0 = p.copy()
    p0[:, 0] = 0.0                       # qp00 = 0 in block 0 for everyone
    assert np.isneginf(O.loglik(b, K, q, p0))
    assert np.isneginf(d.loglikelihood(q, p0))
    q1 = q.copy()
    q1[0, 5] = np.nan
    assert np.isnan(O.loglik(b, K, q1, p))
    assert np.isnan(d.loglikelihood(q1, p))
    p1 = p0.copy()
    p1[:, 4 * coh["J"] - 1] = np.nan     # NaN and zero likelihoods together: NaN
    assert np.isnan(d.loglikelihood(q, p1))
    assert d.loglikelihood(q, p) == pytest.approx(O.loglik(b, K, q, p), rel=1e-8 if precision == "mixed" else 1e-12)


def test_mixed_fit_reaches_fp64_optimum(hx, O):
    # both fits run to (near) full convergence, so that the comparison is
    # between optima and not between two early-stopped points of a flat
    # likelihood (I=400, J=300 pins Q only loosely at rtol 1e-9)
    c = small_cohort(400, 300, 3, seed=21, alpha=0.5, miss=0.01)
    q0, p0 = start(c, seed=1)
    out = {}
    for prec in ("fp64", "mixed"):
        d = make(hx, c, precision=prec)
        d.set_qp(q0, p0)
        info = d.fit(n_iter=3000, rtol=1e-14, em_iters=5)
        out[prec] = (info, d.get_qp()[0])
    assert out["mixed"][0]["ll"] == pytest.approx(out["fp64"][0]["ll"], rel=5e-9)
    assert np.abs(out["mixed"][1] - out["fp64"][1]).max() < 2e-5


def test_errors_are_status_codes(hx, coh):
    from haplo_gb300 import HxError
    with pytest.raises(HxError):
        hx.GB300Admix(coh["bed"], coh["I"], coh["J"], 13)          # K above HX_KMAX
    d = make(hx, coh)
    with pytest.raises(HxError):
        d.update_q()                                               # Q/P not set yet


@pytest.mark.parametrize("opts", [dict(fix_q=True), dict(fix_p=True), dict(guarantee_increase=True),
                                  dict(penalty=True), dict(penalty=False), dict(mode="LBQN")])
def test_loop_options_match_oracle_fp64(hx, O, opts):
    # admixture_qn!/init_em! keywords (src/algorithms_outer.jl:1-3, 38-41)
    c = small_cohort(240, 120, 3, seed=33, alpha=0.5, miss=0.01)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q0, p0 = start(c, seed=5)
    q0, p0 = O.project_q(q0), O.project_p(p0)
    qo, po, llo, ito, _ = O.fit(b, 3, q0, p0, n_iter=60, rtol=1e-8, em_iters=2, **opts)
    d = make(hx, c)
    d.set_loop_opts(**opts)
    d.set_qp(q0, p0)
    info = d.fit(n_iter=60, rtol=1e-8, em_iters=2)
    qd, pd = d.get_qp()
    assert info["ll"] == pytest.approx(llo, rel=1e-9)
    assert abs(info["iters"] - ito) <= 1
    assert np.abs(qd - qo).max() < 1e-6 and np.abs(pd - po).max() < 1e-6
    if opts.get("fix_q"):
        np.testing.assert_allclose(qd, q0, rtol=0, atol=1e-15)
    if opts.get("fix_p"):
        np.testing.assert_allclose(pd, p0, rtol=0, atol=1e-15)


@pytest.mark.parametrize("K", [1, 2, 3, 5, 8, 12])
def test_qp_p_equality_form_matches_oracle(hx, O, K):
    # penalty = false: per block, 4K variables with the K equalities
    # sum_h d[k, h] = 0 (src/algorithms_inner.jl:307-310)
    c = small_cohort(300, 160, K, seed=40 + K, alpha=0.4, miss=0.01)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = start(c, seed=K)
    XtX, Xtz = O.accum_p(b, K, q, p)
    do, fails = O.qp_p_eq(XtX, Xtz, p)
    assert fails == 0
    d = make(hx, c)
    d.set_loop_opts(penalty=False)
    dg = d.qp_p(XtX, Xtz, p)
    scale = np.abs(do).max()
    assert np.abs(dg - do).max() <= 1e-9 * max(scale, 1.0)
    np.testing.assert_allclose(dg.reshape(K, -1, 4).sum(axis=2), 0.0, atol=1e-12)


def test_loop_opts_reject_unknown_penalty(hx, coh):
    import ctypes as C
    from haplo_gb300 import HxError, _lib
    d = make(hx, coh)
    o = _lib.HxLoopOpts()
    d._ck(d.lib.hx_loop_opts_default(C.byref(o)))
    o.penalty = 2
    with pytest.raises(HxError):
        d._ck(d.lib.hx_set_loop_opts(d._h, C.byref(o)))
