"""Analytic pins of the oracle: gradient = finite difference of the
log-likelihood, EM monotonicity, QP optimality (KKT and brute force over
active sets), projection optimality, the ZAL formula, and the fit."""
import itertools

import numpy as np
import pytest

from conftest import small_cohort


@pytest.fixture(scope="module")
def coh(O):
    c = small_cohort(150, 60, 3, seed=11)
    c["b"] = O.Bed(c["bed"], c["I"], c["J"])
    from haplo_gb300.admix import random_init
    c["q0"], c["p0"] = random_init(c["I"], c["J"], c["K"], np.random.default_rng(3))
    return c


def test_two_loglik_formulas_agree(O, coh):
    l1 = O.loglik(coh["b"], coh["K"], coh["q0"], coh["p0"], formula=1)
    l2 = O.loglik(coh["b"], coh["K"], coh["q0"], coh["p0"], formula=2)
    assert l1 == pytest.approx(l2, rel=1e-14)


def test_gradient_is_finite_difference(O, coh):
    b, K, q, p = coh["b"], coh["K"], coh["q0"], coh["p0"]
    l0 = O.loglik(b, K, q, p)
    _, Xtz_q = O.accum_q(b, K, q, p)
    _, Xtz_p = O.accum_p(b, K, q, p)
    for (k, i) in [(0, 3), (2, 77), (1, 149)]:
        e = 1e-6
        qq = q.copy()
        qq[k, i] += e
        fd = (O.loglik(b, K, qq, p) - l0) / e
        assert fd == pytest.approx(Xtz_q[k, i], rel=1e-4)
    for (k, m) in [(0, 5), (2, 101), (1, 239)]:
        e = 1e-6
        pp = p.copy()
        pp[k, m] += e
        fd = (O.loglik(b, K, q, pp) - l0) / e
        assert fd == pytest.approx(Xtz_p[k, m], rel=1e-4)


def test_hessian_is_psd_and_symmetric(O, coh):
    XtX, _ = O.accum_q(coh["b"], coh["K"], coh["q0"], coh["p0"])
    for i in range(0, coh["I"], 17):
        H = XtX[:, :, i]
        np.testing.assert_allclose(H, H.T, rtol=1e-13)
        assert np.linalg.eigvalsh(H).min() > -1e-9 * np.abs(H).max()


def test_em_step_increases_loglik(O, coh):
    b, K = coh["b"], coh["K"]
    q, p = coh["q0"], coh["p0"]
    prev = O.loglik(b, K, q, p)
    for _ in range(4):
        q, p = O.em_step(b, K, q, p)
        cur = O.loglik(b, K, q, p)
        assert cur >= prev - 1e-8 * abs(prev)
        prev = cur
    np.testing.assert_allclose(q.sum(axis=0), 1.0, rtol=1e-12)
    np.testing.assert_allclose(p.reshape(K, -1, 4).sum(axis=2), 1.0, rtol=1e-12)


def _groups(eq, n):
    """Equality groups as index lists: eq False -> none, True -> one sum over
    all variables, G >= 2 -> {a : a % G == k} for every k < G."""
    G = 0 if eq is False else (1 if eq is True else int(eq))
    return [[a for a in range(n) if a % G == k] for k in range(G)] if G else []


def _kkt(H, z, lo, hi, eq, d, tol):
    """KKT of min 0.5 d'Hd - z'd, lo <= d <= hi and the equality groups of
    `eq` (each group sums to 0): with g = Hd - z there is a multiplier nu per
    group (0 off the groups) such that g + nu >= 0 at lower bounds, <= 0 at
    upper bounds and = 0 on free variables."""
    n = len(d)
    g = H @ d - z
    assert np.all(d >= lo - 1e-12) and np.all(d <= hi + 1e-12)
    at_lo = d <= lo + 1e-12
    at_hi = (d >= hi - 1e-12) & ~at_lo
    free = ~at_lo & ~at_hi
    nu = np.zeros(n)
    for grp in _groups(eq, n):
        assert abs(d[grp].sum()) < 1e-10
        nu_min = max([-g[a] for a in grp if at_lo[a] or free[a]], default=-np.inf)
        nu_max = min([-g[a] for a in grp if at_hi[a] or free[a]], default=np.inf)
        assert nu_min <= nu_max + 2 * tol
        nu[grp] = nu_max if np.isfinite(nu_max) else nu_min
    r = g + nu
    assert np.all(r[at_lo] >= -2 * tol)
    assert np.all(r[at_hi] <= 2 * tol)
    assert np.all(np.abs(r[free]) <= 2 * tol)


def _brute(H, z, lo, hi, eq):
    """Minimum over all assignments of variables to {lo, hi, free}."""
    n = len(z)
    grps = _groups(eq, n)
    best, bd = np.inf, None
    for assign in itertools.product((0, 1, 2), repeat=n):
        fixed = [a for a in range(n) if assign[a] != 2]
        free = [a for a in range(n) if assign[a] == 2]
        d = np.zeros(n)
        for a in fixed:
            d[a] = lo[a] if assign[a] == 0 else hi[a]
        if free:
            Hf = H[np.ix_(free, free)]
            r = z[free] - H[np.ix_(free, fixed)] @ d[fixed] if fixed else z[free]
            E = np.array([[1.0 if a in grp else 0.0 for a in free] for grp in grps]).reshape(len(grps), len(free))
            keep = [e for e in range(len(grps)) if E[e].any()]
            if any(abs(d[grps[e]].sum()) > 1e-12 for e in range(len(grps)) if e not in keep):
                continue
            E = E[keep]
            m, c = len(free), len(keep)
            KKT = np.zeros((m + c, m + c))
            KKT[:m, :m] = Hf
            KKT[:m, m:] = E.T
            KKT[m:, :m] = E
            rhs = np.concatenate([r, [-d[[a for a in grps[e] if a in fixed]].sum() for e in keep]])
            try:
                sol = np.linalg.solve(KKT, rhs)
            except np.linalg.LinAlgError:
                continue
            d[free] = sol[:m]
        elif any(abs(d[grp].sum()) > 1e-12 for grp in grps):
            continue
        if np.any(d < lo - 1e-12) or np.any(d > hi + 1e-12):
            continue
        if any(abs(d[grp].sum()) > 1e-9 for grp in grps):
            continue
        f = 0.5 * d @ H @ d - z @ d
        if f < best:
            best, bd = f, d
    return bd, best


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("eq", [True, False])
def test_qp_matches_brute_force(O, seed, eq):
    rng = np.random.default_rng(seed)
    n = 4
    A = rng.normal(size=(n, n))
    H = A @ A.T + 0.1 * np.eye(n)
    z = rng.normal(size=n) * 3
    x = rng.dirichlet(np.ones(n))
    lo, hi = -x, 1 - x
    d, it = O.qp_dense(H, z, lo, hi, eq)
    assert it > 0
    bd, best = _brute(H, z, lo, hi, eq)
    f = 0.5 * d @ H @ d - z @ d
    assert f == pytest.approx(best, rel=1e-9, abs=1e-9)
    np.testing.assert_allclose(d, bd, atol=1e-8)
    _kkt(H, z, lo, hi, eq, d, 1e-8 * (1 + np.abs(z).max()))


@pytest.mark.parametrize("seed", range(8))
def test_qp_groups_match_brute_force(O, seed):
    # the P equality form: 4K variables h*K + k, group k sums to zero (K = 2)
    rng = np.random.default_rng(100 + seed)
    K, n = 2, 8
    H = np.zeros((n, n))
    for l in range(4):
        A = rng.normal(size=(K, K))
        H[l * K:(l + 1) * K, l * K:(l + 1) * K] = A @ A.T + 0.1 * np.eye(K)
    z = rng.normal(size=n) * 3
    x = np.concatenate([rng.dirichlet(np.ones(4)) for _ in range(K)]).reshape(K, 4).T.ravel()
    lo, hi = -x, 1 - x
    d, it = O.qp_dense(H, z, lo, hi, K)
    assert it > 0
    bd, best = _brute(H, z, lo, hi, K)
    f = 0.5 * d @ H @ d - z @ d
    assert f == pytest.approx(best, rel=1e-9, abs=1e-9)
    np.testing.assert_allclose(d, bd, atol=1e-8)
    _kkt(H, z, lo, hi, K, d, 1e-8 * (1 + np.abs(z).max()))


def test_qp_p_equality_form_satisfies_kkt(O, coh):
    b, K, q, p = coh["b"], coh["K"], coh["q0"], coh["p0"]
    XtXp, Xtzp = O.accum_p(b, K, q, p)
    dp, fails = O.qp_p_eq(XtXp, Xtzp, p)
    assert fails == 0
    n = 4 * K
    np.testing.assert_allclose(dp.reshape(K, -1, 4).sum(axis=2), 0.0, atol=1e-12)
    for j in range(0, coh["J"], 5):
        H = np.zeros((n, n))
        for l in range(4):
            H[l * K:(l + 1) * K, l * K:(l + 1) * K] = XtXp[:, :, 4 * j + l]
        z = Xtzp[:, 4 * j:4 * j + 4].ravel(order="F")
        pj = p[:, 4 * j:4 * j + 4].ravel(order="F")
        dj = dp[:, 4 * j:4 * j + 4].ravel(order="F")
        _kkt(H, z, -pj, 1 - pj, K, dj, 1e-7 * (1 + np.abs(z).max()))


def test_qp_batches_satisfy_kkt(O, coh):
    b, K, q, p = coh["b"], coh["K"], coh["q0"], coh["p0"]
    XtX, Xtz = O.accum_q(b, K, q, p)
    d, fails = O.qp_q(XtX, Xtz, q)
    assert fails == 0
    for i in range(0, coh["I"], 13):
        _kkt(XtX[:, :, i], Xtz[:, i], -q[:, i], 1 - q[:, i], True, d[:, i], 1e-7 * np.abs(Xtz[:, i]).max())
    XtXp, Xtzp = O.accum_p(b, K, q, p)
    dp, fails = O.qp_p(XtXp, Xtzp, p, rho=1e7)
    assert fails == 0
    n = 4 * K
    for j in range(0, coh["J"], 7):
        H = np.zeros((n, n))
        for l in range(4):
            H[l * K:(l + 1) * K, l * K:(l + 1) * K] = XtXp[:, :, 4 * j + l]
        for l in range(4):
            for l2 in range(4):
                for k in range(K):
                    H[l * K + k, l2 * K + k] += 1e7
        z = Xtzp[:, 4 * j:4 * j + 4].ravel(order="F")
        pj = p[:, 4 * j:4 * j + 4].ravel(order="F")
        dj = dp[:, 4 * j:4 * j + 4].ravel(order="F")
        _kkt(H, z, -pj, 1 - pj, False, dj, 1e-6 * (1 + np.abs(z).max()))


@pytest.mark.parametrize("n", [2, 3, 4, 6, 9])
def test_projection_is_euclidean_projection(O, n):
    rng = np.random.default_rng(n)
    eps = 1e-5
    V = rng.normal(size=(n, 200)) * 0.7 + 1.0 / n
    P = O.project_q(V, eps)
    assert np.all(P >= eps - 1e-15)
    np.testing.assert_allclose(P.sum(axis=0), 1.0, rtol=1e-13)
    # optimality: v - x = t 1 + mu with mu >= 0 only where x == eps
    for c in range(V.shape[1]):
        r = V[:, c] - P[:, c]
        inner = P[:, c] > eps + 1e-12
        t = r[inner].mean()
        np.testing.assert_allclose(r[inner], t, atol=1e-12)
        assert np.all(r[~inner] <= t + 1e-12)
    np.testing.assert_allclose(O.project_q(P, eps), P, atol=1e-15)


def test_zal_formula(O):
    rng = np.random.default_rng(5)
    n, Qs = 40, 3
    U = rng.normal(size=(n, Qs))
    V = rng.normal(size=(n, Qs))
    for it in (1, 2, 3, 4, 5):
        x, xn, xn2 = rng.normal(size=(3, n))
        xt, U2, V2 = O.zal(x, xn, xn2, U, V, it)
        c = (it - 1) % Qs
        np.testing.assert_allclose(U2[:, c], xn - x)
        np.testing.assert_allclose(V2[:, c], xn2 - xn)
        m = min(it, Qs)
        Um, Vm = U2[:, :m], V2[:, :m]
        want = xn - Vm @ np.linalg.solve(Um.T @ Um - Um.T @ Vm, Um.T @ (x - xn))
        np.testing.assert_allclose(xt, want, rtol=1e-9, atol=1e-12)
        U, V = U2, V2


def test_lbqn_point_is_the_bad_broyden_step(O):
    # mode LBQN: the multi-secant "bad" Broyden inverse H = -I + V (Y'Y)^-1 Y',
    # Y = V - U, satisfies H Y = U, and the point is x - H (F(x) - x)
    rng = np.random.default_rng(6)
    n, Qs = 40, 3
    U = rng.normal(size=(n, Qs))
    V = rng.normal(size=(n, Qs))
    for it in (1, 2, 3, 4, 5):
        x, xn, xn2 = rng.normal(size=(3, n))
        xt, U2, V2 = O.qn(x, xn, xn2, U, V, it, mode="LBQN")
        c = (it - 1) % Qs
        np.testing.assert_allclose(U2[:, c], xn - x)
        np.testing.assert_allclose(V2[:, c], xn2 - xn)
        m = min(it, Qs)
        Um, Vm = U2[:, :m], V2[:, :m]
        Y = Vm - Um
        H = -np.eye(n) + Vm @ np.linalg.solve(Y.T @ Y, Y.T)
        np.testing.assert_allclose(H @ Y, Um, atol=1e-10)
        np.testing.assert_allclose(xt, x - H @ (xn - x), rtol=1e-9, atol=1e-10)
        zt, _, _ = O.qn(x, xn, xn2, U, V, it, mode="ZAL")
        np.testing.assert_allclose(zt, O.zal(x, xn, xn2, U, V, it)[0], rtol=0, atol=0)
        U, V = U2, V2


def test_lbqn_fit_reaches_the_zal_optimum(O, loop_case):
    c, b, q0, p0 = loop_case
    _, _, ll_z, _, _ = O.fit(b, 3, q0, p0, n_iter=400, rtol=1e-12, em_iters=3)
    q, p, ll_l, it, trace = O.fit(b, 3, q0, p0, n_iter=400, rtol=1e-12, em_iters=3, mode="LBQN")
    assert ll_l == pytest.approx(ll_z, rel=1e-7)
    assert np.all(np.diff(trace) >= -1e-9 * np.abs(trace[1:]))   # each iteration keeps the better point


def test_fit_beats_truth_and_converges(O):
    c = small_cohort(400, 300, 3, seed=21, alpha=0.5, miss=0.01)
    b = O.Bed(c["bed"], c["I"], c["J"])
    from haplo_gb300.admix import random_init
    q0, p0 = random_init(c["I"], c["J"], 3, np.random.default_rng(1))
    q, p, ll, iters, trace = O.fit(b, 3, q0, p0, n_iter=300, rtol=1e-7)
    assert iters < 300
    assert ll >= O.loglik(b, 3, c["Q"], c["P"])
    assert trace[-1] > trace[0]
    assert ll == pytest.approx(O.loglik(b, 3, q, p), rel=1e-12)


# ---- loop options of admixture_qn!/init_em! (src/algorithms_outer.jl:1-3, 38-41)

@pytest.fixture(scope="module")
def loop_case(O):
    c = small_cohort(240, 120, 3, seed=33, alpha=0.5, miss=0.01)
    b = O.Bed(c["bed"], c["I"], c["J"])
    from haplo_gb300.admix import random_init
    q0, p0 = random_init(c["I"], c["J"], 3, np.random.default_rng(5))
    # start on the feasible set, which init_em!'s projections leave in place
    return c, b, O.project_q(q0), O.project_p(p0)


def test_fix_q_and_fix_p_keep_that_factor(O, loop_case):
    c, b, q0, p0 = loop_case
    q, p, ll, it, _ = O.fit(b, 3, q0, p0, n_iter=20, rtol=1e-9, em_iters=2, fix_q=True)
    np.testing.assert_allclose(q, q0, rtol=0, atol=1e-15)
    assert not np.allclose(p, p0)
    assert ll > O.loglik(b, 3, q0, p0)
    q, p, ll, it, _ = O.fit(b, 3, q0, p0, n_iter=20, rtol=1e-9, em_iters=2, fix_p=True)
    np.testing.assert_allclose(p, p0, rtol=0, atol=1e-15)
    assert not np.allclose(q, q0)


def test_guarantee_increase_never_lowers_the_loglik(O, loop_case):
    c, b, q0, p0 = loop_case
    q, p, ll, it, trace = O.fit(b, 3, q0, p0, n_iter=40, rtol=1e-10, em_iters=0, guarantee_increase=True)
    assert np.all(np.diff(trace) >= -1e-9 * np.abs(trace[1:]))
    _, _, ll_plain, _, _ = O.fit(b, 3, q0, p0, n_iter=300, rtol=1e-10, em_iters=0)
    assert ll == pytest.approx(ll_plain, rel=1e-4)


def test_q_penalty_form_solves_the_penalised_qp(O, coh):
    # penalty = true: min 0.5 d'(H + rho 1 1')d - z'd over the box, no equality
    b = O.Bed(coh["bed"], coh["I"], coh["J"])
    K = coh["K"]
    from haplo_gb300.admix import random_init
    q, p = random_init(coh["I"], coh["J"], K, np.random.default_rng(2))
    XtX, Xtz = O.accum_q(b, K, q, p)
    rho = 1e7
    for i in range(0, coh["I"], 37):
        H = XtX[:, :, i] + rho
        d, it = O.qp_dense(H, Xtz[:, i], -q[:, i], 1 - q[:, i], False)
        assert it > 0
        g = H @ d - Xtz[:, i]
        lo, hi = -q[:, i], 1 - q[:, i]
        free = (d > lo + 1e-12) & (d < hi - 1e-12)
        assert np.all(np.abs(g[free]) <= 1e-6 * max(1.0, np.abs(Xtz[:, i]).max()))
        assert abs(d.sum()) < 10 * np.abs(Xtz[:, i]).max() / rho   # the penalty leaves O(z / rho)


def test_penalty_true_fit_matches_default_optimum(O, loop_case):
    c, b, q0, p0 = loop_case
    _, _, ll_pen, _, _ = O.fit(b, 3, q0, p0, n_iter=400, rtol=1e-12, em_iters=3, penalty=True)
    _, _, ll_def, _, _ = O.fit(b, 3, q0, p0, n_iter=400, rtol=1e-12, em_iters=3)
    assert ll_pen == pytest.approx(ll_def, rel=1e-6)
    _, _, ll_eq, _, _ = O.fit(b, 3, q0, p0, n_iter=400, rtol=1e-12, em_iters=3, penalty=False)
    assert ll_eq == pytest.approx(ll_def, rel=1e-6)
