"""Failure paths on the GPU, in forms that fault and hang nothing, and the
.bed front end end to end.

* Bounded waits: with a one-cycle wait budget (hx_set_wait_budget) a
  tensor-core pass stops at the first pipeline wait whose phase is still
  open (at the latest the wait for the last window's MMAs), drains what it
  issued and the call returns HX_ETIMEOUT; the same handle then runs the pass again
  with the default budget and matches the oracle (gradient 1e-6, Hessian
  1e-4 relative to the largest entry, the tensor-core bounds of
  test_gpu_tc.py).
* Host-side refusals: K beyond HX_KMAX, a SNP range beyond the matrix, a
  fit with no Q/P set.
* run_admixture (src/driver.jl:38-79) on a .bed written to disk that holds
  more individuals and SNPs than the fit uses: the FP64 fit equals the
  oracle fit on the same bytes (ll 1e-9 relative, Q and P 1e-5, +-1 outer
  iteration).
"""
import numpy as np
import pytest

from conftest import small_cohort

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _make(hx, c, precision):
    return hx.GB300Admix(c["bed"], c["I"], c["J"], c["K"], bytes_per_snp=c["bed"].shape[1],
                         n_snp=c["bed"].shape[0], precision=precision)


@pytest.mark.parametrize("side", ["q", "p"])
def test_wait_timeout_returns_status_and_handle_recovers(hx, O, side):
    from haplo_gb300 import _lib
    from haplo_gb300.admix import random_init
    # enough blocks that the P side's grid fills its waves with few chunks,
    # so that each CTA runs many stages (its waits on earlier MMAs then meet
    # open phases)
    c = small_cohort(1000, 80000, 4, seed=41)
    b = O.Bed(c["bed"], c["I"], c["J"])
    q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(5))
    d = _make(hx, c, "mixed")
    accum = d.update_q_accum if side == "q" else d.update_p_accum
    want = O.accum_q(b, c["K"], q, p) if side == "q" else O.accum_p(b, c["K"], q, p)
    for _ in range(2):
        d.set_wait_budget(1)
        with pytest.raises(hx.HxError) as e:
            accum(q, p)
        assert e.value.status == _lib.HX_ETIMEOUT
        d.set_wait_budget(0)
        XtX, Xtz = accum(q, p)
        assert rel_err(Xtz, want[1]) < 1e-6
        assert rel_err(XtX, want[0]) < 1e-4
    # the whole device-resident loop still runs on the handle
    d.set_qp(q, p)
    d.init_em(1)
    info = d.qn_iteration()
    assert np.isfinite(info["ll_new"]) and info["ll_new"] > O.loglik(b, c["K"], q, p)
    d.close()


def test_fit_timeout_surfaces_from_the_loop(hx):
    from haplo_gb300 import _lib
    from haplo_gb300.admix import random_init
    c = small_cohort(260, 45, 3, seed=42)
    q, p = random_init(c["I"], c["J"], c["K"], np.random.default_rng(6))
    d = _make(hx, c, "mixed")
    d.set_qp(q, p)
    d.set_wait_budget(1)
    with pytest.raises(hx.HxError) as e:
        d.qn_iteration()
    assert e.value.status == _lib.HX_ETIMEOUT
    d.set_wait_budget(0)
    d.set_qp(q, p)
    info = d.fit(n_iter=50, rtol=1e-7, em_iters=2)
    assert np.isfinite(info["ll"])
    d.close()


def test_host_side_refusals(hx):
    from haplo_gb300 import _lib
    c = small_cohort(40, 9, 2, seed=43)
    with pytest.raises(hx.HxError) as e:
        hx.GB300Admix(c["bed"], c["I"], c["J"], 13, bytes_per_snp=c["bed"].shape[1], n_snp=c["bed"].shape[0])
    assert e.value.status == _lib.HX_EUNSUPPORTED
    with pytest.raises(hx.HxError) as e:     # 2J SNPs beyond the matrix
        hx.GB300Admix(c["bed"], c["I"], c["J"] + 1, 2, bytes_per_snp=c["bed"].shape[1], n_snp=c["bed"].shape[0])
    assert e.value.status == _lib.HX_EINVAL
    d = _make(hx, c, "fp64")
    with pytest.raises(hx.HxError) as e:     # no Q/P yet
        d.fit(n_iter=1)
    assert e.value.status == _lib.HX_ESTATE
    d.close()


@pytest.mark.parametrize("precision", ["fp64"])
def test_run_admixture_from_disk_matches_oracle(hx, O, tmp_path, precision):
    from haplo_gb300 import bed as bedio
    from haplo_gb300.admix import run_admixture, random_init
    N, Jf, I, J, K = 150, 40, 131, 33, 3
    c = small_cohort(N, Jf, K, seed=44, miss=0.02)
    path = bedio.write_bed(str(tmp_path / "cohort"), c["bed"], N)
    res, d = run_admixture(path, I, J, K, rng=7, admix_rtol=1e-7, precision=precision, return_handle=True)
    d.close()
    data, n, m = bedio.read_bed(path)
    assert (n, m) == (N, 2 * Jf)
    q0, p0 = random_init(I, J, K, np.random.default_rng(7))
    b = O.Bed(data, I, J, n_snp=m)
    oq, op, oll, oit, _ = O.fit(b, K, q0, p0, n_iter=1000, rtol=1e-7, em_iters=5)
    assert res.ll_new == pytest.approx(oll, rel=1e-9)
    assert abs(res.info["iters"] - oit) <= 1
    assert np.abs(res.q - oq).max() < 1e-5
    assert np.abs(res.p - op).max() < 1e-5


def test_run_admixture_fix_p_with_injected_start(hx, O, tmp_path):
    """fix_p with init_q/init_p (no init_em!): P stays at init_p and the fit
    equals the oracle's admixture_qn! with fix_p from the same start."""
    from haplo_gb300 import bed as bedio
    from haplo_gb300.admix import run_admixture, random_init
    I, J, K = 120, 30, 3
    c = small_cohort(I, J, K, seed=45)
    path = bedio.write_bed(str(tmp_path / "c"), c["bed"], I)
    q0, p0 = random_init(I, J, K, np.random.default_rng(9))
    res, _, _ = run_admixture(path, I, J, K, init_q=q0, init_p=p0, fix_p=True, admix_rtol=1e-8)
    assert np.abs(res.p - p0).max() < 1e-12      # held (the QN point's projection may touch the last bits)
    oq, op, oll, oit, _ = O.fit(O.Bed(c["bed"], I, J), K, q0, p0, n_iter=1000, rtol=1e-8, em_iters=0, fix_p=True)
    assert res.ll_new == pytest.approx(oll, rel=1e-9)
    assert np.abs(res.q - oq).max() < 1e-6
    assert np.abs(res.p - op).max() < 1e-12
