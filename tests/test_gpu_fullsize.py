"""GPU checks at the benchmark's full size: I = 100,000 individuals x 200,000
SNPs (J = 100,000 blocks), K = 8, i.e. 1e10 (individual, block) pairs per
pass.  The CPU oracle cannot run passes of this size in a test, so these
checks use properties that hold at any size:

* the census counts every pair exactly once;
* exact identities of the accumulated sums: with c the E-step counts,
  sum_k q[k,i] Xtz_q[k,i] = sum_{j,h} c_h = 2 (J - dm_i), and the Hessian
  contracted with the point it was formed at returns the gradient,
  sum_k2 XtX_q[k,k2,i] q[k2,i] = Xtz_q[k,i] (likewise with p on the P side);
* the mixed tensor-core passes and log-likelihood agree with the plain FP64
  passes on the same genotype matrix (tolerances as in the small tests);
* an EM step does not lower the log-likelihood (MM property).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def c3(hx):
    import torch
    from haplo_gb300 import synth
    from haplo_gb300.admix import random_init
    cfg = synth.config("C3")
    I, J, K, bps = cfg["I"], cfg["J"], cfg["K"], cfg["bps"]
    bed = torch.empty(bps * 2 * J, dtype=torch.uint8, device="cuda")
    synth.synth_device(cfg["seed"], cfg["Q"], cfg["P"], cfg["miss"], bed.data_ptr())
    torch.cuda.synchronize()
    q, p = random_init(I, J, K, np.random.default_rng(5))
    mixed = hx.GB300Admix(bed.data_ptr(), I, J, K, bytes_per_snp=bps, n_snp=2 * J, precision="mixed",
                          bed_on_device=True)
    fp64 = hx.GB300Admix.shared(mixed, K, precision="fp64")
    yield dict(I=I, J=J, K=K, q=q, p=p, mixed=mixed, fp64=fp64, bed=bed)
    fp64.close()
    mixed.close()


def test_fullsize_census_counts_every_pair(c3):
    d = c3["mixed"]
    counts = d.census()
    assert int(counts.sum()) == c3["I"] * c3["J"]
    dm = d.double_missing()
    assert dm.shape == (c3["I"],) and dm.min() >= 0 and dm.max() <= c3["J"]
    assert int(dm.sum()) == int(counts[15])            # class 15: both SNPs missing


def test_fullsize_q_sums_identities_and_fp64_agreement(c3):
    q, p, J = c3["q"], c3["p"], c3["J"]
    XtX, Xtz = c3["mixed"].update_q_accum(q, p)
    dm = c3["mixed"].double_missing().astype(np.float64)
    # sum_k q_k Xtz_q[k, i] = sum of the expected counts = 2 (J - dm_i)
    assert rel_err((q * Xtz).sum(axis=0), 2.0 * (J - dm)) < 1e-6
    # H_i q_i = g_i
    assert rel_err(np.einsum("abi,bi->ai", XtX, q), Xtz) < 1e-4
    oX, oz = c3["fp64"].update_q_accum(q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4


def test_fullsize_p_sums_identities_and_fp64_agreement(c3):
    q, p = c3["q"], c3["p"]
    XtX, Xtz = c3["mixed"].update_p_accum(q, p)
    # H_m p_m = g_m for every haplotype column m
    assert rel_err(np.einsum("abm,bm->am", XtX, p), Xtz) < 1e-4
    oX, oz = c3["fp64"].update_p_accum(q, p)
    assert rel_err(Xtz, oz) < 1e-6 and rel_err(XtX, oX) < 1e-4


def test_fullsize_loglik_mixed_matches_fp64_and_em_ascends(c3):
    q, p = c3["q"], c3["p"]
    ll_m = c3["mixed"].loglikelihood(q, p)
    ll_d = c3["fp64"].loglikelihood(q, p)
    assert ll_m == pytest.approx(ll_d, rel=1e-8)
    d = c3["mixed"]
    d.set_qp(q, p)
    d.em_step()
    qn, pn = d.get_qp("x_next")
    assert c3["fp64"].loglikelihood(qn, pn) >= ll_d
