"""AIM selection on the GPU (hx_skfr) against the CPU oracle
(oracle/skfr_oracle.py): clusters, selected SNPs and iteration count equal
bit for bit (integer code counts and round-to-nearest FP64 in a fixed order
on both sides), on planted and admixed cohorts with missing genotypes, odd SNP
counts and I not a multiple of 4; then run_admixture's `sparsity` branch end
to end against the oracle's selection, filter and fit."""
import numpy as np
import pytest

from conftest import small_cohort
from test_skfr_oracle import planted

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["planted", "admixed_odd", "k1", "k12"])
def test_skfr_matches_oracle(hx, O, case):
    from haplo_gb300 import skfr
    from oracle import skfr_oracle as S
    if case == "planted":
        I, K, s = 300, 3, 15
        bed = planted(I, 120, K, np.arange(5, 120, 8), seed=3)
    elif case == "admixed_odd":
        c = small_cohort(257, 61, 4, seed=52, miss=0.05, extra_snps=1)   # 123 SNPs: the last is ignored
        I, K, s, bed = 257, 4, 9, c["bed"]
    elif case == "k1":
        c = small_cohort(101, 30, 2, seed=53)
        I, K, s, bed = 101, 1, 5, c["bed"]
    else:
        c = small_cohort(240, 40, 5, seed=54, miss=0.02)
        I, K, s, bed = 240, 12, 12, c["bed"]
    for seed in (0, 7):
        gc, ga, gi, gw = skfr.select_once(bed, I, K, s, seed=seed, max_iter=30)
        oc, oa, oi, ow = S.select(bed, I, K, s, seed=seed, max_iter=30, return_objective=True)
        np.testing.assert_array_equal(ga, oa)
        np.testing.assert_array_equal(gc, oc)
        assert gi == oi and gw == ow
    # several tries keep the start with the smallest within-cluster sum of squares
    runs = [S.select(bed, I, K, s, seed=1000 * t, max_iter=30, return_objective=True) for t in range(3)]
    best = min(range(3), key=lambda t: (runs[t][3], t))
    tc, ta, _ = skfr.select_aims(bed, I, K, s, seed=0, max_iter=30, tries=3)
    np.testing.assert_array_equal(ta, runs[best][1])
    np.testing.assert_array_equal(tc, runs[best][0])


def test_skfr_rejects_bad_sizes(hx):
    """Refused on the host, before any device work."""
    from haplo_gb300 import _lib, skfr
    c = small_cohort(20, 6, 2, seed=55)
    for K, s in ((2, 7), (2, 0)):             # sparsity outside 1..6 blocks
        with pytest.raises(hx.HxError) as e:
            skfr.select_aims(c["bed"], 20, K, s)
        assert e.value.status == _lib.HX_EINVAL
    tiny = small_cohort(5, 6, 2, seed=56)
    with pytest.raises(hx.HxError) as e:      # more clusters than individuals
        skfr.select_aims(tiny["bed"], 5, 6, 2)
    assert e.value.status == _lib.HX_EINVAL
    with pytest.raises(hx.HxError) as e:      # K beyond HX_KMAX
        skfr.select_aims(c["bed"], 20, 13, 2)
    assert e.value.status == _lib.HX_EUNSUPPORTED


def test_run_admixture_with_sparsity(hx, O, tmp_path):
    from haplo_gb300 import bed as bedio, skfr
    from haplo_gb300.admix import run_admixture, random_init
    from oracle import skfr_oracle as S
    I, nb, K, s = 300, 120, 3, 15
    data = planted(I, nb, K, np.arange(5, 120, 8), seed=6)
    path = bedio.write_bed(str(tmp_path / "cohort"), data, I)
    res, clusters, aims = run_admixture(path, I, s, K, rng=11, sparsity=s, skfr_seed=2, admix_rtol=1e-7)
    oc, oa, _ = S.select(data, I, K, s, seed=2)
    np.testing.assert_array_equal(aims, oa)
    np.testing.assert_array_equal(clusters, oc)
    fpath = str(tmp_path / ("cohort_%d_%daims.bed" % (K, 2 * s)))
    fdata, n, m = bedio.read_bed(fpath)
    assert (n, m) == (I, 2 * s)
    np.testing.assert_array_equal(fdata, skfr.filter_bed(data, oa))
    q0, p0 = random_init(I, s, K, np.random.default_rng(11))
    oq, op, oll, oit, _ = O.fit(O.Bed(fdata, I, s), K, q0, p0, n_iter=1000, rtol=1e-7, em_iters=5)
    assert res.ll_new == pytest.approx(oll, rel=1e-9)
    assert abs(res.info["iters"] - oit) <= 1
    assert np.abs(res.q - oq).max() < 1e-5
