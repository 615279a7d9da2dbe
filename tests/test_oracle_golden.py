"""The oracle against the committed golden fixtures (exact-rational
transcription of src/loops.jl, tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden_small.json")))


def test_pair_terms_match_golden(O):
    for t in GOLD["pair_terms"]:
        out = O.pair_terms(t["g1"], t["g2"], t["qp"])
        assert out[0] == pytest.approx(t["ll"], rel=1e-13, abs=1e-13)   # formula 2 (loops.jl:254)
        assert out[1] == pytest.approx(t["ll"], rel=1e-13, abs=1e-13)   # formula 1 (loops.jl:157-212)
        np.testing.assert_allclose(out[2:], t["c"], rtol=1e-13, atol=1e-15)


def test_expected_counts_sum_to_two(O):
    # every class except missing/missing distributes exactly two haplotype copies
    for t in GOLD["pair_terms"]:
        s = sum(t["c"])
        if t["g1"] == 3 and t["g2"] == 3:
            assert s == 0.0
        else:
            assert s == pytest.approx(2.0, rel=1e-14)


def test_counts_are_qp_times_dlogL(O):
    # c_h = qp_h * d log L / d qp_h for all 16 classes (finite difference)
    qp = np.array([0.11, 0.27, 0.19, 0.43])
    for g1 in range(4):
        for g2 in range(4):
            base = O.pair_terms(g1, g2, qp)
            for h in range(4):
                e = 1e-7 * qp[h]
                qq = qp.copy()
                qq[h] += e
                fd = (O.pair_terms(g1, g2, qq)[0] - base[0]) / e
                assert qp[h] * fd == pytest.approx(base[2 + h], rel=2e-6, abs=1e-9)


@pytest.fixture(scope="module")
def gold_cohort(O):
    c = GOLD["cohort"]
    bed = np.array(c["bed"], dtype=np.uint8)
    b = O.Bed(bed, c["I"], c["J"])
    q = np.array(c["q"])
    p = np.array(c["p"])
    return c, b, q, p


def test_cohort_loglik(O, gold_cohort):
    c, b, q, p = gold_cohort
    for formula in (1, 2):
        assert O.loglik(b, c["K"], q, p, formula=formula) == pytest.approx(c["loglik"], rel=1e-13)


def test_cohort_accumulations(O, gold_cohort):
    c, b, q, p = gold_cohort
    K = c["K"]
    XtX, Xtz = O.accum_q(b, K, q, p)
    np.testing.assert_allclose(Xtz, np.array(c["Xtz_q"]), rtol=1e-12)
    np.testing.assert_allclose(XtX, np.transpose(np.array(c["XtX_q"]), (0, 1, 2)), rtol=1e-12)
    XtX, Xtz = O.accum_p(b, K, q, p)
    np.testing.assert_allclose(Xtz, np.array(c["Xtz_p"]), rtol=1e-12)
    np.testing.assert_allclose(XtX, np.array(c["XtX_p"]), rtol=1e-12)
    qn, pn = O.em_accum(b, K, q, p)
    np.testing.assert_allclose(qn, np.array(c["em_q"]), rtol=1e-12)
    np.testing.assert_allclose(pn, np.array(c["em_p"]), rtol=1e-12)


def test_census_matches_decode(O, gold_cohort):
    from haplo_gb300 import bed as bedio
    c, b, q, p = gold_cohort
    G = bedio.genotype_matrix(b.data, c["I"]).astype(int)
    G[G == -1] = 3
    want = np.zeros(16, dtype=np.uint64)
    for j in range(c["J"]):
        for i in range(c["I"]):
            want[G[i, 2 * j] * 4 + G[i, 2 * j + 1]] += 1
    np.testing.assert_array_equal(O.census(b), want)
