"""The CPU oracle of the AIM selection (oracle/skfr_oracle.py): on a planted
cohort, where only some 2-SNP blocks differ between populations, it keeps
those blocks and recovers the populations; the standardisation and the
random stream behave as stated.  CPU only."""
import numpy as np
import pytest

from oracle import skfr_oracle as S


def planted(I, nb, K, informative, seed, miss=0.01):
    """BED matrix of I unadmixed individuals (population i % K), 2*nb SNPs:
    blocks in `informative` have population-specific haplotype frequencies,
    all others one shared distribution."""
    from oracle import oracle as O
    from haplo_gb300 import synth
    rng = np.random.default_rng(seed)
    Q = np.zeros((K, I))
    Q[np.arange(I) % K, np.arange(I)] = 1.0
    shared = rng.dirichlet(np.ones(4), size=nb)
    P = np.repeat(shared[None], K, axis=0)
    for j in informative:
        P[:, j, :] = rng.dirichlet(np.full(4, 0.3), size=K)
    P = np.asfortranarray(P.reshape(K, 4 * nb))
    cq, cp = synth.cumulative(np.asfortranarray(Q), P)
    return O.synth(seed + 1, I, nb, cq, cp, miss)


def test_planted_blocks_and_populations_are_recovered(O):
    I, nb, K = 300, 120, 3
    inf = np.arange(5, 120, 8)                      # 15 informative blocks
    bed = planted(I, nb, K, inf, seed=3)
    clusters, aims, it = S.select(bed, I, K, sparsity=len(inf), seed=1, max_iter=50)
    assert aims.shape == (2 * len(inf),) and np.all(np.diff(aims) > 0)
    kept_blocks = set((aims // 2).tolist())
    assert len(kept_blocks & set(inf.tolist())) >= len(inf) - 1
    truth = np.arange(I) % K
    for k in range(K):                              # each population lands in one cluster
        labels = clusters[truth == k]
        assert np.bincount(labels, minlength=K).max() >= 0.95 * labels.size
    assert len(set(int(np.bincount(clusters[truth == k], minlength=K).argmax()) for k in range(K))) == K
    assert 1 <= it <= 50


def test_deterministic_and_seeded(O):
    bed = planted(150, 40, 2, np.arange(0, 40, 5), seed=4)
    a = S.select(bed, 150, 2, 6, seed=9)
    b = S.select(bed, 150, 2, 6, seed=9)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_tables_standardise_observed_genotypes():
    # SNP 0: genotypes 0, 1, 2, missing, 2 -> mean 1.25, n-1 sd over the 4 observed
    code = np.array([[0], [2], [3], [1], [3]], dtype=np.uint8)
    T = S.tables(code)
    g = np.array([0.0, 1.0, 2.0, 2.0])
    mu, sd = g.mean(), g.std(ddof=1)
    assert T[0, 0] == pytest.approx((0 - mu) / sd, rel=1e-15)
    assert T[0, 2] == pytest.approx((1 - mu) / sd, rel=1e-15)
    assert T[0, 3] == pytest.approx((2 - mu) / sd, rel=1e-15)
    assert T[0, 1] == 0.0
    # monomorphic and nearly empty SNPs carry no information
    np.testing.assert_array_equal(S.tables(np.array([[0], [0], [1]], dtype=np.uint8)), np.zeros((1, 4)))
    np.testing.assert_array_equal(S.tables(np.array([[3], [1], [1]], dtype=np.uint8)), np.zeros((1, 4)))


def test_uniform_stream():
    u = [S.uniform(123, t) for t in range(1000)]
    assert all(0.0 <= x < 1.0 for x in u)
    assert abs(np.mean(u) - 0.5) < 0.05
    # SplitMix64 of 0: the published first output of the generator seeded with 0
    assert S.splitmix(0) == 0xE220A8397B1DCDAF


def test_rejects_bad_sizes(O):
    bed = planted(20, 6, 2, [1], seed=5)
    with pytest.raises(ValueError):
        S.select(bed, 20, 21, 2)
    with pytest.raises(ValueError):
        S.select(bed, 20, 2, 7)
