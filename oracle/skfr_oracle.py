"""CPU oracle of the SKFR AIM selection (test infrastructure only).

The reference selects ancestry-informative markers before the fit with
SparseKmeansFeatureRanking 0.1.2 (src/driver.jl:60-73, 84-105:
ImputedSnpMatrix{Float64}(g, K; rng, blocksize=2), then sparsekmeans1(ISM,
sparsity; max_iter) -> (clusters, _, aims, _, _), then SnpArrays.filter to the
sorted aims).  That package is not in this tree, so this restates the
published method, sparse k-means with feature ranking (Zhang, Lange and Xu,
NeurIPS 2020, algorithm SKFR1), with the choices below written out:

* features: the genotype of each SNP, standardised over the individuals that
  are not missing, x = (g - mean) / sd with the n-1 standard deviation;
  missing genotypes take the mean (x = 0); SNPs with fewer than two
  observations or no variance are 0 everywhere;
* blocks of 2 adjacent SNPs (blocksize = 2): a block's score is the sum of its
  SNPs' scores, and `sparsity` blocks (2 * sparsity SNPs) are kept;
* start: k-means++ over all SNPs, the uniform draws taken from a counter-based
  SplitMix64 stream of the seed (draw t = mix(seed + t), 53-bit uniform);
* iteration: cluster means from the current assignment (an empty cluster keeps
  its centre); score of SNP l = sum_j n_j theta_jl^2; keep the top blocks
  (larger score first, lower index on ties); centres are 0 off the kept SNPs;
  reassign every individual to the nearest centre over the kept SNPs (lowest
  cluster index on ties); stop when no assignment changes or after max_iter
  iterations.

Every sum runs sequentially in index order with separate multiplies and adds,
and the cluster sums come from integer counts of genotype codes, so the GPU
implementation (hx_skfr) reproduces this one bit for bit.
"""
import numpy as np

TWO64 = 1 << 64


def splitmix(x):
    """SplitMix64 finaliser of x (Python int), as a Python int in [0, 2^64)."""
    z = (x + 0x9E3779B97F4A7C15) % TWO64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) % TWO64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) % TWO64
    return z ^ (z >> 31)


def uniform(seed, t):
    """The t-th uniform draw in [0, 1) of the stream."""
    return (splitmix((seed + t) % TWO64) >> 11) * (1.0 / (1 << 53))


def codes(bed, I):
    """(I, M) raw 2-bit codes of the first I individuals of a SNP-major matrix."""
    M = bed.shape[0]
    sh = np.arange(4, dtype=np.uint8) * 2
    c = (bed[:, :, None] >> sh[None, None, :]) & 3
    return np.ascontiguousarray(c.reshape(M, -1)[:, :I].T)


def tables(code):
    """T[l, c]: standardised value of raw code c at SNP l (code 1 = missing)."""
    I, M = code.shape
    n0 = (code == 0).sum(axis=0).astype(np.float64)
    n1 = (code == 2).sum(axis=0).astype(np.float64)     # heterozygote: genotype 1
    n2 = (code == 3).sum(axis=0).astype(np.float64)     # genotype 2
    T = np.zeros((M, 4))
    for l in range(M):
        nobs = n0[l] + n1[l] + n2[l]
        if nobs < 2.0:
            continue
        mu = (n1[l] * 1.0 + n2[l] * 2.0) / nobs
        var = (n0[l] * (mu * mu) + n1[l] * ((1.0 - mu) * (1.0 - mu)) + n2[l] * ((2.0 - mu) * (2.0 - mu))) / (nobs - 1.0)
        if not var > 0.0:
            continue
        sd = np.sqrt(var)
        T[l, 0] = (0.0 - mu) / sd
        T[l, 2] = (1.0 - mu) / sd
        T[l, 3] = (2.0 - mu) / sd
    return T


def _dist(x_rows, theta, snps):
    """Squared distances (n, K) over the SNPs `snps`, summed in their order."""
    n = x_rows.shape[0]
    K = theta.shape[1]
    d = np.zeros((n, K))
    for l in snps:
        diff = x_rows[:, l][:, None] - theta[l][None, :]
        d = d + diff * diff
    return d


def select(bed, I, K, sparsity, seed=0, max_iter=50, return_objective=False):
    """(clusters (I,), aims (2*sparsity,) sorted SNP indices, iterations), and
    with return_objective the within-cluster sum of squares over the kept
    SNPs (each individual's distance to its centre, summed in order)."""
    M = bed.shape[0] - bed.shape[0] % 2
    nb = M // 2
    if not (1 <= K <= I) or not (1 <= sparsity <= nb):
        raise ValueError("need 1 <= K <= I and 1 <= sparsity <= SNP blocks")
    code = codes(bed[:M], I)
    T = tables(code)
    X = T[np.arange(M)[None, :], code]                 # (I, M)
    allsnp = range(M)
    # k-means++ start
    theta = np.zeros((M, K))
    c0 = min(int(uniform(seed, 0) * I), I - 1)
    theta[:, 0] = X[c0]
    d2 = _dist(X, theta[:, :1], allsnp)[:, 0]
    for t in range(1, K):
        cs = np.cumsum(d2)
        target = uniform(seed, t) * cs[-1]
        hit = np.nonzero(cs > target)[0]
        ct = int(hit[0]) if hit.size else I - 1
        theta[:, t] = X[ct]
        dt = _dist(X, theta[:, t:t + 1], allsnp)[:, 0]
        d2 = np.where(dt < d2, dt, d2)
    assign = np.argmin(_dist(X, theta, allsnp), axis=1)
    keep = None
    it = 0
    for it in range(1, max_iter + 1):
        n = np.bincount(assign, minlength=K).astype(np.float64)
        # cluster sums from integer code counts, in code order 0, 2, 3
        for j in range(K):
            if n[j] == 0:
                continue
            m = assign == j
            c0n = (code[m] == 0).sum(axis=0).astype(np.float64)
            c2n = (code[m] == 2).sum(axis=0).astype(np.float64)
            c3n = (code[m] == 3).sum(axis=0).astype(np.float64)
            s = ((c0n * T[:, 0]) + (c2n * T[:, 2])) + (c3n * T[:, 3])
            theta[:, j] = s / n[j]
        score = np.zeros(M)
        for j in range(K):
            score = score + n[j] * (theta[:, j] * theta[:, j])
        bscore = score[0::2] + score[1::2]
        order = np.lexsort((np.arange(nb), -bscore))
        kb = np.sort(order[:sparsity])
        keep = np.sort(np.concatenate([2 * kb, 2 * kb + 1]))
        mask = np.zeros(M, dtype=bool)
        mask[keep] = True
        theta[~mask] = 0.0
        dk = _dist(X, theta, keep)
        new = np.argmin(dk, axis=1)
        changed = bool(np.any(new != assign))
        assign = new
        if not changed:
            break
    out = (assign.astype(np.int32), keep.astype(np.int64), it)
    if return_objective:
        out = out + (float(np.cumsum(dk[np.arange(I), assign])[-1]),)
    return out
