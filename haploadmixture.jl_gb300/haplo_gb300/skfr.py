"""AIM selection before the fit: run_admixture's `sparsity` branch
(src/driver.jl:60-73 and _filter_SKFR, 84-105).

select_aims runs sparse k-means with feature ranking on the GPU (hx_skfr in
include/haplo_gb300.h) and returns the clusters and the sorted indices of the
2 * sparsity selected SNPs (blocks of 2 adjacent SNPs, as the reference's
blocksize = 2).  filter_bed keeps every individual and only those SNPs, the
SnpArrays.filter(prefix, trues(I), aims_sorted) step; write_filtered writes
the result as `<prefix>_<K>_<2*sparsity>aims.bed/.bim/.fam`, the reference's
file name (src/driver.jl:100-103).
"""
import ctypes as C

import numpy as np

from . import _lib
from . import bed as bedio


def select_once(bed, I, K, sparsity, seed=0, max_iter=50, device=0):
    """One run of hx_skfr: (clusters (I,) int32, aims (2*sparsity,) int64
    sorted, iterations, within-cluster sum of squares over the kept SNPs)."""
    b = np.ascontiguousarray(bed, dtype=np.uint8)
    if b.ndim != 2:
        raise ValueError("bed must be a (n_snp, bytes_per_snp) matrix")
    clusters = np.zeros(int(I), dtype=np.int32)
    aims = np.zeros(2 * int(sparsity), dtype=np.int64)
    it = C.c_int32()
    obj = C.c_double()
    st = _lib.load().hx_skfr(_lib.ptr(b), b.shape[1], b.shape[0], int(I), int(K), int(sparsity), int(max_iter),
                             int(seed) % (1 << 64), int(device), _lib.ptr(clusters), _lib.ptr(aims), C.byref(it),
                             C.byref(obj))
    _lib.check(st)
    return clusters, aims, int(it.value), float(obj.value)


def select_aims(bed, I, K, sparsity, seed=0, max_iter=50, device=0, tries=1):
    """(clusters (I,) int32, aims (2*sparsity,) int64 sorted, iterations) for
    the first I individuals of a (n_snp, ceil(N/4)) uint8 BED matrix.  With
    tries > 1 (the reference's skfr_tries, sparsekmeans_repeat), the runs
    start from seeds seed + 1000 t and the one with the smallest within-
    cluster sum of squares is kept (the first on ties)."""
    best = None
    for t in range(max(1, int(tries))):
        r = select_once(bed, I, K, sparsity, seed=int(seed) + 1000 * t, max_iter=max_iter, device=device)
        if best is None or r[3] < best[3]:
            best = r
    return best[0], best[1], best[2]


def filter_bed(bed, snps):
    """Rows `snps` (sorted SNP indices) of the SNP-major matrix, all individuals."""
    return np.ascontiguousarray(np.asarray(bed)[np.asarray(snps, dtype=np.int64)])


def write_filtered(prefix, bed, n_individuals, K, aims):
    """Writes the selected SNPs as <prefix>_<K>_<len(aims)>aims.bed (+ .bim/.fam);
    returns the .bed path."""
    des = "%s_%d_%daims" % (prefix, int(K), len(aims))
    return bedio.write_bed(des, filter_bed(bed, aims), n_individuals)
