"""PLINK 1 binary genotype files (.bed/.bim/.fam), SNP-major.

The on-disk layout is the one SnpArrays exposes as SnpArray.data (used by the
reference at src/loops.jl:57-58 and src/cuda/structs.jl:37): after the magic
bytes 0x6C 0x1B 0x01, one row of ceil(N/4) bytes per SNP; individual i sits in
byte i>>2 at bit offset 2*(i&3); codes 0b00 hom A1, 0b01 missing, 0b10 het,
0b11 hom A2.  Padding bits of the last byte are zero.
"""
import os

import numpy as np

MAGIC = bytes([0x6C, 0x1B, 0x01])


def _count_lines(path):
    with open(path, "rb") as f:
        return sum(1 for line in f if line.strip())


def read_bed(path, n_individuals=None, n_snps=None):
    """Returns (data, N, M): data is a uint8 array of shape (M, ceil(N/4)).

    N and M default to the line counts of the sibling .fam and .bim files."""
    stem = path[:-4] if path.endswith(".bed") else path
    if n_individuals is None:
        fam = stem + ".fam"
        if not os.path.exists(fam):
            raise ValueError("no .fam next to %s; pass n_individuals" % path)
        n_individuals = _count_lines(fam)
    bps = (n_individuals + 3) // 4
    raw = np.fromfile(stem + ".bed", dtype=np.uint8)
    if raw.size < 3 or bytes(raw[:3]) != MAGIC:
        raise ValueError("%s: not a SNP-major PLINK 1 .bed (bad magic bytes)" % path)
    body = raw[3:]
    if n_snps is None:
        bim = stem + ".bim"
        n_snps = _count_lines(bim) if os.path.exists(bim) else body.size // bps
    if body.size != bps * n_snps:
        raise ValueError("%s: %d data bytes, expected %d x %d" % (path, body.size, n_snps, bps))
    return body.reshape(n_snps, bps), n_individuals, n_snps


def write_bed(prefix, data, n_individuals):
    """Writes prefix.bed (+ minimal .bim/.fam) from a (M, ceil(N/4)) uint8 array."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    M = data.shape[0]
    with open(prefix + ".bed", "wb") as f:
        f.write(MAGIC)
        f.write(data.tobytes())
    with open(prefix + ".bim", "w") as f:
        for s in range(M):
            f.write("1\tsnp%d\t0\t%d\tA\tB\n" % (s + 1, s + 1))
    with open(prefix + ".fam", "w") as f:
        for i in range(n_individuals):
            f.write("fam%d ind%d 0 0 0 -9\n" % (i + 1, i + 1))
    return prefix + ".bed"


def genotype_matrix(data, N):
    """Decodes to an (N, M) int8 matrix of allele-2 counts, missing = -1
    (src/loops.jl:62-71).  For small inputs and tests."""
    M = data.shape[0]
    shifts = np.arange(4, dtype=np.uint8) * 2
    codes = (data[:, :, None] >> shifts[None, None, :]) & 3
    codes = codes.reshape(M, -1)[:, :N].T
    lut = np.array([0, -1, 1, 2], dtype=np.int8)
    return lut[codes]


def encode_genotypes(G):
    """Inverse of genotype_matrix: (N, M) counts in {0,1,2,-1} -> (M, ceil(N/4)) bytes."""
    G = np.asarray(G)
    N, M = G.shape
    code = np.select([G == 0, G == -1, G == 1, G == 2], [0, 1, 2, 3]).astype(np.uint8)
    pad = (-N) % 4
    if pad:
        code = np.vstack([code, np.zeros((pad, M), dtype=np.uint8)])
    code = code.T.reshape(M, -1, 4)
    out = code[:, :, 0] | (code[:, :, 1] << 2) | (code[:, :, 2] << 4) | (code[:, :, 3] << 6)
    return np.ascontiguousarray(out.astype(np.uint8))
