"""The .bed/.bim/.fam front end (the SnpArray(filename) + SnpLinAlg step of
src/driver.jl:148-151; byte layout of src/loops.jl:55-71): round trips, the
checks that refuse corrupt files, and the first-I / first-2J subsetting with
the whole file's row stride (src/cuda/structs.jl:37 uploads the full matrix).
CPU only."""
import os

import numpy as np
import pytest

from haplo_gb300 import bed as bedio


def _random_genotypes(N, M, seed, miss=0.05):
    rng = np.random.default_rng(seed)
    G = rng.integers(0, 3, size=(N, M)).astype(np.int8)
    G[rng.random((N, M)) < miss] = -1
    return G


@pytest.mark.parametrize("N,M", [(1, 2), (4, 6), (7, 10), (130, 33)])
def test_write_read_round_trip(tmp_path, N, M):
    G = _random_genotypes(N, M, seed=N + M)
    data = bedio.encode_genotypes(G)
    assert data.shape == (M, (N + 3) // 4)
    path = bedio.write_bed(str(tmp_path / "c"), data, N)
    got, n, m = bedio.read_bed(path)
    assert (n, m) == (N, M)
    np.testing.assert_array_equal(got, data)
    np.testing.assert_array_equal(bedio.genotype_matrix(got, N), G)


def test_codes_and_padding_bits():
    # individual i in byte i>>2, bits 2(i&3); 0b00 hom A1, 0b01 missing, 0b10 het, 0b11 hom A2
    G = np.array([[0], [-1], [1], [2], [2]], dtype=np.int8)
    data = bedio.encode_genotypes(G)
    assert data.tolist() == [[0b11100100, 0b00000011]]      # padding bits of the last byte are zero


def test_bad_magic(tmp_path):
    data = bedio.encode_genotypes(_random_genotypes(8, 4, seed=1))
    path = bedio.write_bed(str(tmp_path / "c"), data, 8)
    raw = bytearray(open(path, "rb").read())
    raw[2] = 0x00                      # individual-major mode byte: not supported
    open(path, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="magic"):
        bedio.read_bed(path)
    open(path, "wb").write(b"\x6c")    # shorter than the magic
    with pytest.raises(ValueError, match="magic"):
        bedio.read_bed(path)


def test_truncated_body(tmp_path):
    data = bedio.encode_genotypes(_random_genotypes(9, 6, seed=2))
    path = bedio.write_bed(str(tmp_path / "c"), data, 9)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:-1])
    with pytest.raises(ValueError, match="data bytes"):
        bedio.read_bed(path)


def test_fam_bim_count_mismatch(tmp_path):
    data = bedio.encode_genotypes(_random_genotypes(12, 5, seed=3))
    path = bedio.write_bed(str(tmp_path / "c"), data, 12)
    with open(str(tmp_path / "c.bim"), "a") as f:          # one SNP more than the .bed holds
        f.write("1\tsnpX\t0\t99\tA\tB\n")
    with pytest.raises(ValueError, match="data bytes"):
        bedio.read_bed(path)
    path2 = bedio.write_bed(str(tmp_path / "d"), data, 12)
    with open(str(tmp_path / "d.fam"), "a") as f:          # 13 individuals: 4 bytes per SNP, not 3
        f.write("famX indX 0 0 0 -9\n")
    with pytest.raises(ValueError, match="data bytes"):
        bedio.read_bed(path2)


def test_missing_fam_needs_count(tmp_path):
    data = bedio.encode_genotypes(_random_genotypes(8, 4, seed=4))
    path = bedio.write_bed(str(tmp_path / "c"), data, 8)
    os.remove(str(tmp_path / "c.fam"))
    with pytest.raises(ValueError, match="fam"):
        bedio.read_bed(path)
    got, n, m = bedio.read_bed(path, n_individuals=8)
    assert (n, m) == (8, 4)
    np.testing.assert_array_equal(got, data)


@pytest.mark.parametrize("N,M,I,J", [(23, 14, 10, 5), (40, 20, 37, 9), (9, 8, 9, 4), (64, 30, 1, 1)])
def test_subsetting_uses_file_row_stride(O, N, M, I, J):
    """The fit reads the first I individuals and first 2J SNPs in place, with
    the file's ceil(N/4) bytes per SNP: its genotype-pair census equals that of
    a file holding only that corner."""
    G = _random_genotypes(N, M, seed=N * M + I)
    full = bedio.encode_genotypes(G)
    corner = bedio.encode_genotypes(G[:I, :2 * J])
    b_full = O.Bed(full, I, J, n_snp=M)
    b_corner = O.Bed(corner, I, J)
    np.testing.assert_array_equal(O.census(b_full), O.census(b_corner))
    assert int(O.census(b_full).sum()) == I * J
    # per-pair class counts by direct decoding
    g = bedio.genotype_matrix(full, N)[:I, :2 * J]
    code = np.where(g < 0, 3, g).astype(np.int64)
    want = np.bincount((code[:, 0::2] * 4 + code[:, 1::2]).ravel(), minlength=16)
    np.testing.assert_array_equal(O.census(b_full).astype(np.int64), want)


def test_double_missing_counts_the_whole_file(O):
    """count_double_missing! (src/utils.jl:1-18) counts over every SNP pair of
    the file, not only the first 2J SNPs."""
    G = _random_genotypes(12, 10, seed=9, miss=0.4)
    full = bedio.encode_genotypes(G)
    b = O.Bed(full, 12, 2, n_snp=10)
    want = ((G[:, 0::2] < 0) & (G[:, 1::2] < 0)).sum(axis=1)
    np.testing.assert_array_equal(O.double_missing(b), want)


def test_run_admixture_checks_before_any_device_work(tmp_path):
    from haplo_gb300.admix import run_admixture
    data = bedio.encode_genotypes(_random_genotypes(8, 6, seed=5))
    path = bedio.write_bed(str(tmp_path / "c"), data, 8)
    with pytest.raises(ValueError, match=".bed"):
        run_admixture(str(tmp_path / "c.bim"), 8, 3, 2)
    with pytest.raises(ValueError, match="individuals"):
        run_admixture(path, 9, 3, 2)
    with pytest.raises(ValueError, match="SNPs"):
        run_admixture(path, 8, 4, 2)
