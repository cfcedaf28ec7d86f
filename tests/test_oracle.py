"""The CPU oracle, pinned before it is trusted.

* its suffix arrays against a naive sort,
* its occurrence counts against a direct count over the BWT,
* its seeds against the committed golden records (tests/golden, produced by
  the brute-force substring matcher, no FM index involved),
* its seeds against the brute-force matcher on fresh random cases,
* its containment-stopped walk (CPU baseline) against its full walk.
"""
import os

import numpy as np
import pytest

import bruteforce as bf
import pyoracle
from helpers import build_index, pack, random_reference, sample_reads

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_suffix_array_naive(built):
    for n, seed in ((1, 0), (2, 1), (17, 2), (300, 3), (2000, 4)):
        codes = random_reference(n, seed) if n > 2 else np.array([1, 1][:n], np.uint8)
        text = "".join("ACGT"[c] for c in codes)
        sa = pyoracle.suffix_array(codes)
        assert list(sa) == sorted(range(n + 1), key=lambda p: text[p:])
    homo = np.zeros(500, np.uint8)
    assert list(pyoracle.suffix_array(homo)) == list(range(500, -1, -1))


def test_occ_and_lf(built, tmp_path):
    codes = random_reference(3000, 5)
    prefix = build_index(tmp_path, codes, sa_intv=5)
    idx = pyoracle.Index(prefix)
    sa = pyoracle.suffix_array(codes)
    n = codes.size
    bwt = [(-1 if p == 0 else int(codes[p - 1])) for p in sa]
    cum = np.zeros((n + 2, 4), np.int64)
    for r, c in enumerate(bwt):
        cum[r + 1] = cum[r]
        if c >= 0:
            cum[r + 1, c] += 1
    for k in list(range(0, n + 1, 7)) + [idx.primary - 1, idx.primary, idx.primary + 1, n]:
        for c in range(4):
            assert idx.occ(k, c) == cum[k + 1, c]
    assert idx.occ(0xFFFFFFFF, 2) == 0
    inv = np.empty(n + 1, np.int64)
    inv[sa] = np.arange(n + 1)
    for row in range(n + 1):
        exp_lf = 0 if sa[row] == 0 else inv[sa[row] - 1]
        assert idx.lf(row, pyoracle.LF_BWA) == exp_lf
        got = idx.lf(row, pyoracle.LF_GPUSEED)
        assert got == (0 if row == idx.primary + 1 else exp_lf)
        p, _ = idx.locate(row, pyoracle.LF_BWA)
        assert p == (sa[row] if row else 0xFFFFFFFF)


@pytest.fixture(scope="module")
def golden(built, tmp_path_factory):
    text = open(os.path.join(GOLD, "ref20k.txt")).read().strip()
    codes = np.array(["ACGT".index(ch) for ch in text], np.uint8)
    d = tmp_path_factory.mktemp("gold")
    prefix = build_index(d, codes, sa_intv=7)
    reads = [ln.strip().encode() for ln in open(os.path.join(GOLD, "reads60.fa")) if not ln.startswith(">")]
    return pyoracle.Index(prefix), reads, d


@pytest.mark.parametrize("smem", [False, True], ids=["mem", "smem"])
@pytest.mark.parametrize("n_stop", [False, True], ids=["nwild", "nstop"])
@pytest.mark.parametrize("pruned", [False, True], ids=["full", "pruned"])
def test_golden_records(golden, smem, n_stop, pruned):
    idx, reads, d = golden
    seqs, offs, lens = pack(reads)
    b = idx.seed(seqs, offs, lens, k=19, smem=smem, n_mode=int(n_stop), lf_mode=pyoracle.LF_BWA,
                 pruned=pruned, threads=2)
    out = os.path.join(str(d), "o.txt")
    b.write_text(out, 1, smem)
    name = "k19_%s_%s.txt" % ("smem" if smem else "mem", "nstop" if n_stop else "nwild")
    assert open(out).read() == open(os.path.join(GOLD, name)).read()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_bruteforce_random(built, tmp_path, seed):
    n = (700, 2500, 6000)[seed - 1]
    codes = random_reference(n, 100 + seed)
    text = "".join("ACGT"[c] for c in codes)
    prefix = build_index(tmp_path, codes, sa_intv=3 + seed)
    idx = pyoracle.Index(prefix)
    reads = sample_reads(codes, 25, seed=seed, lengths=(13, 14, 20, 45, 90))
    seqs, offs, lens = pack(reads)
    for k in (13, 16, 20):
        for smem in (False, True):
            for n_stop in (False, True):
                b = idx.seed(seqs, offs, lens, k=k, smem=smem, n_mode=int(n_stop),
                             lf_mode=pyoracle.LF_BWA, threads=2)
                bp = idx.seed(seqs, offs, lens, k=k, smem=smem, n_mode=int(n_stop),
                              lf_mode=pyoracle.LF_BWA, pruned=True, threads=2)
                for r in range(len(reads)):
                    got = [(x, y, ps) for (x, y, l, u, ps) in b.read_records(r)]
                    assert got == bf.seed_read(text, reads[r], k, smem, n_stop)
                    assert bp.read_records(r) == b.read_records(r)
                assert bp.work["n_steps"] <= b.work["n_steps"]


def test_kmer_table_small(built, tmp_path):
    codes = random_reference(4000, 9)
    prefix = build_index(tmp_path, codes)
    idx = pyoracle.Index(prefix)
    text = "".join("ACGT"[c] for c in codes)
    t = idx.kmer_table(5)
    for patt in range(0, 1 << 10, 13):
        s = "".join("ACGT"[(patt >> (2 * j)) & 3] for j in range(5))[::-1]
        cnt = len(bf.occurrences(text, s))
        l, u = int(t[2 * patt]), int(t[2 * patt + 1])
        assert (u - l + 1 if l <= u else 0) == cnt
