"""The benchmark configurations at their own sizes, against the oracle.

* config 2 (100 Mbp, 150 bp, SMEM k=19): all 1,000,000 reads against the
  oracle's containment-stopped walk, and 20,000 against its unpruned walk;
* config 3 (3.1 Gbp, mixed lengths, SMEM k=19): 1,000,000 reads against the
  oracle with every kernel, with the text structures and without them (the
  sampled-SA walk); over 200,000 reads the size-independent property that
  every reported position spells the seed: the forward seed's read substring
  (or the reverse complement of a reverse seed's) occurs in the reference at
  that position, non-ACGT read bases skipped as the wildcard rule reads them;
* config 4 (the same 3.1 Gbp reference, log-normal 500 bp - 10 kbp reads, MEM
  k=20): 20,000 reads against the oracle with every kernel.

The oracle seeds from the GPU's 13-mer table (a copy; the interval of a
13-mer does not depend on who computes it, and test_kmer_table_matches_oracle
checks the table itself) so that a million reads take seconds on the host.
"""
import os

import numpy as np
import pytest

import pyoracle

pytestmark = pytest.mark.gpu


def _gpu_index(tmp, codes, name):
    import gpuseed_gb300 as gs
    prefix = os.path.join(str(tmp), name)
    idx = gs.build_index(codes, 7, prefix=prefix)
    idx.set_text(4)         # full SA, text and ISA samples: locate and text mode use them
    return prefix, idx


def _compare(gres, ob, n):
    assert gres.n_reads == ob.n_reads == n
    for r in range(n):
        assert gres.read_records(r) == ob.read_records(r), f"read {r}"


def _mismatches(gres, ob, r0=0):
    """reads of the oracle batch whose records differ from the GPU result's"""
    return pyoracle.mismatched_reads(ob, gres.seeds, gres.pos, gres.read_seed_off,
                                     gres.read_pos_off, r0=r0, cols=(0, 1, 2, 3, 6))


@pytest.fixture(scope="module")
def human(built, tmp_path_factory):
    """The 3.1 Gbp config-3 reference, its GPU-built index with text
    structures, the oracle on the same files and the GPU's 13-mer table."""
    from gpuseed_gb300 import workloads as W
    tmp = tmp_path_factory.mktemp("human")
    codes, nmask = W.make_reference(W.ref_spec(3))
    prefix, idx = _gpu_index(tmp, codes, "cfg3")
    assert idx.info().seq_len == 3_100_000_000
    oidx = pyoracle.Index(prefix)
    yield dict(codes=codes, nmask=nmask, prefix=prefix, idx=idx, oidx=oidx,
               table=idx.kmer_table())
    idx.close()


def test_config2_full(built, tmp_path):
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    codes, nmask = W.make_reference(W.ref_spec(2))
    prefix, idx = _gpu_index(tmp_path, codes, "cfg2")
    seqs, offs, lens = W.make_reads(codes, nmask, W.read_spec(2))
    assert lens.size == 1_000_000
    assert any(b"N" in seqs[int(o):int(o) + int(n)].tobytes() for o, n in zip(offs[:20_000], lens))
    ctx = gs.Context(idx)
    oidx = pyoracle.Index(prefix)
    ob = oidx.seed(seqs, offs, lens, k=19, smem=True, pruned=True, table=idx.kmer_table())
    for kernel in (0, 1, 2):
        bad = _mismatches(ctx.seed(seqs, offs, lens, k=19, smem=True, kernel=kernel), ob)
        assert bad.size == 0, (kernel, bad[:10])
    # the unpruned checker walk on a subset
    m = 20_000
    ob = oidx.seed(seqs, offs[:m], lens[:m], k=19, smem=True)
    bad = _mismatches(ctx.seed(seqs, offs[:m], lens[:m], k=19, smem=True), ob)
    assert bad.size == 0, bad[:10]


def test_config2_text_in_chunks(built, tmp_path):
    """The GPU-formatted records of a result larger than one 64 MiB copy-out
    chunk equal the host-formatted ones."""
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    codes, nmask = W.make_reference(W.ref_spec(2))
    prefix, idx = _gpu_index(tmp_path, codes, "cfg2t")
    seqs, offs, lens = W.make_reads(codes, nmask, W.read_spec(2, 400_000))
    ctx = gs.Context(idx)
    ctx.seed(seqs, offs, lens, k=19, smem=True)
    paths = []
    for host in (False, True):
        p = tmp_path / f"t{host}.txt"
        with open(p, "wb") as f:
            ctx.write_text(f.fileno(), 1, True, host=host)
        paths.append(p)
    assert paths[0].stat().st_size > (64 << 20)
    assert paths[0].read_bytes() == paths[1].read_bytes()


COMP = np.array([3, 2, 1, 0], np.uint8)


def test_config3_million_reads(human):
    """1M config-3 reads, every kernel, text structures on and off."""
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    idx, oidx = human["idx"], human["oidx"]
    seqs, offs, lens = W.make_reads(human["codes"], human["nmask"], W.read_spec(3, 1_000_000))
    ob = oidx.seed(seqs, offs, lens, k=19, smem=True, pruned=True, table=human["table"])
    ctx = gs.Context(idx)
    try:
        for kernel in (gs.KERNEL_BATCHED, gs.KERNEL_PLAIN, gs.KERNEL_LOCKSTEP):
            bad = _mismatches(ctx.seed(seqs, offs, lens, k=19, smem=True, kernel=kernel), ob)
            assert bad.size == 0, ("text", kernel, bad[:10])
        # the sampled-SA walk: locate by LF steps to a sampled row, no text mode
        idx.set_text(0)
        for kernel in (gs.KERNEL_BATCHED, gs.KERNEL_PLAIN):
            bad = _mismatches(ctx.seed(seqs, offs, lens, k=19, smem=True, kernel=kernel), ob)
            assert bad.size == 0, ("sampled SA", kernel, bad[:10])
    finally:
        idx.set_text(4)
        ctx.close()


def test_config3_positions_spell_seeds(human):
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    codes = human["codes"]
    seqs, offs, lens = W.make_reads(codes, human["nmask"], W.read_spec(3, 200_000))
    ctx = gs.Context(human["idx"])
    # bwa's LF: the reference's quirk at row primary+1 would misplace a walk
    # that passes through that row
    res = ctx.seed(seqs, offs, lens, k=19, smem=True, lf_mode=gs.LF_BWA)
    table = np.full(256, 255, np.uint8)
    for i, ch in enumerate(b"ACGT"):
        table[ch] = i
        table[ch + 32] = i
    checked = 0
    for r in range(lens.size):
        read = table[seqs[int(offs[r]):int(offs[r]) + int(lens[r])]]
        for x, y, l, u, poss in res.read_records(r):
            b, e = x & 0x7FFFFFFF, y & 0x7FFFFFFF
            seg = read[b:e]
            if y >> 31:
                seg = COMP[seg[::-1][seg[::-1] != 255]]
            else:
                seg = seg[seg != 255]
            for p in poss[:4]:
                assert np.array_equal(codes[p:p + seg.size], seg), (r, x, y, p)
                checked += 1
    assert checked > 200_000
    ctx.close()


def test_config4_full_size(human):
    """Config 4 as stated: log-normal long reads (median 2 kbp, 500 bp - 10 kbp,
    2% substitutions, 1% indels) over the 3.1 Gbp reference, MEM, k=20."""
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    seqs, offs, lens = W.make_reads(human["codes"], human["nmask"], W.read_spec(4, 20_000))
    assert lens.min() >= 500 and lens.max() <= 10_000
    ob = human["oidx"].seed(seqs, offs, lens, k=20, smem=False, pruned=True, table=human["table"])
    ctx = gs.Context(human["idx"])
    for kernel in (gs.KERNEL_BATCHED, gs.KERNEL_PLAIN, gs.KERNEL_LOCKSTEP):
        bad = _mismatches(ctx.seed(seqs, offs, lens, k=20, smem=False, kernel=kernel), ob)
        assert bad.size == 0, (kernel, bad[:10])
    ctx.close()


def test_very_long_reads(built, tmp_path):
    """Reads of 50-100 kbp (one an exact 80 kbp copy, whose last candidate walks
    80,000 steps) over a 400 kbp reference with a 20 kbp duplicated segment:
    every kernel gives the oracle's seeds (its containment-stopped walk: the
    unpruned one would take ~10^9 steps on the exact read)."""
    import gpuseed_gb300 as gs
    rng = np.random.default_rng(0x10C5)
    codes = rng.integers(0, 4, 400_000, dtype=np.uint8)
    codes[300_000:320_000] = codes[100_000:120_000]
    prefix, idx = _gpu_index(tmp_path, codes, "long")
    text = np.frombuffer(b"ACGT", np.uint8)[codes]
    reads = []
    for L in (50_000, 70_000, 100_000):
        st = int(rng.integers(0, codes.size - L))
        s = text[st:st + L].copy()
        errs = rng.random(L) < 0.005
        s[errs] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(errs.sum()))]
        reads.append(s.tobytes())
    reads.append(text[90_000:170_000].tobytes())          # exact, spans the duplicated segment
    reads.append(b"ACGT" * 10 + text[5_000:60_000].tobytes())
    lens = np.array([len(r) for r in reads], np.uint32)
    offs = np.concatenate([[0], np.cumsum(lens[:-1])]).astype(np.uint64)
    seqs = b"".join(reads)
    ctx = gs.Context(idx)
    oidx = pyoracle.Index(prefix)
    for smem, k in ((True, 19), (False, 20)):
        ob = oidx.seed(seqs, offs, lens, k=k, smem=smem, pruned=True)
        for kernel in (0, 1, 2):
            _compare(ctx.seed(seqs, offs, lens, k=k, smem=smem, kernel=kernel), ob, lens.size)
