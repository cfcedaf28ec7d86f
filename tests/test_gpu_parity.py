"""GPU seeding (through the C-ABI) against the CPU oracle, bit for bit.

Every case runs the CUDA path and the oracle on the same index files and the
same reads and compares, per read, every output seed (begin, end, strand bit,
SA interval) and every resolved reference position in output order.
Integer work: the tolerance is zero.
"""
import os
import subprocess

import numpy as np
import pytest

import pyoracle
from helpers import build_index, device_bytes, pack, random_reference, sample_reads

pytestmark = pytest.mark.gpu


def _gs():
    import gpuseed_gb300 as gs
    return gs


def assert_same(gres, obatch, n_reads, ctx=""):
    assert gres.n_reads == obatch.n_reads == n_reads
    for r in range(n_reads):
        g = gres.read_records(r)
        o = obatch.read_records(r)
        assert g == o, f"{ctx} read {r}: gpu {g[:4]} oracle {o[:4]}"


@pytest.fixture(scope="module")
def small(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("small")
    codes = random_reference(60_000, 7)
    prefix = build_index(d, codes, sa_intv=7)
    gs = _gs()
    gidx = gs.Index(prefix)
    gidx.set_text(4)        # the text structures are built on request
    oidx = pyoracle.Index(prefix)
    ctx = gs.Context(gidx)
    return dict(codes=codes, prefix=prefix, gidx=gidx, oidx=oidx, ctx=ctx, dir=d)


def test_kmer_table_matches_oracle(small):
    g = small["gidx"].kmer_table()
    o = small["oidx"].kmer_table(13)
    assert g.shape == o.shape
    assert np.array_equal(g, o)


@pytest.mark.parametrize("kernel", [0, 1, 2], ids=["batched", "plain", "lockstep"])
@pytest.mark.parametrize("smem", [False, True], ids=["mem", "smem"])
@pytest.mark.parametrize("n_mode", [0, 1], ids=["nwild", "nstop"])
def test_random_reads(small, kernel, smem, n_mode):
    reads = sample_reads(small["codes"], 400, seed=11 + kernel + 2 * n_mode,
                         lengths=(13, 14, 19, 20, 33, 64, 100, 150, 300))
    seqs, offs, lens = pack(reads)
    for k in (13, 19, 20, 31):
        for lf in (0, 1):
            gres = small["ctx"].seed(seqs, offs, lens, k=k, smem=smem, n_mode=n_mode, lf_mode=lf,
                                     kernel=kernel)
            ob = small["oidx"].seed(seqs, offs, lens, k=k, smem=smem, n_mode=n_mode, lf_mode=lf)
            assert_same(gres, ob, len(reads), f"k={k} lf={lf}")


def edge_reads(small):
    codes = small["codes"]
    text = "".join("ACGT"[c] for c in codes)
    sa = pyoracle.suffix_array(codes)
    primary = small["oidx"].primary
    q = int(sa[primary + 1])      # text position whose row is primary+1 (LF quirk)
    return [
        b"",                                   # empty read
        b"ACGT",                               # shorter than k
        text[1000:1020].encode(),              # exactly k
        text[2000:2013].encode(),              # exactly 13 bases
        b"A" * 80, b"C" * 40 + b"G" * 40,      # homopolymers
        text[5000:5150].encode(),              # exact forward match
        text[7000:7100].lower().encode(),      # lowercase letters
        (text[9000:9030] + "N" + text[9031:9080]).encode(),   # N after the 13-mer
        (text[9500:9505] + "N" + text[9506:9600]).encode(),   # N inside early 13-mers
        (text[11000:11050] + "\r").encode(),   # CR kept as a base, as getline gives it
        b"NNNNNNNNNNNNNNNNNNNNNNNNNNNNNN",
        text[max(0, q - 60):q + 60].encode(),  # walks through row primary+1
        text[max(0, q - 3):q + 40].encode(),
        text[:120].encode(), text[-120:].encode(),
        b"ACGTRYKMSWBDHV@X" * 4,               # other letters (codes 0 and 5)
    ]


def test_edge_cases(small):
    reads = edge_reads(small)
    seqs, offs, lens = pack(reads)
    for kernel in (0, 1, 2):
        for smem in (False, True):
            for lf in (0, 1):
                for k in (13, 20):
                    gres = small["ctx"].seed(seqs, offs, lens, k=k, smem=smem, lf_mode=lf,
                                             kernel=kernel)
                    ob = small["oidx"].seed(seqs, offs, lens, k=k, smem=smem, lf_mode=lf)
                    assert_same(gres, ob, len(reads), f"edge kernel={kernel} smem={smem} lf={lf} k={k}")


def test_text_structures(small):
    """The full suffix array, packed text and inverse-SA samples that
    gs_index_set_text builds in HBM from the .bwt and .sa equal the oracle's
    suffix array and the text."""
    gidx = small["gidx"]
    assert gidx.info().text_min > 0
    codes = small["codes"]
    n = codes.size
    sa = pyoracle.suffix_array(codes)
    want = sa.copy()
    want[0] = 0xffffffff                  # row 0 keeps the sa[0] sentinel
    assert np.array_equal(gidx.text_table(0), want)
    padded = np.zeros(((n + 15) // 16) * 16, np.uint32)
    padded[:n] = codes
    words = np.bitwise_or.reduce(padded.reshape(-1, 16) << (2 * np.arange(16, dtype=np.uint32)),
                                 axis=1)
    assert np.array_equal(gidx.text_table(1), words.astype(np.uint32))
    isa = np.empty(n + 1, np.int64)
    isa[sa.astype(np.int64)] = np.arange(n + 1)
    assert np.array_equal(gidx.text_table(2), isa[::2].astype(np.uint32))


def text_mode_reads(small):
    """Long exact copies (text mode runs far), copies with a wildcard or a
    substitution mid-way, copies at both ends of the text, random reads."""
    codes = small["codes"]
    text = "".join("ACGT"[c] for c in codes)
    n = len(text)
    rng = np.random.default_rng(5)
    reads = edge_reads(small)
    for L in (40, 90, 160, 300):
        for _ in range(6):
            a = int(rng.integers(0, n - L))
            s = text[a:a + L]
            reads.append(s.encode())
            j = int(rng.integers(5, L - 5))
            reads.append((s[:j] + "N" + s[j + 1:]).encode())
            reads.append((s[:j] + "ACGT"[("ACGT".index(s[j]) + 1) % 4] + s[j + 1:]).encode())
            reads.append((s[:j] + "NN" + s[j + 2:]).lower().encode())
        reads.append(text[:L].encode())
        reads.append(text[n - L:].encode())
        reads.append((text[:L // 2] + "N" + text[L // 2 + 1:L]).encode())
    reads += sample_reads(codes, 200, seed=73, lengths=(20, 33, 64, 100, 150, 300), err=0.01)
    return reads


@pytest.mark.parametrize("text_min", [1, 5, 16, -1, 0], ids=["t1", "t5", "t16", "locate", "off"])
def test_text_mode(small, text_min):
    """Text mode at several entry thresholds, the full-SA locate alone, and
    neither: every kernel, both modes, both N and LF modes, and every walk in
    the start pass (walker_slots < 0) give the oracle's seeds and positions."""
    gs = _gs()
    gidx = gs.Index(small["prefix"])
    gidx.set_text(text_min)
    assert gidx.info().text_min == (text_min if text_min > 0 else text_min and -1)
    ctx = gs.Context(gidx)
    reads = text_mode_reads(small)
    seqs, offs, lens = pack(reads)
    for kernel, slots in ((0, 0), (0, -1), (1, 0), (2, 0)):
        for smem in (False, True):
            for n_mode in (0, 1):
                for lf in (0, 1):
                    gres = ctx.seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode, lf_mode=lf,
                                    kernel=kernel, walker_slots=slots)
                    ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode,
                                            lf_mode=lf)
                    assert_same(gres, ob, len(reads),
                                f"text_min={text_min} kernel={kernel}/{slots} smem={smem} "
                                f"n_mode={n_mode} lf={lf}")


def test_text_build_checks_samples(small):
    """Building the text structures for an .sa whose samples do not continue
    the BWT's chains fails with GS_EFORMAT and leaves the index seeding by LF
    walks; the consistent files build them."""
    gs = _gs()
    prefix = small["prefix"]
    bwt = np.fromfile(prefix + ".bwt", dtype=np.uint32)
    sa = np.fromfile(prefix + ".sa", dtype=np.uint32)
    samples = sa[7:].copy()
    samples[[3, 4]] = samples[[4, 3]]
    gidx = gs.Index(arrays=(int(bwt[0]), bwt[1:5], bwt[5:], samples, int(sa[5])))
    assert gidx.info().text_min == 0
    with pytest.raises(gs.GsError) as e:
        gidx.set_text(24)
    assert e.value.code == -3        # GS_EFORMAT
    ok = gs.Index(arrays=(int(bwt[0]), bwt[1:5], bwt[5:], sa[7:], int(sa[5])))
    assert ok.info().text_min == 0      # not built at load
    ok.set_text(4)
    assert ok.info().text_min == 4


def test_empty_batch(small):
    gres = small["ctx"].seed(b"", np.zeros(0, np.uint64), np.zeros(0, np.uint32), k=20)
    assert gres.n_reads == 0 and gres.seeds.shape[0] == 0


def test_invalid_k(small):
    gs = _gs()
    seqs, offs, lens = pack([b"ACGTACGTACGTACGTACGT"])
    with pytest.raises(gs.GsError) as e:
        small["ctx"].seed(seqs, offs, lens, k=12)
    assert e.value.code == -1


def test_text_output_identical(small, tmp_path):
    """The -o records formatted on the GPU, by the host and by the oracle are
    the same bytes (short reads without seeds, repeats with many positions,
    read numbers that need every digit width and wrap past 2^32)."""
    text = "".join("ACGT"[c] for c in small["codes"])
    reads = sample_reads(small["codes"], 300, seed=5, lengths=(50, 100, 150))
    reads += [b"ACGTACGT", b"A" * 60, text[500:520].encode() * 4, b""]
    seqs, offs, lens = pack(reads)
    for smem in (False, True):
        for first in (1, 9_999_990, 4_294_967_000):
            small["ctx"].seed(seqs, offs, lens, k=19, smem=smem)
            outs = []
            for host in (False, True):
                path = tmp_path / f"g{smem}{host}.txt"
                with open(path, "wb") as f:
                    small["ctx"].write_text(f.fileno(), first, smem, host=host)
                outs.append(path.read_bytes())
            d, n = small["ctx"].text_device(first, smem)
            outs.append(device_bytes(d, n))
            ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem)
            opath = tmp_path / f"o{smem}.txt"
            ob.write_text(str(opath), first, smem)
            want = opath.read_bytes()
            for i, o in enumerate(outs):
                assert o == want, (smem, first, i)


def test_cli_matches_oracle(small, tmp_path):
    gs = _gs()
    reads = sample_reads(small["codes"], 200, seed=9, lengths=(40, 100))
    fa = tmp_path / "reads.fa"
    with open(fa, "wb") as f:
        for i, r in enumerate(reads):
            f.write(b">r%d\n%s\n" % (i, r))
    seqs, offs, lens = pack(reads)
    for smem in (False, True):
        ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem)
        opath = tmp_path / "o.txt"
        ob.write_text(str(opath), 1, smem)
        # default batch, and batches of one read, ~10 reads, ~70 reads (the
        # reader thread parses the next batch while one is seeded), with and
        # without the text structures (-T)
        for batch in ([], ["-B", "1"], ["-B", "1000"], ["-B", "7000"], ["-T"], ["-T", "-B", "1000"]):
            args = ([gs.CLI_PATH, "-k", "19"] + (["-s"] if smem else []) + batch +
                    ["-o", small["prefix"], str(fa)])
            out = subprocess.run(args, capture_output=True, check=True).stdout
            assert out == opath.read_bytes(), batch
    empty = tmp_path / "empty.fa"
    empty.write_bytes(b">only a header\n")
    out = subprocess.run([gs.CLI_PATH, "-k", "19", "-o", small["prefix"], str(empty)],
                         capture_output=True, check=True).stdout
    assert out == b""


def test_config1_full(built, tmp_path_factory):
    """Config 1 at full size: 1 Mbp, 10,000 x 100 bp, k=20, MEM."""
    gs = _gs()
    from gpuseed_gb300 import workloads as W
    d = tmp_path_factory.mktemp("cfg1")
    codes, nmask = W.make_reference(W.ref_spec(1))
    prefix = build_index(d, codes, sa_intv=7)
    seqs, offs, lens = W.make_reads(codes, nmask, W.read_spec(1))
    gidx = gs.Index(prefix)
    ctx = gs.Context(gidx)
    oidx = pyoracle.Index(prefix)
    ob = oidx.seed(seqs, offs, lens, k=20, smem=False)
    for kernel in (0, 1, 2):
        gres = ctx.seed(seqs, offs, lens, k=20, smem=False, kernel=kernel)
        assert_same(gres, ob, lens.size, f"cfg1 kernel={kernel}")
    assert ob.seeds.shape[0] > 10_000


def test_work_counters_match_oracle(small):
    """The plain kernel's containment-stopped walk does exactly the oracle's
    canonical work (13-mer lookups, occurrence blocks, LF steps, SA samples)
    on an index without text structures; with them, locate reads the full
    suffix array once per position and takes no LF steps."""
    gs = _gs()
    reads = sample_reads(small["codes"], 300, seed=21, lengths=(50, 100, 150, 250))
    seqs, offs, lens = pack(reads)
    bare = gs.Index(small["prefix"])
    bare.set_text(0)
    ctx = gs.Context(bare)
    for smem in (False, True):
        ctx.seed(seqs, offs, lens, k=19, smem=smem, kernel=1, count_work=True)
        w = ctx.last_work()
        ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem, pruned=True)
        assert w["n_kmer"] == ob.work["n_kmer"]
        assert w["n_occ_blocks"] == ob.work["n_occ_blocks"]
        assert w["n_lf"] == ob.work["n_lf"]
        assert w["n_sa"] == ob.work["n_sa"]
        small["ctx"].seed(seqs, offs, lens, k=19, smem=smem, kernel=1, count_work=True)
        wt = small["ctx"].last_work()
        assert wt["n_lf"] == 0 and wt["n_sa"] == ob.work["n_sa"]


@pytest.mark.parametrize("kx", [14, 16])
def test_longer_start_table(small, kx):
    """A 14- or 16-mer start table (used when k > its length) gives the same
    seeds, including reads whose start window holds an N after base 13."""
    codes = small["codes"]
    text = "".join("ACGT"[c] for c in codes)
    reads = sample_reads(codes, 300, seed=60 + kx, lengths=(20, 40, 100, 150), err=0.03, n_rate=0.5)
    reads += [(text[3000 + i:3000 + i + 14] + "N" + text[3015 + i:3080 + i]).encode() for i in range(6)]
    seqs, offs, lens = pack(reads)
    small["gidx"].set_kmer_len(kx)
    try:
        assert small["gidx"].info().kmer_len == kx
        for kernel in (0, 1, 2):
            for k in (13, kx, kx + 1, 25):
                for n_mode in (0, 1):
                    for smem in (False, True):
                        gres = small["ctx"].seed(seqs, offs, lens, k=k, smem=smem, n_mode=n_mode,
                                                 kernel=kernel)
                        ob = small["oidx"].seed(seqs, offs, lens, k=k, smem=smem, n_mode=n_mode)
                        assert_same(gres, ob, len(reads), f"kx={kx} kernel={kernel} k={k} n={n_mode}")
        # k > kx: the batched start pairs each window's two candidates; with
        # a walker buffer of a few entries, or none, they are left to the
        # leftover pass, which walks them without J
        for slots in (1, -1):
            for n_mode in (0, 1):
                for smem in (False, True):
                    gres = small["ctx"].seed(seqs, offs, lens, k=kx + 3, smem=smem, n_mode=n_mode,
                                             kernel=0, walker_slots=slots)
                    ob = small["oidx"].seed(seqs, offs, lens, k=kx + 3, smem=smem, n_mode=n_mode)
                    assert_same(gres, ob, len(reads), f"kx={kx} slots={slots} n={n_mode} smem={smem}")
    finally:
        small["gidx"].set_kmer_len(13)


@pytest.mark.parametrize("lanes,steps", [(-1, 0), (1, 1), (8, 4), (32, 1), (32, 30)])
def test_handoff_settings(small, lanes, steps):
    """The lockstep search gives the same seeds whether candidates finish in
    lockstep or are handed to the tail pass, at any threshold."""
    reads = sample_reads(small["codes"], 400, seed=70 + lanes, lengths=(30, 100, 150, 300, 700),
                         err=0.02, n_rate=0.3)
    seqs, offs, lens = pack(reads)
    for smem in (False, True):
        for n_mode in (0, 1):
            gres = small["ctx"].seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode, kernel=2,
                                     handoff_lanes=lanes, handoff_steps=steps)
            ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode)
            assert_same(gres, ob, len(reads), f"handoff {lanes}/{steps} smem={smem} n={n_mode}")


@pytest.mark.parametrize("slots", [-1, 1, 0, 496])
def test_walker_buffer(small, slots):
    """The batched search gives the same seeds whether its survivors are walked
    by the walk pass, by the leftover pass (no buffer), or split between them
    (a buffer that overflows)."""
    reads = sample_reads(small["codes"], 400, seed=80 + slots, lengths=(30, 100, 150, 300, 700),
                         err=0.02, n_rate=0.3)
    seqs, offs, lens = pack(reads)
    for smem in (False, True):
        for n_mode in (0, 1):
            ctx = small["ctx"]
            gres = ctx.seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode, kernel=0,
                            walker_slots=slots)
            n_w, cap = ctx.last_walkers()
            assert (cap == 0) == (slots < 0)
            if slots == 1:
                assert n_w > cap, "the 1-slot buffer should overflow"
            ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode)
            assert_same(gres, ob, len(reads), f"walkers {slots} smem={smem} n={n_mode}")


def test_batched_executes_canonical_steps(small):
    """The batched walk stops every candidate at the canonical step: its
    executed occurrence blocks stay within a small factor of the canonical
    count, and no walk runs past a containment (ACGT-only reads)."""
    reads = sample_reads(small["codes"], 300, seed=33, lengths=(100, 150, 250), err=0.01)
    seqs, offs, lens = pack(reads)
    ctx = small["ctx"]
    ctx.seed(seqs, offs, lens, k=19, smem=True, kernel=1, count_work=True)
    canon = ctx.last_work()
    ctx.seed(seqs, offs, lens, k=19, smem=True, kernel=0, count_work=True)
    batched = ctx.last_work()
    assert batched["n_kmer"] >= canon["n_kmer"]
    assert batched["n_occ_blocks"] <= 2 * canon["n_occ_blocks"] + 64


@pytest.mark.parametrize("kernel", [0, 1])
def test_max_occ_cap(small, kernel):
    """max_occ drops exactly the output seeds whose interval is larger than
    the cap and leaves the others (and their positions) as they were."""
    codes = small["codes"]
    text = "".join("ACGT"[c] for c in codes)
    reads = sample_reads(codes, 300, seed=44, lengths=(50, 100, 150), err=0.02)
    reads += [text[500:530].encode() * 3, b"ACGT" * 20]
    seqs, offs, lens = pack(reads)
    for smem in (False, True):
        ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=smem)
        for cap in (1, 2, 5):
            gres = small["ctx"].seed(seqs, offs, lens, k=19, smem=smem, kernel=kernel, max_occ=cap)
            dropped = 0
            for r in range(len(reads)):
                want = [rec for rec in ob.read_records(r) if rec[3] - rec[2] + 1 <= cap]
                dropped += len(ob.read_records(r)) - len(want)
                assert gres.read_records(r) == want, (smem, cap, r)
            if cap == 1:
                assert dropped > 0


def test_graph_replay(small):
    """Captured passes: the first call sizes and captures, later calls replay;
    new content in the same buffers (other outputs, possibly larger) still
    gives the oracle's seeds."""
    import torch
    dev = torch.device("cuda", 0)
    batches = [sample_reads(small["codes"], 300, seed=90 + i, lengths=(100, 150), err=0.02)
               for i in range(3)]
    # same shape for every batch: 300 reads, equal lengths per slot
    packed = [pack(b) for b in batches]
    lens0 = packed[0][2]
    for seqs, offs, lens in packed[1:]:
        lens[:] = lens0[:lens.size]
    d_seqs = torch.zeros(int(lens0.sum()) + 16, dtype=torch.uint8, device=dev)
    d_offs = torch.from_numpy(packed[0][1].view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens0.view(np.int32)).to(dev)
    ctx = small["ctx"]
    for rep, (seqs, offs, lens) in enumerate(packed + packed[:1]):
        # rebuild each batch's reads at batch 0's lengths and offsets
        reads = [seqs[int(o):int(o) + int(n)] for o, n in zip(offs, lens)]
        buf = b"".join(r[:int(n)].ljust(int(n), b"A") for r, n in zip(reads, lens0))
        d_seqs[:len(buf)].copy_(torch.frombuffer(bytearray(buf), dtype=torch.uint8))
        torch.cuda.synchronize()
        for _ in range(2):
            gres = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(),
                                   lens0.size, fetch=True, k=19, smem=True, graph=True)
            ob = small["oidx"].seed(buf, packed[0][1], lens0, k=19, smem=True)
            assert_same(gres, ob, lens0.size, f"graph rep {rep}")


def test_graph_replay_longer_reads(small):
    """A pass captured on short reads, replayed on the same buffers holding
    longer reads (more candidate slots than it was sized for): the replay
    notices, sizes a new pass, and the seeds are the oracle's."""
    import torch
    dev = torch.device("cuda", 0)
    short = sample_reads(small["codes"], 200, seed=97, lengths=(40,), err=0.01)
    longr = sample_reads(small["codes"], 200, seed=98, lengths=(240,), err=0.01)
    ctx = small["ctx"]
    d_seqs = torch.zeros(200 * 240 + 16, dtype=torch.uint8, device=dev)
    d_offs = torch.zeros(200, dtype=torch.int64, device=dev)
    d_lens = torch.zeros(200, dtype=torch.int32, device=dev)
    for reads in (short, short, longr, longr, short):
        seqs, offs, lens = pack(reads)
        d_seqs[:len(seqs)].copy_(torch.frombuffer(bytearray(seqs), dtype=torch.uint8))
        d_offs.copy_(torch.from_numpy(offs.view(np.int64)))
        d_lens.copy_(torch.from_numpy(lens.view(np.int32)))
        torch.cuda.synchronize()
        gres = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), 200,
                               fetch=True, k=19, smem=True, graph=True)
        ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=True)
        assert_same(gres, ob, 200, f"replay len {int(lens[0])}")


def test_cli_record_input(small, tmp_path):
    """seed_gen -F reads multi-line FASTA, FASTQ, CR LF and gzip input; the
    records equal the oracle's on the joined sequences."""
    import gzip
    gs = _gs()
    reads = sample_reads(small["codes"], 60, seed=123, lengths=(40, 100, 170))
    seqs, offs, lens = pack(reads)
    ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=True)
    want = tmp_path / "o.txt"
    ob.write_text(str(want), 1, True)
    fa = b"".join(b">r%d desc\r\n" % i + b"\r\n".join(r[j:j + 33] for j in range(0, len(r), 33)) + b"\r\n"
                  for i, r in enumerate(reads))
    fq = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r)) for i, r in enumerate(reads))
    files = {"multi.fa": fa, "reads.fq": fq}
    for name, data in files.items():
        (tmp_path / name).write_bytes(data)
    (tmp_path / "multi.fa.gz").write_bytes(gzip.compress(fa))
    for name in ("multi.fa", "reads.fq", "multi.fa.gz"):
        out = subprocess.run([gs.CLI_PATH, "-F", "-k", "19", "-s", "-o", small["prefix"],
                              str(tmp_path / name)], capture_output=True, check=True).stdout
        assert out == want.read_bytes(), name


def _text_digest(ctx, smem):
    """SHA-1 of the context's -o records, streamed through a pipe."""
    import hashlib
    import threading
    rfd, wfd = os.pipe()
    h = hashlib.sha1()

    def drain():
        with os.fdopen(rfd, "rb") as f:
            for block in iter(lambda: f.read(1 << 20), b""):
                h.update(block)

    t = threading.Thread(target=drain)
    t.start()
    try:
        ctx.write_text(wfd, 1, smem)
    finally:
        os.close(wfd)
        t.join()
    return h.hexdigest()


def _many_reads(codes, n, seed):
    """n reads of 20-90 bases copied from the text with 1 % substitutions and
    a few N, packed in order: (bytes, offsets, lengths)."""
    rng = np.random.default_rng(seed)
    lens = rng.choice(np.array([20, 33, 47, 64, 90], np.uint32), n)
    starts = rng.integers(0, codes.size - 100, n)
    offs = np.zeros(n, np.uint64)
    offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
    total = int(lens.sum())
    idx = np.repeat(starts - offs.astype(np.int64), lens) + np.arange(total)
    buf = np.frombuffer(b"ACGT", np.uint8)[codes[idx]].copy()
    sub = rng.random(total) < 0.01
    buf[sub] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(sub.sum()))]
    buf[rng.random(total) < 0.001] = ord("N")
    return buf, offs, lens


@pytest.mark.parametrize("smem", [False, True], ids=["mem", "smem"])
def test_seed_in_chunks_matches_one_pass(small, smem):
    """gs_seed runs a batch of 2^22 or more reads held in order as chunks,
    copying each chunk up and its results down while the next one runs. Its
    host result equals one device pass over the same reads, array for array.
    A batch whose reads are not in order runs as one pass."""
    import torch
    ctx = small["ctx"]
    buf, offs, lens = _many_reads(small["codes"], (1 << 22) + 123_457, seed=101 + smem)
    got = ctx.seed(buf, offs, lens, k=19, smem=smem)
    got_text = _text_digest(ctx, smem)      # formatted by the host: no device result
    dev = torch.device("cuda", 0)
    d_seqs = torch.from_numpy(buf).to(dev)
    d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
    want = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), lens.size,
                           fetch=True, k=19, smem=smem)
    for name in ("read_seed_off", "read_pos_off", "seeds", "pos"):
        assert np.array_equal(getattr(got, name), getattr(want, name)), name
    assert got_text == _text_digest(ctx, smem)   # the device pass's, formatted on the GPU
    # the same reads with their order in the buffer reversed: not chunked
    roffs = (buf.size - (offs + lens)).astype(np.uint64)
    rbuf = np.empty_like(buf)
    rbuf[np.repeat(roffs.astype(np.int64) - offs.astype(np.int64), lens) + np.arange(buf.size)] = buf
    rev = ctx.seed(rbuf, roffs, lens, k=19, smem=smem)
    for name in ("read_seed_off", "read_pos_off", "seeds", "pos"):
        assert np.array_equal(getattr(rev, name), getattr(want, name)), name


def test_graph_recaptures_after_index_change(small):
    """A pass captured into a CUDA graph holds the index's device pointers;
    freeing or rebuilding the text structures or the start table bumps the
    index's generation, so the next call captures again instead of replaying
    with freed buffers.  Every call gives the oracle's seeds."""
    import torch
    gs = _gs()
    gidx = gs.Index(small["prefix"])
    gidx.set_text(4)
    ctx = gs.Context(gidx)
    reads = sample_reads(small["codes"], 300, seed=131, lengths=(60, 120, 250), err=0.01)
    seqs, offs, lens = pack(reads)
    dev = torch.device("cuda", 0)
    d_seqs = torch.from_numpy(np.frombuffer(seqs, np.uint8).copy()).to(dev)
    d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
    ob = small["oidx"].seed(seqs, offs, lens, k=19, smem=True)
    changes = [lambda: None, lambda: gidx.set_text(0), lambda: gidx.set_text(4),
               lambda: gidx.set_text(-1), lambda: gidx.set_kmer_len(14), lambda: gidx.set_text(2)]
    for step, change in enumerate(changes):
        change()
        for rep in range(2):     # capture (or replay), then replay
            gres = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(),
                                   lens.size, fetch=True, k=19, smem=True, graph=True)
            assert_same(gres, ob, lens.size, f"change {step} rep {rep}")


@pytest.mark.parametrize("n", [50_001, 49_999, 65_537], ids=["odd", "odd2", "pow2+1"])
def test_text_structures_odd_lengths(built, tmp_path, n):
    """References whose length is odd and not a multiple of 16: the packed
    text ends in a partial word and the text end has no inverse-SA sample
    (its row is row 0).  Reads at both ends of the text walk there in text
    mode (entered after one step); every kernel and mode gives the oracle's
    seeds, and the structures equal the oracle's suffix array and text."""
    gs = _gs()
    codes = random_reference(n, 500 + n % 97)
    prefix = build_index(tmp_path, codes, sa_intv=7)
    gidx = gs.Index(prefix)
    gidx.set_text(1)
    oidx = pyoracle.Index(prefix)
    sa = pyoracle.suffix_array(codes)
    want = sa.copy()
    want[0] = 0xffffffff
    assert np.array_equal(gidx.text_table(0), want)
    isa = np.empty(n + 1, np.int64)
    isa[sa.astype(np.int64)] = np.arange(n + 1)
    assert np.array_equal(gidx.text_table(2), isa[::2].astype(np.uint32))
    text = "".join("ACGT"[c] for c in codes)
    reads = []
    for L in (19, 20, 33, 64, 130, 250):
        reads += [text[:L].encode(), text[n - L:].encode(), text[n - L - 7:n - 7].encode()]
        j = L // 2
        s = text[n - L:]
        reads.append((s[:j] + "ACGT"[("ACGT".index(s[j]) + 2) % 4] + s[j + 1:]).encode())
    reads += sample_reads(codes, 150, seed=n, lengths=(20, 64, 150, 250), err=0.01)
    seqs, offs, lens = pack(reads)
    ctx = gs.Context(gidx)
    for kernel in (0, 1, 2):
        for smem in (False, True):
            for n_mode in (0, 1):
                gres = ctx.seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode, kernel=kernel)
                ob = oidx.seed(seqs, offs, lens, k=19, smem=smem, n_mode=n_mode)
                assert_same(gres, ob, len(reads), f"n={n} kernel={kernel} smem={smem} N={n_mode}")
