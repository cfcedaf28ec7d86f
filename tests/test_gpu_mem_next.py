"""MEM mode with GS_MEM_NEXT_GPUSEED: the reference's cross-read exclusion
interval (seeds_to_threads_mem, seed_gen.cu:635-650; quirk Q10), against the
oracle's restatement of it, which tests/test_ref_pin.py pins to the
reference's own kernels.

Adjacent identical reads trigger it: a read from the forward strand has no
reverse record, so the scan from its last forward record meets its twin's
first forward record, with the same begin and the same interval; the read
then emits the row after its interval instead of its own.  Reads between
twins that have no seeds are skipped by the scan, as in the reference's
compacted arrays.
"""
import subprocess

import numpy as np
import pytest

import pyoracle
from helpers import build_index, pack, random_reference, sample_reads

pytestmark = pytest.mark.gpu


def _mism(gres, ob):
    return pyoracle.mismatched_reads(ob, gres.seeds, gres.pos, gres.read_seed_off,
                                     gres.read_pos_off, cols=(0, 1, 2, 3, 6))


def _records(res):
    return [res.read_records(r) for r in range(res.n_reads)]


@pytest.fixture(scope="module")
def twins(built, tmp_path_factory):
    import gpuseed_gb300 as gs
    d = tmp_path_factory.mktemp("twins")
    codes = random_reference(80_000, 311, dups=10)
    prefix = build_index(d, codes, sa_intv=7)
    reads = []
    for r in sample_reads(codes, 60, seed=12, lengths=(80, 120), err=0.0):
        reads += [r, r]
    # twins with a read between them that has no seeds (shorter than k),
    # and twins one substitution apart
    for r in sample_reads(codes, 20, seed=13, lengths=(100,), err=0.0):
        reads += [r, b"ACGTACGT", r]
    for r in sample_reads(codes, 20, seed=14, lengths=(100,), err=0.0):
        t = bytearray(r)
        t[50] = ord("A") if t[50] != ord("A") else ord("C")
        reads += [r, bytes(t)]
    reads += sample_reads(codes, 200, seed=15, lengths=(60, 100, 150), err=0.02)
    gidx = gs.Index(prefix)
    return dict(codes=codes, prefix=prefix, gidx=gidx, oidx=pyoracle.Index(prefix),
                reads=reads, dir=d)


@pytest.mark.parametrize("text", [False, True], ids=["lf_walk", "full_sa"])
def test_mem_next_matches_oracle(twins, text):
    import torch

    import gpuseed_gb300 as gs
    gidx = twins["gidx"]
    gidx.set_text(4 if text else 0)
    ctx = gs.Context(gidx)
    seqs, offs, lens = pack(twins["reads"])
    ob = twins["oidx"].seed(seqs, offs, lens, k=19, smem=False, mem_next=1)
    per_read = twins["oidx"].seed(seqs, offs, lens, k=19, smem=False)
    differ = pyoracle.mismatched_reads(ob, per_read.seeds, per_read.pos, per_read.read_seed_off,
                                       per_read.read_pos_off)
    assert differ.size >= 60
    for kernel in (gs.KERNEL_BATCHED, gs.KERNEL_PLAIN, gs.KERNEL_LOCKSTEP):
        bad = _mism(ctx.seed(seqs, offs, lens, k=19, smem=False, kernel=kernel, mem_next=1), ob)
        assert bad.size == 0, (kernel, bad[:10])
    # device reads: the graph-captured pass (capture, then replay) and the
    # allocation-free entry point
    dev = torch.device("cuda", 0)
    d_seqs = torch.from_numpy(np.frombuffer(seqs, np.uint8).copy()).to(dev)
    d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
    args = (d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), lens.size)
    for _ in range(2):
        bad = _mism(ctx.seed_device(*args, fetch=True, k=19, smem=False, graph=True, mem_next=1),
                    ob)
        assert bad.size == 0, ("graph", bad[:10])
    ns, npos = ob.seeds.shape[0], ob.pos.size
    d_seeds = torch.zeros(ns * 8 + 8, dtype=torch.int32, device=dev)
    d_pos = torch.zeros(npos + 1, dtype=torch.int32, device=dev)
    d_off = torch.zeros(2 * (lens.size + 1), dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    got = gs.seed_noalloc(gidx, *args, d_seeds.data_ptr(), ns + 1, d_pos.data_ptr(), npos + 1,
                          d_off.data_ptr(), d_off.data_ptr() + 8 * (lens.size + 1), k=19,
                          smem=False, mem_next=1)
    torch.cuda.synchronize()
    assert got == (ns, npos)
    s = d_seeds.cpu().numpy().view(np.uint32).reshape(-1, 8)[:ns]
    assert np.array_equal(s[:, [0, 1, 2, 3, 6]], ob.seeds)
    assert np.array_equal(d_pos.cpu().numpy().view(np.uint32)[:npos], ob.pos)
    # SMEM mode has no exclusion interval: the switch changes nothing there
    a = ctx.seed(seqs, offs, lens, k=19, smem=True, mem_next=1)
    b = ctx.seed(seqs, offs, lens, k=19, smem=True)
    assert _records(a) == _records(b)
    ctx.close()


def test_mem_next_cli_and_server(twins, tmp_path):
    import gpuseed_gb300 as gs
    reads = twins["reads"]
    fa = tmp_path / "twins.fa"
    with open(fa, "wb") as f:
        for i, r in enumerate(reads):
            f.write(b">r%d\n%s\n" % (i, r))
    seqs, offs, lens = pack(reads)
    ob = twins["oidx"].seed(seqs, offs, lens, k=19, smem=False, mem_next=1)
    opath = tmp_path / "o.txt"
    ob.write_text(str(opath), 1, False)
    out = subprocess.run([gs.CLI_PATH, "-k", "19", "-Q", "-o", twins["prefix"], str(fa)],
                         capture_output=True, check=True).stdout
    assert out == opath.read_bytes()
    # a server's request must not depend on the requests merged with it
    with pytest.raises(gs.GsError) as e:
        gs.Server(twins["gidx"], k=19, smem=False, mem_next=1)
    assert e.value.code == -1


@pytest.mark.parametrize("cfg", [1, 2])
def test_mem_next_on_configs(built, tmp_path, cfg):
    """Configs 1 and 2 in MEM mode: both modes match the oracle; the reads on
    which they differ are counted (printed)."""
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    codes, nmask = W.make_reference(W.ref_spec(cfg))
    prefix = str(tmp_path / f"cfg{cfg}")
    idx = gs.build_index(codes, 7, prefix=prefix)
    seqs, offs, lens = W.make_reads(codes, nmask, W.read_spec(cfg))
    k = W.CONFIG_K[cfg]
    oidx = pyoracle.Index(prefix)
    table = idx.kmer_table()
    ctx = gs.Context(idx)
    res = {}
    for mode in (0, 1):
        ob = oidx.seed(seqs, offs, lens, k=k, smem=False, mem_next=mode, pruned=True, table=table)
        res[mode] = ctx.seed(seqs, offs, lens, k=k, smem=False, mem_next=mode)
        bad = _mism(res[mode], ob)
        assert bad.size == 0, (cfg, mode, bad[:10])
        del ob
    ob0 = oidx.seed(seqs, offs, lens, k=k, smem=False, pruned=True, table=table)
    differ = _mism(res[1], ob0)
    print(f"config {cfg} MEM k={k}: {lens.size:,} reads, {differ.size} differ between the "
          f"per-read and the cross-read exclusion")
