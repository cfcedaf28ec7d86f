"""The allocation-free entry point gs_seed_noalloc, against gs_seed_device.

gs_seed_noalloc exists for callers that may not allocate device memory while
they run -- a process that reserved its HBM at start-up, or one that cannot
let cudaMalloc/cudaFree synchronise the device under other streams' work.
It runs the same batched pass with all scratch in one static device array.
Here it is called through the C-ABI twice in a row, on two different batches
(so the second call starts from the first call's leftovers in the shared
array), and every seed, position and per-read offset must equal what the
allocating entry point returns for the same batch (integer results: exact).

This file is named to be collected last.
"""
import numpy as np
import pytest

from helpers import build_index, pack, random_reference, sample_reads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("text", [False, True], ids=["lf_walk", "full_sa"])
def test_noalloc_matches_allocating_entry_point(built, tmp_path, text):
    """text: the index holds the full suffix array, so both entry points
    locate by one read of it instead of walking to a sampled row."""
    import torch

    import gpuseed_gb300 as gs

    codes = random_reference(120_000, 31, dups=30)
    prefix = build_index(tmp_path, codes, sa_intv=7)
    idx = gs.Index(prefix)
    if text:
        idx.set_text(4)
    ctx = gs.Context(idx)
    dev = torch.device("cuda", 0)
    batches = [sample_reads(codes, 700, seed=41, lengths=(50, 100, 150, 250), err=0.02),
               sample_reads(codes, 400, seed=42, lengths=(19, 40, 90), err=0.01)]
    for call, (reads, smem) in enumerate(zip(batches, (True, False))):
        seqs, offs, lens = pack(reads)
        d_seqs = torch.from_numpy(np.frombuffer(seqs, np.uint8).copy()).to(dev)
        d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
        d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
        n = lens.size
        want = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n,
                               fetch=True, k=19, smem=smem)
        seed_cap, pos_cap = want.seeds.shape[0] + 8, want.pos.size + 8
        d_seeds = torch.zeros(seed_cap * 8, dtype=torch.int32, device=dev)
        d_pos = torch.zeros(pos_cap, dtype=torch.int32, device=dev)
        d_rso = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        d_rpo = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        ns, npos = gs.seed_noalloc(idx, d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n,
                                   d_seeds.data_ptr(), seed_cap, d_pos.data_ptr(), pos_cap,
                                   d_rso.data_ptr(), d_rpo.data_ptr(), k=19, smem=smem)
        torch.cuda.synchronize()
        assert (ns, npos) == (want.seeds.shape[0], want.pos.size), f"call {call}"
        got_seeds = d_seeds.cpu().numpy().view(np.uint32).reshape(-1, 8)[:ns]
        assert np.array_equal(got_seeds, want.seeds), f"call {call}: seeds differ"
        assert np.array_equal(d_pos.cpu().numpy().view(np.uint32)[:npos], want.pos), f"call {call}"
        assert np.array_equal(d_rso.cpu().numpy().view(np.uint64), want.read_seed_off)
        assert np.array_equal(d_rpo.cpu().numpy().view(np.uint64), want.read_pos_off)
        assert ns > 100 and npos >= ns


def test_noalloc_rejects_oversized_batch(built, tmp_path):
    import gpuseed_gb300 as gs

    codes = random_reference(5_000, 32)
    idx = gs.Index(build_index(tmp_path, codes, sa_intv=7))
    with pytest.raises(gs.GsError) as e:
        gs.seed_noalloc(idx, 1, 1, 1, 65537, 1, 1, 1, 1, 1, 1, k=19)
    assert e.value.code == -1 and "at most 65536" in str(e.value)


def _device_reads(reads, dev):
    import torch
    seqs, offs, lens = pack(reads)
    return (torch.from_numpy(np.frombuffer(seqs, np.uint8).copy()).to(dev),
            torch.from_numpy(offs.view(np.int64)).to(dev),
            torch.from_numpy(lens.view(np.int32)).to(dev), lens.size)


def test_noalloc_overflow_side_stream_and_slot_limit(built, tmp_path):
    """Through the C-ABI: output buffers one seed or one position too small
    give GS_EOVERFLOW with the counts still reported; a call on a side
    stream gives the allocating entry point's result; a batch beyond the
    candidate-slot limit is refused with GS_EINVAL."""
    import ctypes as C

    import torch

    import gpuseed_gb300 as gs

    codes = random_reference(80_000, 33, dups=20)
    idx = gs.Index(build_index(tmp_path, codes, sa_intv=7))
    ctx = gs.Context(idx)
    dev = torch.device("cuda", 0)
    d_seqs, d_offs, d_lens, n = _device_reads(
        sample_reads(codes, 500, seed=43, lengths=(60, 120, 200), err=0.02), dev)
    want = ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n,
                           fetch=True, k=19, smem=True)
    ns_want, np_want = want.seeds.shape[0], want.pos.size
    L = gs.lib()
    p = gs.Context.params(k=19, smem=True)
    d_rso = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    d_rpo = torch.zeros(n + 1, dtype=torch.int64, device=dev)

    def call(seed_cap, pos_cap, stream=None, reads=None):
        rs, ro, rl, rn = reads or (d_seqs, d_offs, d_lens, n)
        d_seeds = torch.zeros(max(seed_cap, 1) * 8, dtype=torch.int32, device=dev)
        d_pos = torch.zeros(max(pos_cap, 1), dtype=torch.int32, device=dev)
        ns, npos = C.c_uint64(), C.c_uint64()
        torch.cuda.synchronize()
        rc = L.gs_seed_noalloc(idx.h, C.c_void_p(rs.data_ptr()), C.c_void_p(ro.data_ptr()),
                               C.c_void_p(rl.data_ptr()), rn, C.byref(p),
                               C.c_void_p(stream) if stream else None,
                               C.c_void_p(d_seeds.data_ptr()), seed_cap,
                               C.c_void_p(d_pos.data_ptr()), pos_cap,
                               C.c_void_p(d_rso.data_ptr()), C.c_void_p(d_rpo.data_ptr()),
                               C.byref(ns), C.byref(npos))
        torch.cuda.synchronize()
        return rc, int(ns.value), int(npos.value), d_seeds, d_pos

    for caps in ((ns_want - 1, np_want), (ns_want, np_want - 1)):
        rc, ns, npos, _, _ = call(*caps)
        assert rc == -7    # GS_EOVERFLOW
        assert (ns, npos) == (ns_want, np_want)

    side = torch.cuda.Stream(device=dev)
    rc, ns, npos, d_seeds, d_pos = call(ns_want, np_want, stream=side.cuda_stream)
    assert rc == 0 and (ns, npos) == (ns_want, np_want)
    assert np.array_equal(d_seeds.cpu().numpy().view(np.uint32).reshape(-1, 8)[:ns], want.seeds)
    assert np.array_equal(d_pos.cpu().numpy().view(np.uint32)[:npos], want.pos)
    assert np.array_equal(d_rso.cpu().numpy().view(np.uint64), want.read_seed_off)

    # 5,000 reads of 250 bases: 2 x 5,000 x 232 candidate slots > 2^21
    big = _device_reads([b"ACGT" * 62 + b"AC"] * 5_000, dev)
    d_rso = torch.zeros(5_001, dtype=torch.int64, device=dev)
    d_rpo = torch.zeros(5_001, dtype=torch.int64, device=dev)
    rc, _, _, _, _ = call(16, 16, reads=big)
    assert rc == -1 and "candidate slots" in gs.lib().gs_last_error().decode()
