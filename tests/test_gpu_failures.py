"""Failure paths that end in an error code instead of an exit (the reference
prints and exits: seed_gen.cu:2692-2707, :3555-3558), driven without any GPU
fault: the inputs are valid memory, and every device loop involved is
bounded.

* GS_EWALK: an index whose BWT has two bases of one block swapped (its block
  counts still agree, so it loads) has an LF cycle that passes no sampled
  row; locating a row of it by LF steps stops at the walk's step limit
  (seq_len + 2), sets the error flag, and every entry point reports
  GS_EWALK.  Building the text structures of that index fails its
  consistency checks (GS_EFORMAT).  The GPU stays usable afterwards.
* GS_ETIMEOUT: gs_server_wait with a zero limit on a request that is still
  running; the request then completes normally.
"""
import numpy as np
import pytest

from helpers import build_index, lf_cycle_index, pack, random_reference, sample_reads

pytestmark = pytest.mark.gpu

GS_EFORMAT, GS_EWALK, GS_ETIMEOUT = -3, -6, -8


def _code(fn):
    import gpuseed_gb300 as gs
    with pytest.raises(gs.GsError) as e:
        fn()
    return e.value.code


def test_walk_limit_reports_gs_ewalk(built, tmp_path):
    import torch

    import gpuseed_gb300 as gs

    arrays, read = lf_cycle_index(tmp_path)
    idx = gs.Index(arrays=arrays)
    ctx = gs.Context(idx)
    seqs, offs, lens = pack([read, b"ACGTTGCA" * 5, read])
    for smem in (True, False):
        assert _code(lambda: ctx.seed(seqs, offs, lens, k=19, smem=smem)) == GS_EWALK
    dev = torch.device("cuda", 0)
    d_seqs = torch.from_numpy(np.frombuffer(seqs, np.uint8).copy()).to(dev)
    d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
    args = (d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), lens.size)
    for graph in (False, True):
        for _ in range(2):      # with graph: the capture, then a replay
            assert _code(lambda: ctx.seed_device(*args, fetch=True, k=19, smem=True,
                                                 graph=graph)) == GS_EWALK
    d_seeds = torch.zeros(64 * 8, dtype=torch.int32, device=dev)
    d_pos = torch.zeros(4096, dtype=torch.int32, device=dev)
    d_off = torch.zeros(2 * (lens.size + 1), dtype=torch.int64, device=dev)
    assert _code(lambda: gs.seed_noalloc(idx, *args, d_seeds.data_ptr(), 64, d_pos.data_ptr(),
                                         4096, d_off.data_ptr(),
                                         d_off.data_ptr() + 8 * (lens.size + 1),
                                         k=19, smem=True)) == GS_EWALK
    # the text structures' build checks the chains against the samples
    assert _code(lambda: idx.set_text(4)) == GS_EFORMAT
    ctx.close()
    idx.close()
    # the device still works: a consistent index seeds normally
    codes = random_reference(5_000, 78)
    good = gs.Index(build_index(tmp_path, codes, sa_intv=16, name="good"))
    res = gs.Context(good).seed(*pack(sample_reads(codes, 50, seed=3, lengths=(60,))), k=19)
    assert res.n_reads == 50 and res.seeds.shape[0] > 0


def test_server_wait_times_out(built, tmp_path):
    import gpuseed_gb300 as gs

    codes = random_reference(400_000, 79, dups=40)
    idx = gs.Index(build_index(tmp_path, codes, sa_intv=7))
    reads = sample_reads(codes, 20_000, seed=4, lengths=(150, 250), err=0.01)
    seqs, offs, lens = pack(reads)
    want = gs.Context(idx).seed(seqs, offs, lens, k=19, smem=True)
    srv = gs.Server(idx, k=19, smem=True)
    try:
        rid = srv.submit(seqs, offs, lens)
        assert srv.wait(rid, 0) == GS_ETIMEOUT
        assert srv.wait(rid, -1) == 0
        got, _ = srv.result(rid)
        assert np.array_equal(got.seeds, want.seeds) and np.array_equal(got.pos, want.pos)
        assert np.array_equal(got.read_seed_off, want.read_seed_off)
    finally:
        srv.stop()
