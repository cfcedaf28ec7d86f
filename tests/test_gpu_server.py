"""Serving loop: requests submitted concurrently are merged into passes, and
every request's seeds equal those of the same reads seeded alone (exact)."""
import threading

import numpy as np
import pytest

from helpers import build_index, pack, random_reference, sample_reads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built, tmp_path_factory):
    import gpuseed_gb300 as gs
    codes = random_reference(200_000, 77, dups=40)
    prefix = build_index(tmp_path_factory.mktemp("srv"), codes, sa_intv=7)
    idx = gs.Index(prefix)
    idx.set_text(4)     # a resident server would build them: passes use text mode
    return dict(codes=codes, idx=idx, ctx=gs.Context(idx))


def _requests(codes, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        m = int(np.exp(rng.uniform(0, np.log(400))))   # 1..400 reads, log-uniform
        out.append(sample_reads(codes, m, seed=seed * 1000 + i, lengths=(100, 150, 250), err=0.01))
    return out


@pytest.mark.parametrize("smem", [True, False])
def test_mixed_requests_equal_alone(env, smem):
    import gpuseed_gb300 as gs
    reqs = _requests(env["codes"], 60, seed=5 if smem else 6)
    srv = gs.Server(env["idx"], n_slots=3, k=19, smem=smem)
    ids = [None] * len(reqs)

    def client(lo, hi):
        for i in range(lo, hi):
            ids[i] = srv.submit(*pack(reqs[i]))

    th = [threading.Thread(target=client, args=(j * 15, (j + 1) * 15)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    results = []
    for rid in ids:
        assert srv.wait(rid, 60_000) == 0
        results.append(srv.result(rid))
    st = srv.stats()
    srv.stop()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["passes"] < len(reqs), "no request was merged with another"
    for i, (res, lat) in enumerate(results):
        alone = env["ctx"].seed(*pack(reqs[i]), k=19, smem=smem)
        assert res.n_reads == alone.n_reads
        assert np.array_equal(res.seeds, alone.seeds), f"request {i}"
        assert np.array_equal(res.pos, alone.pos), f"request {i}"
        assert np.array_equal(res.read_seed_off, alone.read_seed_off)
        assert lat > 0


def test_admission_refuses_what_cannot_fit(env):
    import gpuseed_gb300 as gs
    srv = gs.Server(env["idx"], n_slots=2, hbm_budget=8 << 20, k=19, smem=True)
    small = srv.submit(*pack(sample_reads(env["codes"], 5, seed=1, lengths=(100,))))
    big = srv.submit(*pack(sample_reads(env["codes"], 30_000, seed=2, lengths=(250,))))
    assert srv.wait(small, 60_000) == 0
    assert srv.wait(big, 60_000) == -4      # GS_ENOMEM: larger than the whole budget
    srv.stop()


def test_submit_by_reference(env):
    """gs_server_submit_ref: reads back to back in the caller's buffer are
    read in place, others are copied; either way each request's seeds equal
    a direct pass over its reads."""
    import gpuseed_gb300 as gs
    reqs = _requests(env["codes"], 30, seed=8)
    srv = gs.Server(env["idx"], n_slots=2, k=19, smem=True)
    try:
        ids = []
        for i, reads in enumerate(reqs):
            seqs, offs, lens = pack(reads)
            if i % 3 == 2 and lens.size > 1:
                # not back to back: a gap of 7 bytes before every read
                buf = b"".join(b"NNNNNNN" + r for r in reads)
                offs = (np.cumsum(np.concatenate([[0], lens[:-1] + 7])) + 7).astype(np.uint64)
                seqs = buf
            ids.append(srv.submit(seqs, offs, lens, copy=False))
        for reads, rid in zip(reqs, ids):
            assert srv.wait(rid) == 0
            got, _ = srv.result(rid)
            want = env["ctx"].seed(*pack(reads), k=19, smem=True)
            assert np.array_equal(got.seeds, want.seeds) and np.array_equal(got.pos, want.pos)
            assert np.array_equal(got.read_seed_off, want.read_seed_off)
    finally:
        srv.stop()
