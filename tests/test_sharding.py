"""Multi-process path on CPU: two gloo ranks shard the reads, seed their shard
(with the CPU oracle standing in for each rank's GPU), and the records gathered
in rank order equal the single-process records; timing reductions take the
max time and the total reads."""
import os
import socket

import numpy as np
import pytest

from gpuseed_gb300.sharding import first_read_number, reduce_timing, shard_range


def test_shard_ranges_partition():
    for n in (0, 1, 7, 10, 1001):
        for w in (1, 2, 3, 8):
            ranges = [shard_range(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, prefix, reads_path, out_dir):
    import torch.distributed as dist
    import pyoracle
    from helpers import pack
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    reads = [ln.strip().encode() for ln in open(reads_path) if not ln.startswith(">")]
    lo, hi = shard_range(len(reads), rank, world)
    seqs, offs, lens = pack(reads[lo:hi])
    idx = pyoracle.Index(prefix)
    b = idx.seed(seqs, offs, lens, k=19, smem=True, threads=1)
    path = os.path.join(out_dir, f"rank{rank}.txt")
    b.write_text(path, first_read_number(len(reads), rank, world), True)
    t, n = reduce_timing(dist, 1.0 + rank, hi - lo)
    assert t == 1.0 + (world - 1) and n == len(reads)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_single_process(built, tmp_path):
    import torch.multiprocessing as mp
    import pyoracle
    from helpers import build_index, pack

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    text = open(os.path.join(gold, "ref20k.txt")).read().strip()
    codes = np.array(["ACGT".index(ch) for ch in text], np.uint8)
    prefix = build_index(tmp_path, codes, sa_intv=7)
    reads_path = os.path.join(gold, "reads60.fa")
    mp.spawn(_rank_main, args=(2, _free_port(), prefix, reads_path, str(tmp_path)), nprocs=2,
             join=True)
    merged = open(tmp_path / "rank0.txt").read() + open(tmp_path / "rank1.txt").read()
    reads = [ln.strip().encode() for ln in open(reads_path) if not ln.startswith(">")]
    seqs, offs, lens = pack(reads)
    b = pyoracle.Index(prefix).seed(seqs, offs, lens, k=19, smem=True, threads=1)
    b.write_text(str(tmp_path / "single.txt"), 1, True)
    assert merged == open(tmp_path / "single.txt").read()
