"""GPU index construction against the oracle's SA-IS construction: the
.bwt/.sa files must be byte-identical."""
import os

import numpy as np
import pytest

import pyoracle
from helpers import random_reference

pytestmark = pytest.mark.gpu


def _texts():
    yield "tiny1", np.array([2], np.uint8), 7
    yield "tiny5", np.array([0, 1, 0, 1, 0], np.uint8), 1
    yield "homo", np.zeros(1000, np.uint8), 7
    yield "n64", random_reference(640, 3), 7
    yield "n65", random_reference(65, 4), 3
    yield "rand", random_reference(50_000, 5), 7
    yield "rep", np.tile(random_reference(300, 6), 40), 5
    yield "big", random_reference(3_000_000, 8), 7


@pytest.mark.parametrize("name,codes,intv", list(_texts()), ids=[t[0] for t in _texts()])
def test_gpu_build_matches_oracle(built, tmp_path, name, codes, intv):
    import gpuseed_gb300 as gs
    gp = os.path.join(str(tmp_path), "g")
    op = os.path.join(str(tmp_path), "o")
    gs.build_index(codes, intv, prefix=gp, load=False)
    pyoracle.build_index(codes, intv, op)
    for ext in (".bwt", ".sa"):
        g = open(gp + ext, "rb").read()
        o = open(op + ext, "rb").read()
        assert len(g) == len(o) and g == o, f"{name}{ext} differs"


def test_gpu_build_loaded_index_seeds(built, tmp_path):
    """The index returned by the builder seeds like the one loaded from its files."""
    import gpuseed_gb300 as gs
    from helpers import pack, sample_reads
    codes = random_reference(80_000, 12)
    prefix = os.path.join(str(tmp_path), "g")
    idx_built = gs.build_index(codes, 7, prefix=prefix)
    idx_file = gs.Index(prefix)
    reads = sample_reads(codes, 200, seed=3, lengths=(50, 100, 150))
    seqs, offs, lens = pack(reads)
    a = gs.Context(idx_built).seed(seqs, offs, lens, k=19, smem=True)
    b = gs.Context(idx_file).seed(seqs, offs, lens, k=19, smem=True)
    for r in range(len(reads)):
        assert a.read_records(r) == b.read_records(r)
