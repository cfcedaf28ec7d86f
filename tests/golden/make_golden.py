"""Generates the golden fixtures in this directory.

The expected outputs come from the brute-force matcher (tests/bruteforce.py),
which finds every match by plain substring search -- no FM index, no BWT, no
oracle code -- and orders positions by comparing suffixes.  They pin the
oracle (and through it the GPU path) independently of any index arithmetic.
Positions are the true suffix-array values, i.e. the bwa LF convention
(oracle lf_mode = LF_BWA).

Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bruteforce as bf  # noqa: E402
from helpers import random_reference, sample_reads  # noqa: E402

HEADER = ("/*===================================%s seeds in read no. %d (Read[begin, End] -> "
          "starting position(s) on the reference)===================================*/\n")


def text_records(per_read, smem):
    out = []
    for i, recs in enumerate(per_read):
        out.append(HEADER % ("SMEM" if smem else "MEM", i + 1))
        for x, y, poss in recs:
            sign = "-" if (y >> 31) else "+"
            out.append("\nRead[%d, %d] -> %s%d" % (x & 0x7FFFFFFF, y & 0x7FFFFFFF, sign, poss[0]))
            for p in poss[1:]:
                out.append(", %s%d" % (sign, p))
        out.append("\n")
    return "".join(out)


def main():
    codes = random_reference(20_000, 2024)
    text = "".join("ACGT"[c] for c in codes)
    reads = sample_reads(codes, 60, seed=77, lengths=(19, 40, 100, 150), err=0.02, n_rate=0.3)
    with open(os.path.join(HERE, "ref20k.txt"), "w") as f:
        f.write(text + "\n")
    with open(os.path.join(HERE, "reads60.fa"), "wb") as f:
        for i, r in enumerate(reads):
            f.write(b">g%d\n%s\n" % (i + 1, r))
    for smem in (False, True):
        for n_stop in (False, True):
            per = [bf.seed_read(text, r, 19, smem, n_stop) for r in reads]
            name = "k19_%s_%s.txt" % ("smem" if smem else "mem", "nstop" if n_stop else "nwild")
            with open(os.path.join(HERE, name), "w") as f:
                f.write(text_records(per, smem))


if __name__ == "__main__":
    main()
