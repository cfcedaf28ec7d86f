"""The bidirectional design's alternative stop, counted: a walker that drops
J and checks containment once at its natural end (the check a right
extension allows) walks every contained candidate on to the end of its match.

`walk_forms.c` counts both forms with the oracle's FM primitives on config
3's composition (seeded synthetic reference and reads, k = 19).  The
canonical containment-stopped walk is what every kernel here does; the
monotone form's extra steps are what it would add.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_monotone_check_walks_far_more(built, tmp_path):
    from gpuseed_gb300 import workloads as W
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "walk_forms")
    subprocess.run([gcc, "-O2", "-o", exe, os.path.join(HERE, "walk_forms.c"),
                    os.path.join(ROOT, "oracle", "oracle.c"), os.path.join(ROOT, "oracle", "sa_build.c"),
                    "-I", os.path.join(ROOT, "oracle"), "-lpthread", "-lm"], check=True)
    codes, nmask = W.make_reference(W.ref_spec(3, 4_000_000))
    prefix = str(tmp_path / "ref")
    pyoracle.build_index(codes, 7, prefix)
    seqs, offs, lens = W.make_reads(codes, nmask, W.read_spec(3, 20_000))
    b = np.frombuffer(seqs, np.uint8) if not isinstance(seqs, np.ndarray) else seqs
    with open(tmp_path / "reads.txt", "w") as f:
        for o, n in zip(offs, lens):
            f.write(bytes(b[o:o + n]).decode() + "\n")
    out = subprocess.run([exe, prefix, str(tmp_path / "reads.txt"), "19", "20000"],
                         capture_output=True, check=True, text=True).stdout
    c = json.loads(out)
    print(c)
    assert c["reads"] == 20_000
    assert c["steps_canonical"] == c["steps_with_j"] + c["steps_without_j"]
    assert 0 < c["j_steps_i_shrank"] <= c["steps_with_j"]
    assert c["killed"] > 0
    # the monotone form's extra steps dwarf the whole canonical walk
    assert c["extra_steps_to_natural_end"] > 3 * c["steps_canonical"]
