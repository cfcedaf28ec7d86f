"""C-ABI library: loads, exports every declared symbol, rejects bad input
without a GPU (file checks happen before any CUDA call)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(built):
    import gpuseed_gb300 as gs
    L = C.CDLL(gs.LIB_PATH)
    names = declared("gpuseed.h") + declared("gpuseed_synth.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(gs.EXPORTS) <= set(declared("gpuseed.h"))


def test_strerror_and_version(built):
    import gpuseed_gb300 as gs
    L = gs.lib()
    assert L.gs_version() >= 100
    assert L.gs_strerror(-3) == b"index format error"


def _write_index(d, primary=5, seq_len=100, words=None, sa_primary=None, sa_len=None, sa_n=None):
    L2 = [25, 50, 75, seq_len]
    n_occ = (seq_len + 63) // 64 + 1
    need = 4 * n_occ + (seq_len + 15) // 16
    w = need if words is None else words
    with open(os.path.join(d, "x.bwt"), "wb") as f:
        f.write(np.array([primary] + L2, dtype=np.uint32).tobytes())
        f.write(np.zeros(w, dtype=np.uint32).tobytes())
    n_sa = (seq_len + 7) // 7
    with open(os.path.join(d, "x.sa"), "wb") as f:
        hdr = [primary if sa_primary is None else sa_primary] + L2 + [7, seq_len if sa_len is None else sa_len]
        f.write(np.array(hdr, dtype=np.uint32).tobytes())
        f.write(np.zeros((n_sa - 1) if sa_n is None else sa_n, dtype=np.uint32).tobytes())
    return os.path.join(d, "x")


@pytest.mark.parametrize("case,code", [
    ("missing", -2),
    ("truncated_bwt", -3),
    ("primary_mismatch", -3),
    ("seq_len_mismatch", -3),
    ("short_sa", -3),
])
def test_index_load_rejects_bad_files(built, tmp_path, case, code):
    import gpuseed_gb300 as gs
    d = str(tmp_path)
    if case == "missing":
        prefix = os.path.join(d, "nothing")
    elif case == "truncated_bwt":
        prefix = _write_index(d, words=3)
    elif case == "primary_mismatch":
        prefix = _write_index(d, sa_primary=6)
    elif case == "seq_len_mismatch":
        prefix = _write_index(d, sa_len=99)
    else:
        prefix = _write_index(d, sa_n=2)
    with pytest.raises(gs.GsError) as e:
        gs.Index(prefix)
    assert e.value.code == code


def test_null_arguments(built):
    import gpuseed_gb300 as gs
    L = gs.lib()
    assert L.gs_seed(None, None, None, None, 0, None) == -1
    assert L.gs_index_load(None, 0, None) == -1
    assert L.gs_result_host(None, None) == -1
    assert L.gs_index_set_text(None, 4) == -1
    assert L.gs_index_text_table(None, 0, 0, 0, None) == -1
    assert L.gs_ctx_last_text_jobs(None, None, None) == -1
    assert L.gs_ctx_last_walkers(None, None, None) == -1


def test_python_structs_match_the_header(built, tmp_path):
    """Every ctypes mirror of a header struct has the C size and field offsets
    (gcc on include/gpuseed.h prints them)."""
    import subprocess
    import gpuseed_gb300 as gs
    mirrors = {"gs_params": gs.Params, "gs_seed_rec": gs.SeedRec, "gs_result_view": gs.ResultView,
               "gs_index_info": gs.IndexInfo, "gs_server_opts": gs.ServerOpts,
               "gs_server_stats": gs.ServerStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gpuseed.h"', 'int main(void) {']
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, check=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
