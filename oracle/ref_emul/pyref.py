"""ctypes front end of the CPU build of the reference's own kernels.

TEST INFRASTRUCTURE ONLY (see build_ref.py).  run() seeds a batch through the
reference's kernel bodies and returns the text records seed_gen -o prints.
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "_ref")


def available(init="zero"):
    return os.path.exists(os.path.join(REF_DIR, f"libref_{init}.so"))


_libs = {}


def _lib(init):
    if init not in _libs:
        L = C.CDLL(os.path.join(REF_DIR, f"libref_{init}.so"))
        L.ref_run.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int,
                              C.c_int, C.c_char_p, C.c_void_p]
        _libs[init] = L
    return _libs[init]


def run(prefix, seqs: bytes, offs, lens, k, smem, init="zero", counts=False):
    """Text records; with counts=True also, per read, the forward records the
    reference's search kept after its own pruning."""
    offs = np.ascontiguousarray(offs, dtype=np.uint64)
    lens = np.ascontiguousarray(lens, dtype=np.uint32)
    buf = np.frombuffer(seqs, dtype=np.uint8) if isinstance(seqs, (bytes, bytearray)) else seqs
    buf = np.ascontiguousarray(buf, dtype=np.uint8)
    n_fwd = np.zeros(max(lens.size, 1), dtype=np.uint32)
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "out.txt")
        rc = _lib(init).ref_run(prefix.encode(), buf.ctypes.data, offs.ctypes.data, lens.ctypes.data,
                                lens.size, k, 1 if smem else 0, out.encode(), n_fwd.ctypes.data)
        if rc:
            raise RuntimeError(f"ref_run failed: {rc}")
        text = open(out).read()
    return (text, n_fwd[:lens.size]) if counts else text
