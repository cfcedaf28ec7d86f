"""Shared test helpers: small indexes built by the oracle's SA-IS, random reads."""
from __future__ import annotations

import os
import random

import numpy as np


def random_reference(n, seed, dups=6):
    r = np.random.default_rng(seed)
    codes = r.integers(0, 4, n, dtype=np.uint8)
    if n > 400:
        for _ in range(dups):
            a, b = r.integers(0, n - 300, 2)
            ln = int(r.integers(50, 300))
            codes[b:b + ln] = codes[a:a + ln]
    return codes


def build_index(tmpdir, codes, sa_intv=7, name="ref"):
    import pyoracle
    prefix = os.path.join(str(tmpdir), name)
    pyoracle.build_index(codes, sa_intv, prefix)
    return prefix


COMP = {"A": "T", "C": "G", "G": "C", "T": "A", "N": "N"}


def sample_reads(codes, n_reads, seed, lengths=(14, 20, 40, 60, 100), err=0.03, n_rate=0.2):
    rng = random.Random(seed)
    text = "".join("ACGT"[c] for c in codes)
    n = len(text)
    reads = []
    for _ in range(n_reads):
        L = min(rng.choice(lengths), n)
        st = rng.randrange(0, n - L + 1)
        s = list(text[st:st + L])
        if rng.random() < 0.5:
            s = [COMP[c] for c in reversed(s)]
        for i in range(L):
            if rng.random() < err:
                s[i] = rng.choice("ACGTN" if rng.random() < n_rate else "ACGT")
        reads.append("".join(s).encode())
    return reads


def pack(reads):
    lens = np.array([len(x) for x in reads], dtype=np.uint32)
    offs = np.zeros(len(reads), dtype=np.uint64)
    if len(reads):
        offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
    return b"".join(reads), offs, lens


def device_bytes(ptr, n):
    """n bytes of device memory at ptr, copied with the CUDA runtime."""
    import ctypes
    import glob
    if n == 0:
        return b""
    rt = None
    for name in ["libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    assert rt is not None, "CUDA runtime library not found"
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    buf = (ctypes.c_char * n)()
    assert rt.cudaMemcpy(ctypes.addressof(buf), ptr, n, 2) == 0   # device to host
    return bytes(buf)
