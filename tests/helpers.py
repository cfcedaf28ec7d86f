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


# ---------------------------------------------------------------------------
# an inconsistent index: an LF cycle that passes no sampled row

def _bwt_codes(words, seq_len):
    """the $-removed BWT string (codes 0..3) held by .bwt words after the header"""
    w = np.zeros((words.size + 7) // 8 * 8, np.uint32)
    w[:words.size] = words
    sh = (15 - np.arange(16, dtype=np.uint32)) * 2
    b = (w.reshape(-1, 8)[:, 4:, None] >> sh[None, None, :]) & 3
    return b.reshape(-1)[:seq_len].astype(np.uint8)


def _bwt_words(codes, words):
    """words with their base fields rewritten from codes (counts kept)"""
    full = np.zeros((words.size + 7) // 8 * 8, np.uint32)
    full[:words.size] = words
    full = full.reshape(-1, 8)
    pad = np.zeros(full.shape[0] * 64, np.uint32)
    pad[:codes.size] = codes
    sh = (15 - np.arange(16, dtype=np.uint32)) * 2
    packed = (pad.reshape(-1, 4, 16) << sh[None, None, :]).sum(axis=2, dtype=np.uint64)
    full[:, 4:] = packed.astype(np.uint32)
    return full.reshape(-1)[:words.size]


def _lf(L, primary, L2):
    """LF of every row 0..seq_len (row primary holds $ and maps to row 0)"""
    n = L.size
    rows = np.arange(n + 1)
    ka = np.minimum(rows - (rows > primary), n - 1)
    lf = np.zeros(n + 1, np.int64)
    for c in range(4):
        rank = np.cumsum(L == c)
        sel = (rows != primary) & (L[ka] == c)
        lf[sel] = L2[c] + rank[ka[sel]]
    lf[primary] = 0
    return lf


def _cycles(perm):
    seen = np.zeros(perm.size, bool)
    out = []
    for s in range(perm.size):
        x, c = s, []
        while not seen[x]:
            seen[x] = True
            c.append(x)
            x = perm[x]
        if c:
            out.append(c)
    return out


def lf_cycle_index(tmpdir, n=3000, sa_intv=16, seed=77, read_len=40):
    """Index arrays (primary, L2[1..4], .bwt words, SA samples, sa_intv) of a
    random text whose BWT has two bases of one 64-row block swapped -- the
    block counts stay right, so the files load -- chosen so that LF has a
    cycle through no sampled row; and a read whose forward seed's interval
    holds a row of that cycle, so locating it by LF steps never ends."""
    prefix = build_index(tmpdir, random_reference(n, seed, dups=0), sa_intv=sa_intv, name="cyc")
    bwt = np.fromfile(prefix + ".bwt", np.uint32)
    sa = np.fromfile(prefix + ".sa", np.uint32)
    primary = int(bwt[0])
    L2 = np.concatenate([[0], bwt[1:5]]).astype(np.int64)
    L = _bwt_codes(bwt[5:], int(L2[4]))
    assert len(_cycles(_lf(L, primary, L2))) == 1      # a consistent index: one cycle
    rng = np.random.default_rng(seed)
    for _ in range(100_000):
        blk = int(rng.integers(0, L.size // 64))
        i, j = (blk * 64 + rng.integers(0, 64, 2)).tolist()
        if L[i] == L[j]:
            continue
        M = L.copy()
        M[i], M[j] = L[j], L[i]
        lf = _lf(M, primary, L2)
        bad = [c for c in _cycles(lf) if all(r % sa_intv for r in c) and primary not in c]
        if not bad:
            continue
        # R[e - t] is the BWT base of LF^t(row): backward search of the read
        # keeps LF^(t+1)(row), a row of the cycle, in its interval
        row, read = bad[0][0], []
        for _ in range(read_len):
            read.append("ACGT"[M[row - (row > primary)]])
            row = lf[row]
        arrays = (primary, bwt[1:5].copy(), _bwt_words(M, bwt[5:]), sa[7:].copy(), sa_intv)
        return arrays, "".join(reversed(read)).encode()
    raise AssertionError("no swap gave an unsampled cycle")
