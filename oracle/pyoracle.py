"""ctypes front end of the CPU oracle (oracle.c / sa_build.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline,
never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

N_WILDCARD, N_STOP = 0, 1
LF_GPUSEED, LF_BWA = 0, 1


class _Params(C.Structure):
    _fields_ = [("k", C.c_int32), ("smem", C.c_int32), ("n_mode", C.c_int32), ("lf_mode", C.c_int32),
                ("mem_next", C.c_int32)]


class _Seed(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("l", C.c_uint32), ("u", C.c_uint32),
                ("n_pos", C.c_uint32)]


class _Batch(C.Structure):
    _fields_ = [("n_reads", C.c_uint32),
                ("read_n_seeds", C.POINTER(C.c_uint32)),
                ("read_seed_off", C.POINTER(C.c_uint64)),
                ("read_pos_off", C.POINTER(C.c_uint64)),
                ("n_seeds", C.c_uint64), ("n_pos", C.c_uint64),
                ("seeds", C.POINTER(_Seed)),
                ("pos", C.POINTER(C.c_uint32)),
                ("n_kmer", C.c_uint64), ("n_occ_blocks", C.c_uint64), ("n_lf", C.c_uint64),
                ("n_sa", C.c_uint64), ("n_steps", C.c_uint64),
                ("status", C.c_int32),
                ("read_n_fwd", C.POINTER(C.c_uint32))]


def build():
    """Compiles liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.or_index_load.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.or_index_from_arrays.argtypes = [u32, vp, vp, u64, u32, vp, u64, C.POINTER(vp)]
        L.or_index_free.argtypes = [vp]
        L.or_index_seq_len.argtypes = [vp]; L.or_index_seq_len.restype = u32
        L.or_index_primary.argtypes = [vp]; L.or_index_primary.restype = u32
        L.or_index_sa_intv.argtypes = [vp]; L.or_index_sa_intv.restype = u32
        L.or_index_L2.argtypes = [vp, vp]
        L.or_occ.argtypes = [vp, u32, i32]; L.or_occ.restype = u32
        L.or_lf.argtypes = [vp, u32, i32]; L.or_lf.restype = u32
        L.or_locate.argtypes = [vp, u32, i32, C.POINTER(u32)]; L.or_locate.restype = u32
        L.or_kmer_table.argtypes = [vp, i32, vp, i32]
        L.or_encode.argtypes = [C.c_char_p, u32, vp, vp]
        L.or_seed_batch.argtypes = [vp, vp, vp, vp, vp, u32, C.POINTER(_Params), i32, i32,
                                    C.POINTER(C.POINTER(_Batch))]
        L.or_batch_free.argtypes = [C.POINTER(_Batch)]
        L.or_batch_write_text.argtypes = [C.POINTER(_Batch), C.c_char_p, u32, i32, i32]
        L.or_build_index.argtypes = [vp, u64, u32, C.c_char_p]
        L.or_suffix_array.argtypes = [vp, u64, vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def suffix_array(codes: np.ndarray) -> np.ndarray:
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    out = np.empty(codes.size + 1, dtype=np.uint32)
    rc = lib().or_suffix_array(_ptr(codes), codes.size, _ptr(out))
    if rc:
        raise RuntimeError(f"or_suffix_array failed: {rc}")
    return out


def build_index(codes: np.ndarray, sa_intv: int, prefix: str) -> None:
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    rc = lib().or_build_index(_ptr(codes), codes.size, sa_intv, prefix.encode())
    if rc:
        raise RuntimeError(f"or_build_index failed: {rc}")


class Index:
    def __init__(self, prefix: str):
        h = C.c_void_p()
        rc = lib().or_index_load(prefix.encode(), C.byref(h))
        if rc:
            raise RuntimeError(f"or_index_load({prefix}) failed: {rc}")
        self.h = h
        self._table = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_index_free(self.h)
            self.h = None

    @property
    def seq_len(self):
        return lib().or_index_seq_len(self.h)

    @property
    def primary(self):
        return lib().or_index_primary(self.h)

    @property
    def sa_intv(self):
        return lib().or_index_sa_intv(self.h)

    @property
    def L2(self):
        a = np.zeros(5, dtype=np.uint32)
        lib().or_index_L2(self.h, _ptr(a))
        return a

    def occ(self, k, c):
        return lib().or_occ(self.h, k & 0xFFFFFFFF, c)

    def lf(self, row, lf_mode=LF_GPUSEED):
        return lib().or_lf(self.h, row, lf_mode)

    def locate(self, row, lf_mode=LF_GPUSEED):
        steps = C.c_uint32()
        p = lib().or_locate(self.h, row, lf_mode, C.byref(steps))
        return p, steps.value

    def kmer_table(self, K=13, threads=0) -> np.ndarray:
        out = np.empty(2 * (1 << (2 * K)), dtype=np.uint32)
        rc = lib().or_kmer_table(self.h, K, _ptr(out), threads)
        if rc:
            raise RuntimeError(f"or_kmer_table failed: {rc}")
        return out

    def table13(self, threads=0):
        if self._table is None:
            self._table = self.kmer_table(13, threads)
        return self._table

    def seed(self, seqs: bytes, offsets, lengths, k=20, smem=False, n_mode=N_WILDCARD,
             lf_mode=LF_GPUSEED, pruned=False, threads=0, use_table=False, table=None,
             mem_next=0) -> "Batch":
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
        buf = np.frombuffer(seqs, dtype=np.uint8) if isinstance(seqs, (bytes, bytearray)) else seqs
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        p = _Params(k, 1 if smem else 0, n_mode, lf_mode, mem_next)
        out = C.POINTER(_Batch)()
        if table is None and use_table:
            table = self.table13(threads)
        rc = lib().or_seed_batch(self.h, _ptr(table), _ptr(buf), _ptr(offsets), _ptr(lengths),
                                 lengths.size, C.byref(p), 1 if pruned else 0, threads,
                                 C.byref(out))
        if rc:
            raise RuntimeError(f"or_seed_batch failed: {rc}")
        return Batch(out)


class Batch:
    """Oracle output of one batch, copied into numpy arrays."""

    def __init__(self, ptr):
        b = ptr.contents
        n = b.n_reads
        self.n_reads = n
        self.read_n_seeds = np.ctypeslib.as_array(b.read_n_seeds, (n,)).copy() if n else np.zeros(0, np.uint32)
        self.read_seed_off = np.ctypeslib.as_array(b.read_seed_off, (n + 1,)).copy()
        self.read_pos_off = np.ctypeslib.as_array(b.read_pos_off, (n + 1,)).copy()
        ns, npos = b.n_seeds, b.n_pos
        if ns:
            raw = np.ctypeslib.as_array(C.cast(b.seeds, C.POINTER(C.c_uint32)), (ns * 5,)).copy()
            self.seeds = raw.reshape(ns, 5)  # x, y, l, u, n_pos (x, y as uint32 bit patterns)
        else:
            self.seeds = np.zeros((0, 5), np.uint32)
        self.pos = np.ctypeslib.as_array(b.pos, (npos,)).copy() if npos else np.zeros(0, np.uint32)
        self.read_n_fwd = np.ctypeslib.as_array(b.read_n_fwd, (n,)).copy() if n else np.zeros(0, np.uint32)
        self.work = dict(n_kmer=b.n_kmer, n_occ_blocks=b.n_occ_blocks, n_lf=b.n_lf, n_sa=b.n_sa,
                         n_steps=b.n_steps)
        self._ptr = ptr

    def write_text(self, path, first_read_no=1, smem=False, append=False):
        rc = lib().or_batch_write_text(self._ptr, path.encode(), first_read_no, 1 if smem else 0,
                                       1 if append else 0)
        if rc:
            raise RuntimeError(f"or_batch_write_text failed: {rc}")

    def __del__(self):
        if getattr(self, "_ptr", None):
            lib().or_batch_free(self._ptr)
            self._ptr = None

    def read_records(self, r):
        """[(x, y, [positions...]), ...] of read r in output order."""
        s0, s1 = self.read_seed_off[r], self.read_seed_off[r + 1]
        p = int(self.read_pos_off[r])
        out = []
        for s in range(s0, s1):
            x, y, l, u, n = (int(v) for v in self.seeds[s])
            out.append((x, y, l, u, self.pos[p:p + n].tolist()))
            p += n
        return out


def _ranges(starts, counts):
    """concatenation of arange(starts[i], starts[i] + counts[i]) and the read
    index of each element"""
    counts = counts.astype(np.int64)
    tot = int(counts.sum())
    reads = np.repeat(np.arange(counts.size, dtype=np.int64), counts)
    first = np.cumsum(counts) - counts
    return starts.astype(np.int64)[reads] + (np.arange(tot, dtype=np.int64) - first[reads]), reads


def mismatched_reads(ob: Batch, seeds, pos, read_seed_off, read_pos_off, r0=0,
                     cols=(0, 1, 2, 3, 4)) -> np.ndarray:
    """Reads of the oracle batch `ob` (its read i = read r0 + i of the other
    result) whose seeds or positions differ from the other result's: seed
    rows whose columns `cols` are [x, y, l, u, n_pos] (uint32; (0, 1, 2, 3, 6)
    for the library's gs_seed_rec rows), positions, and per-read offsets
    (n_reads + 1 entries).  Exact comparison, vectorised; returns the batch's
    read indices that differ."""
    n = ob.n_reads
    gso = np.asarray(read_seed_off[r0:r0 + n + 1], dtype=np.int64)
    gpo = np.asarray(read_pos_off[r0:r0 + n + 1], dtype=np.int64)
    oso = ob.read_seed_off[:n + 1].astype(np.int64)
    opo = ob.read_pos_off[:n + 1].astype(np.int64)
    ons, onp = np.diff(oso), np.diff(opo)
    bad = (np.diff(gso) != ons) | (np.diff(gpo) != onp)
    ok = ~bad
    oi, reads = _ranges(oso[:-1], np.where(ok, ons, 0))
    gi, _ = _ranges(gso[:-1], np.where(ok, ons, 0))
    if oi.size:
        rowbad = np.any(np.asarray(seeds)[gi][:, list(cols)] != ob.seeds[oi], axis=1)
        bad[np.unique(reads[rowbad])] = True
    oi, reads = _ranges(opo[:-1], np.where(ok, onp, 0))
    gi, _ = _ranges(gpo[:-1], np.where(ok, onp, 0))
    if oi.size:
        posbad = np.asarray(pos)[gi] != ob.pos[oi]
        bad[np.unique(reads[posbad])] = True
    return np.nonzero(bad)[0]
