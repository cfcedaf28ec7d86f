"""gpuseed_gb300 -- GB300-native seeding (MEM/SMEM by FM-index backward search).

Python front end of libgpuseed.so, mirroring the reference's seed_gen interface
(nahmedraja/GPUseed seed_gen.cu:2817-3815): an index loaded from the .bwt/.sa
files, a batch of reads, the -k/-s switches, and seeds in the reference's
output order and text format.  All compute runs in the CUDA library; importing
this module fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libgpuseed.so")
CLI_PATH = os.path.join(_PKG, "seed_gen")

N_WILDCARD, N_STOP = 0, 1
LF_GPUSEED, LF_BWA = 0, 1
KERNEL_BATCHED, KERNEL_PLAIN, KERNEL_LOCKSTEP = 0, 1, 2
MEM_NEXT_READ, MEM_NEXT_GPUSEED = 0, 1

GS_ERRORS = {-1: "EINVAL", -2: "EIO", -3: "EFORMAT", -4: "ENOMEM", -5: "ECUDA", -6: "EWALK",
             -7: "EOVERFLOW", -8: "ETIMEOUT", -9: "ESTATE"}

# Every symbol include/gpuseed.h declares.
EXPORTS = ["gs_index_load", "gs_index_from_host", "gs_index_build", "gs_index_set_kmer_len", "gs_index_set_text", "gs_index_text_table", "gs_index_free", "gs_index_get_info",
           "gs_index_kmer_table", "gs_index_set_l2_window", "gs_ctx_create", "gs_ctx_free",
           "gs_seed", "gs_seed_device", "gs_result_host", "gs_result_device",
           "gs_result_write_text", "gs_result_write_text_host", "gs_result_text_device",
           "gs_ctx_stream", "gs_ctx_last_timing", "gs_ctx_last_work",
           "gs_ctx_last_walkers", "gs_ctx_last_text_jobs",
           "gs_seed_noalloc", "gs_autotune", "gs_server_start", "gs_server_submit", "gs_server_wait",
           "gs_server_result", "gs_server_release", "gs_server_get_stats", "gs_server_stop", "gs_server_replay",
           "gs_last_error",
           "gs_strerror", "gs_version"]


class GsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{GS_ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("k", C.c_int32), ("smem", C.c_int32), ("n_mode", C.c_int32),
                ("lf_mode", C.c_int32), ("kernel", C.c_int32), ("queue_chunk", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("count_work", C.c_int32),
                ("handoff_lanes", C.c_int32), ("handoff_steps", C.c_int32), ("graph", C.c_int32),
                ("walker_slots", C.c_int32), ("max_occ", C.c_int32), ("mem_next", C.c_int32)]


class SeedRec(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("l", C.c_uint32), ("u", C.c_uint32),
                ("xl", C.c_uint32), ("xu", C.c_uint32), ("n_pos", C.c_uint32),
                ("pad", C.c_uint32)]


class ResultView(C.Structure):
    _fields_ = [("n_reads", C.c_uint32), ("n_seeds", C.c_uint64), ("n_pos", C.c_uint64),
                ("read_seed_off", C.POINTER(C.c_uint64)), ("read_pos_off", C.POINTER(C.c_uint64)),
                ("seeds", C.POINTER(SeedRec)), ("pos", C.POINTER(C.c_uint32))]


class ServerOpts(C.Structure):
    _fields_ = [("n_slots", C.c_int32), ("max_batch_reads", C.c_int32), ("hbm_budget", C.c_uint64),
                ("params", Params)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "failed", "passes", "reads",
                                          "max_batch_reads", "pending", "reserved_bytes",
                                          "budget_bytes", "submit_us", "merge_us", "seed_us",
                                          "split_us")]


class IndexInfo(C.Structure):
    _fields_ = [("seq_len", C.c_uint32), ("primary", C.c_uint32), ("sa_intv", C.c_uint32),
                ("n_sa", C.c_uint32), ("L2", C.c_uint32 * 5), ("device", C.c_int32),
                ("device_bytes", C.c_uint64), ("kmer_len", C.c_int32), ("text_min", C.c_int32)]


_lib = None


def lib():
    """Loads libgpuseed.so; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                              "(nvcc for sm_103a); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.gs_index_load.argtypes = [C.c_char_p, i32, C.POINTER(vp)]
        L.gs_index_from_host.argtypes = [u32, vp, vp, u64, u32, vp, u64, i32, C.POINTER(vp)]
        L.gs_index_build.argtypes = [vp, u64, u32, i32, C.c_char_p, C.POINTER(vp)]
        L.gs_index_free.argtypes = [vp]
        L.gs_index_get_info.argtypes = [vp, C.POINTER(IndexInfo)]
        L.gs_index_kmer_table.argtypes = [vp, u64, u64, vp]
        L.gs_index_set_l2_window.argtypes = [vp, C.c_float]
        L.gs_index_set_kmer_len.argtypes = [vp, i32]
        L.gs_index_set_text.argtypes = [vp, i32]
        L.gs_index_text_table.argtypes = [vp, i32, u64, u64, vp]
        L.gs_ctx_create.argtypes = [vp, vp, C.POINTER(vp)]
        L.gs_ctx_free.argtypes = [vp]
        L.gs_seed.argtypes = [vp, vp, vp, vp, u32, C.POINTER(Params)]
        L.gs_seed_device.argtypes = [vp, vp, vp, vp, u32, C.POINTER(Params), i32]
        L.gs_result_host.argtypes = [vp, C.POINTER(ResultView)]
        L.gs_result_device.argtypes = [vp, C.POINTER(ResultView)]
        L.gs_result_write_text.argtypes = [vp, i32, u32, i32]
        L.gs_result_write_text_host.argtypes = [vp, i32, u32, i32]
        L.gs_result_text_device.argtypes = [vp, u32, i32, C.POINTER(vp), C.POINTER(u64)]
        L.gs_ctx_stream.argtypes = [vp]
        L.gs_ctx_stream.restype = vp
        L.gs_ctx_last_timing.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.gs_ctx_last_work.argtypes = [vp, vp]
        L.gs_ctx_last_walk_counts.argtypes = [vp, vp]
        L.gs_ctx_last_walkers.argtypes = [vp, C.POINTER(u64), C.POINTER(u64)]
        L.gs_ctx_last_text_jobs.argtypes = [vp, C.POINTER(u64), C.POINTER(u64)]
        L.gs_autotune.argtypes = [vp, vp, vp, vp, u32, C.POINTER(Params), u32, C.POINTER(C.c_float)]
        L.gs_server_start.argtypes = [vp, C.POINTER(ServerOpts), C.POINTER(vp)]
        L.gs_server_submit.argtypes = [vp, vp, vp, vp, u32, C.POINTER(u64)]
        L.gs_server_submit_ref.argtypes = [vp, vp, vp, vp, u32, C.POINTER(u64)]
        L.gs_server_wait.argtypes = [vp, u64, i32]
        L.gs_server_result.argtypes = [vp, u64, C.POINTER(ResultView), C.POINTER(C.c_double)]
        L.gs_server_release.argtypes = [vp, u64]
        L.gs_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
        L.gs_server_stop.argtypes = [vp]
        L.gs_server_replay.argtypes = [vp, vp, vp, vp, u32, vp, vp, vp, vp, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
        L.gs_seed_noalloc.argtypes = [vp, vp, vp, vp, u32, C.POINTER(Params), vp, vp, u64, vp, u64,
                                      vp, vp, C.POINTER(u64), C.POINTER(u64)]
        L.gs_last_error.restype = C.c_char_p
        L.gs_strerror.restype = C.c_char_p
        L.gs_strerror.argtypes = [i32]
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        raise GsError(rc, lib().gs_last_error().decode(errors="replace"))
    return rc


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Index:
    """Device-resident index (.bwt + .sa + 13-mer table)."""

    def __init__(self, prefix: str | None = None, device: int = 0, *, arrays=None):
        h = C.c_void_p()
        if arrays is not None:
            primary, L2_1to4, bwt, sa_samples, sa_intv = arrays
            L2a = np.ascontiguousarray(L2_1to4, dtype=np.uint32)
            bwt = np.ascontiguousarray(bwt, dtype=np.uint32)
            sa_samples = np.ascontiguousarray(sa_samples, dtype=np.uint32)
            check(lib().gs_index_from_host(primary, _ptr(L2a), _ptr(bwt), bwt.size, sa_intv,
                                           _ptr(sa_samples), sa_samples.size, device, C.byref(h)))
        else:
            check(lib().gs_index_load(prefix.encode(), device, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().gs_index_free(self.h)
            self.h = None

    __del__ = close

    def info(self) -> IndexInfo:
        inf = IndexInfo()
        check(lib().gs_index_get_info(self.h, C.byref(inf)))
        return inf

    def kmer_table(self, first=0, count=None) -> np.ndarray:
        if count is None:
            count = (1 << 26) - first
        out = np.empty(2 * count, dtype=np.uint32)
        check(lib().gs_index_kmer_table(self.h, first, count, _ptr(out)))
        return out

    def set_kmer_len(self, kmer_len: int):
        check(lib().gs_index_set_kmer_len(self.h, kmer_len))

    def text_table(self, which: int) -> np.ndarray:
        """Full SA (0), packed text words (1) or inverse-SA samples (2)."""
        info = self.info()
        n = {0: info.seq_len + 1, 1: (info.seq_len + 15) // 16, 2: info.seq_len // 2 + 1}[which]
        out = np.empty(n, dtype=np.uint32)
        check(lib().gs_index_text_table(self.h, which, 0, n, _ptr(out)))
        return out

    def set_text(self, min_steps: int):
        """Text structures: > 0 build and enter text mode after min_steps
        one-row steps; < 0 build, locate only; 0 free them."""
        check(lib().gs_index_set_text(self.h, min_steps))

    def set_l2_window(self, hit_ratio: float):
        check(lib().gs_index_set_l2_window(self.h, hit_ratio))


def build_index(codes, sa_intv: int = 7, prefix: str | None = None, device: int = 0,
                load: bool = True):
    """Builds the .bwt/.sa index of a forward-strand text (codes 0..3) on the GPU;
    writes the files when `prefix` is given and returns the loaded Index when `load`."""
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    h = C.c_void_p()
    check(lib().gs_index_build(_ptr(codes), codes.size, sa_intv, device,
                               prefix.encode() if prefix else None, C.byref(h) if load else None))
    if not load:
        return None
    idx = Index.__new__(Index)
    idx.h = h
    return idx


def seed_noalloc(index: Index, d_seqs: int, d_offsets: int, d_lengths: int, n_reads: int,
                 d_seeds: int, seed_cap: int, d_pos: int, pos_cap: int, d_read_seed_off: int,
                 d_read_pos_off: int, stream: int = 0, **kw):
    """gs_seed_noalloc: the batched pass with no allocation (device pointers in
    and out); returns (n_seeds, n_pos)."""
    p = Context.params(**kw)
    ns, npos = C.c_uint64(), C.c_uint64()
    check(lib().gs_seed_noalloc(index.h, C.c_void_p(d_seqs), C.c_void_p(d_offsets),
                                C.c_void_p(d_lengths), n_reads, C.byref(p),
                                C.c_void_p(stream) if stream else None, C.c_void_p(d_seeds),
                                seed_cap, C.c_void_p(d_pos), pos_cap, C.c_void_p(d_read_seed_off),
                                C.c_void_p(d_read_pos_off), C.byref(ns), C.byref(npos)))
    return int(ns.value), int(npos.value)


class Result:
    """Host copy of one batch's seeds in output order."""

    def __init__(self, view: ResultView):
        n = view.n_reads
        self.n_reads = n
        self.read_seed_off = np.ctypeslib.as_array(view.read_seed_off, (n + 1,)).copy()
        self.read_pos_off = np.ctypeslib.as_array(view.read_pos_off, (n + 1,)).copy()
        ns, npos = int(view.n_seeds), int(view.n_pos)
        if ns:
            raw = np.ctypeslib.as_array(C.cast(view.seeds, C.POINTER(C.c_uint32)), (ns * 8,))
            self.seeds = raw.reshape(ns, 8).copy()  # x y l u xl xu n_pos pad
        else:
            self.seeds = np.zeros((0, 8), np.uint32)
        self.pos = np.ctypeslib.as_array(view.pos, (npos,)).copy() if npos else np.zeros(0, np.uint32)

    def read_records(self, r):
        """[(x, y, l, u, [positions...]), ...] of read r in output order."""
        out = []
        p = int(self.read_pos_off[r])
        for s in range(int(self.read_seed_off[r]), int(self.read_seed_off[r + 1])):
            x, y, l, u, xl, xu, n, _ = (int(v) for v in self.seeds[s])
            out.append((x, y, l, u, self.pos[p:p + n].tolist()))
            p += n
        return out


class Context:
    """One stream + workspace; seeds batches of reads."""

    def __init__(self, index: Index, stream=None):
        self.index = index
        h = C.c_void_p()
        check(lib().gs_ctx_create(index.h, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().gs_ctx_free(self.h)
            self.h = None

    __del__ = close

    @staticmethod
    def params(k=20, smem=False, n_mode=N_WILDCARD, lf_mode=LF_GPUSEED, kernel=KERNEL_BATCHED,
               queue_chunk=0, ctas_per_sm=0, count_work=False, handoff_lanes=0,
               handoff_steps=0, graph=False, walker_slots=0, max_occ=0,
               mem_next=0) -> Params:
        return Params(k, 1 if smem else 0, n_mode, lf_mode, kernel, queue_chunk, ctas_per_sm,
                      1 if count_work else 0, handoff_lanes, handoff_steps, 1 if graph else 0,
                      walker_slots, max_occ, mem_next)

    def seed(self, seqs, offsets, lengths, **kw) -> Result:
        """Reads in host memory; returns the host result."""
        buf = np.frombuffer(seqs, dtype=np.uint8) if isinstance(seqs, (bytes, bytearray)) else \
            np.ascontiguousarray(seqs, dtype=np.uint8)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
        p = self.params(**kw)
        check(lib().gs_seed(self.h, _ptr(buf), _ptr(offsets), _ptr(lengths), lengths.size,
                            C.byref(p)))
        return self.result()

    def seed_device(self, d_seqs: int, d_offsets: int, d_lengths: int, n_reads: int,
                    fetch=False, **kw):
        """Reads already in device memory (raw device pointers)."""
        p = self.params(**kw)
        check(lib().gs_seed_device(self.h, C.c_void_p(d_seqs), C.c_void_p(d_offsets),
                                   C.c_void_p(d_lengths), n_reads, C.byref(p), 1 if fetch else 0))
        return self.result() if fetch else None

    def autotune(self, d_seqs: int, d_offsets: int, d_lengths: int, n_reads: int,
                 sample: int = 1 << 20, **kw):
        """Fastest launch knobs on a sample of device-resident reads: (params dict, search ms)."""
        p = self.params(**kw)
        ms = C.c_float()
        check(lib().gs_autotune(self.h, C.c_void_p(d_seqs), C.c_void_p(d_offsets),
                                C.c_void_p(d_lengths), n_reads, C.byref(p), sample, C.byref(ms)))
        knobs = {n: getattr(p, n) for n in ("queue_chunk", "ctas_per_sm", "handoff_lanes",
                                            "handoff_steps")}
        return knobs, ms.value

    def result(self) -> Result:
        v = ResultView()
        check(lib().gs_result_host(self.h, C.byref(v)))
        return Result(v)

    def device_counts(self):
        v = ResultView()
        check(lib().gs_result_device(self.h, C.byref(v)))
        return int(v.n_seeds), int(v.n_pos)

    def write_text(self, fd: int, first_read_no: int = 1, smem: bool = False, host=False):
        """The -o records to an open fd (formatted on the GPU unless host=True)."""
        f = lib().gs_result_write_text_host if host else lib().gs_result_write_text
        check(f(self.h, fd, first_read_no, 1 if smem else 0))

    def text_device(self, first_read_no: int = 1, smem: bool = False):
        """(device pointer, bytes) of the -o records formatted on the GPU."""
        d, n = C.c_void_p(), C.c_uint64()
        check(lib().gs_result_text_device(self.h, first_read_no, 1 if smem else 0, C.byref(d),
                                          C.byref(n)))
        return int(d.value or 0), int(n.value)

    def stream(self) -> int:
        return lib().gs_ctx_stream(self.h) or 0

    def last_work(self):
        """{n_kmer, n_occ_blocks, n_lf, n_sa} of the last count_work pass."""
        a = np.zeros(4, dtype=np.uint64)
        check(lib().gs_ctx_last_work(self.h, _ptr(a)))
        return dict(n_kmer=int(a[0]), n_occ_blocks=int(a[1]), n_lf=int(a[2]), n_sa=int(a[3]))

    def last_walk_counts(self):
        """walk-pass counters of the last count_work batched pass"""
        a = np.zeros(7, dtype=np.uint64)
        check(lib().gs_ctx_last_walk_counts(self.h, _ptr(a)))
        return dict(zip(("steps", "steps_with_j", "j_only_blocks", "j_steps_i_shrank",
                         "walkers_with_j", "lines_256_rows", "lines_384_rows"),
                        (int(v) for v in a)))

    def last_walkers(self):
        """(walkers handed to the walk pass, buffer capacity) of the last batched pass."""
        n, cap = C.c_uint64(), C.c_uint64()
        check(lib().gs_ctx_last_walkers(self.h, C.byref(n), C.byref(cap)))
        return int(n.value), int(cap.value)

    def last_text_jobs(self):
        """(walkers handed to the text pass, room for them) of the last batched pass."""
        n, cap = C.c_uint64(), C.c_uint64()
        check(lib().gs_ctx_last_text_jobs(self.h, C.byref(n), C.byref(cap)))
        return int(n.value), int(cap.value)

    def last_timing(self):
        a, b = C.c_float(), C.c_float()
        check(lib().gs_ctx_last_timing(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value


class Server:
    """Serving loop: resident index, requests merged into passes as slots free up."""

    def __init__(self, index: Index, n_slots=0, max_batch_reads=0, hbm_budget=0, **params):
        self.index = index
        o = ServerOpts(n_slots, max_batch_reads, hbm_budget, Context.params(**params))
        h = C.c_void_p()
        check(lib().gs_server_start(index.h, C.byref(o), C.byref(h)))
        self.h = h
        self._held = {}

    def submit(self, seqs, offsets, lengths, copy=True) -> int:
        """copy=False: gs_server_submit_ref -- the bases are read in place,
        and this object keeps the buffer alive until the request is released"""
        buf = np.frombuffer(seqs, dtype=np.uint8) if isinstance(seqs, (bytes, bytearray)) else \
            np.ascontiguousarray(seqs, dtype=np.uint8)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
        rid = C.c_uint64()
        fn = lib().gs_server_submit if copy else lib().gs_server_submit_ref
        check(fn(self.h, _ptr(buf), _ptr(offsets), _ptr(lengths), lengths.size, C.byref(rid)))
        if not copy:
            self._held[rid.value] = buf
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1) -> int:
        return lib().gs_server_wait(self.h, rid, timeout_ms)

    def result(self, rid: int, release: bool = True):
        v = ResultView()
        lat = C.c_double()
        check(lib().gs_server_result(self.h, rid, C.byref(v), C.byref(lat)))
        res = Result(v)
        if release:
            lib().gs_server_release(self.h, rid)
            self._held.pop(rid, None)
        return res, lat.value

    def replay(self, pool_seqs, pool_offsets, pool_lengths, first, count, gap_ms):
        """Submits requests on a schedule from C and waits for all of them:
        (latencies ms, wall ms, submission span ms)."""
        first = np.ascontiguousarray(first, dtype=np.uint32)
        count = np.ascontiguousarray(count, dtype=np.uint32)
        gap = np.ascontiguousarray(gap_ms, dtype=np.float64)
        lat = np.zeros(first.size, dtype=np.float64)
        wall, sub = C.c_double(), C.c_double()
        check(lib().gs_server_replay(self.h, _ptr(pool_seqs), _ptr(np.ascontiguousarray(pool_offsets, np.uint64)),
                                     _ptr(np.ascontiguousarray(pool_lengths, np.uint32)), first.size,
                                     _ptr(first), _ptr(count), _ptr(gap), _ptr(lat), C.byref(wall),
                                     C.byref(sub)))
        return lat, wall.value, sub.value

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().gs_server_get_stats(self.h, C.byref(st)))
        return {n: getattr(st, n) for n, _ in ServerStats._fields_}

    def stop(self):
        if getattr(self, "h", None):
            lib().gs_server_stop(self.h)
            self.h = None

    __del__ = stop
