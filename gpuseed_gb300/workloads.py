"""Seeded synthetic workloads standing in for the reference's benchmark configs.

No public dataset is used by the reference or named for its metric; these
specs reproduce the shapes, sizes and distributions of the five configs
(reference length and composition, read count, read-length distribution,
error model, k and mode) with the generator in gs_synth.c.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import lib as _gslib


class RefSpec(C.Structure):
    _fields_ = [("length", C.c_uint64), ("seed", C.c_uint64), ("gc", C.c_double),
                ("dup_frac", C.c_double), ("dup_len_min", C.c_uint32), ("dup_len_max", C.c_uint32),
                ("dup_div_min", C.c_double), ("dup_div_max", C.c_double),
                ("fam_unit", C.c_uint32), ("fam_copies", C.c_uint32), ("fam_count", C.c_uint32),
                ("fam_div_min", C.c_double), ("fam_div_max", C.c_double),
                ("n_frac", C.c_double), ("n_block_min", C.c_uint32), ("n_block_max", C.c_uint32)]


class ReadSpec(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_reads", C.c_uint32), ("len_mode", C.c_uint32),
                ("len_fixed", C.c_uint32), ("n_choices", C.c_uint32),
                ("len_choices", C.c_uint32 * 8), ("ln_median", C.c_double), ("ln_sigma", C.c_double),
                ("len_min", C.c_uint32), ("len_max", C.c_uint32), ("sub_rate", C.c_double),
                ("indel_rate", C.c_double), ("indel_max", C.c_uint32), ("nrun_frac", C.c_double),
                ("nrun_min", C.c_uint32), ("nrun_max", C.c_uint32)]


LEN_FIXED, LEN_CHOICE, LEN_LOGNORMAL, LEN_UNIFORM = 0, 1, 2, 3


def ref_spec(config: int, length: int | None = None) -> RefSpec:
    """Reference composition of a config; `length` rescales it (repeats scale along)."""
    s = RefSpec()
    s.seed = 0x5EED0000 + config
    if config == 1:
        s.length = length or 1_000_000
        s.gc = 0.5
        s.dup_frac, s.dup_len_min, s.dup_len_max = 0.02, 500, 500
        s.dup_div_min = s.dup_div_max = 0.01
    else:
        s.length = length or (100_000_000 if config == 2 else 3_100_000_000)
        s.gc = 0.41
        s.dup_frac, s.dup_len_min, s.dup_len_max = 0.05, 1000, 10000
        s.dup_div_min, s.dup_div_max = 0.01, 0.03
        s.fam_unit, s.fam_copies = 300, 20000
        s.fam_div_min, s.fam_div_max = 0.10, 0.15
        if config == 2:
            s.fam_count = 1
        else:
            # repeats scaled to 45% of the sequence: 5% segdups + families
            s.fam_count = max(1, int(0.40 * s.length / (300 * 20000)))
            s.n_frac, s.n_block_min, s.n_block_max = 0.01, 1000, 100000
        if s.fam_unit * s.fam_copies * s.fam_count > s.length:
            s.fam_copies = max(1, int(s.length // (4 * s.fam_unit)))
    return s


def read_spec(config: int, n_reads: int | None = None) -> ReadSpec:
    r = ReadSpec()
    r.seed = 0x5EED1000 + config
    if config == 1:
        r.n_reads = n_reads or 10_000
        r.len_mode, r.len_fixed = LEN_FIXED, 100
        r.sub_rate = 0.005
    elif config == 2:
        r.n_reads = n_reads or 1_000_000
        r.len_mode, r.len_fixed = LEN_FIXED, 150
        r.sub_rate, r.indel_rate, r.indel_max = 0.01, 0.0005, 3
        r.nrun_frac, r.nrun_min, r.nrun_max = 0.001, 5, 20
    elif config == 3:
        r.n_reads = n_reads or 10_000_000
        r.len_mode, r.n_choices = LEN_CHOICE, 5
        for i, v in enumerate((50, 75, 100, 150, 250)):
            r.len_choices[i] = v
        r.sub_rate, r.indel_rate, r.indel_max = 0.01, 0.0005, 3
    elif config == 4:
        r.n_reads = n_reads or 200_000
        r.len_mode = LEN_LOGNORMAL
        r.ln_median, r.ln_sigma, r.len_min, r.len_max = 2000.0, 0.6, 500, 10000
        r.sub_rate, r.indel_rate, r.indel_max = 0.02, 0.01, 3
    else:
        r.n_reads = n_reads or 4096
        r.len_mode, r.len_min, r.len_max = LEN_UNIFORM, 100, 250
        r.sub_rate = 0.01
    return r


CONFIG_K = {1: 20, 2: 19, 3: 19, 4: 20, 5: 19}
CONFIG_SMEM = {1: False, 2: True, 3: True, 4: False, 5: True}


def _setup():
    L = _gslib()
    if not hasattr(L, "_synth_ready"):
        L.gs_synth_reference.argtypes = [C.POINTER(RefSpec), C.c_void_p, C.c_void_p, C.c_int]
        L.gs_synth_reads_capacity.argtypes = [C.POINTER(ReadSpec)]
        L.gs_synth_reads_capacity.restype = C.c_uint64
        L.gs_synth_reads.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(ReadSpec),
                                     C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int]
        L._synth_ready = True
    return L


def make_reference(spec: RefSpec, threads: int = 0):
    """(codes uint8[n] in 0..3, nmask uint8[n])."""
    L = _setup()
    codes = np.empty(spec.length, dtype=np.uint8)
    nmask = np.empty(spec.length, dtype=np.uint8)
    rc = L.gs_synth_reference(C.byref(spec), codes.ctypes.data, nmask.ctypes.data,
                              threads or (os.cpu_count() or 8))
    if rc:
        raise RuntimeError(f"gs_synth_reference failed: {rc}")
    return codes, nmask


def make_reads(codes, nmask, spec: ReadSpec, threads: int = 0):
    """(seqs uint8[], offsets uint64[n], lengths uint32[n]) of ASCII reads."""
    L = _setup()
    cap = L.gs_synth_reads_capacity(C.byref(spec))
    seqs = np.empty(cap, dtype=np.uint8)
    offs = np.empty(spec.n_reads, dtype=np.uint64)
    lens = np.empty(spec.n_reads, dtype=np.uint32)
    rc = L.gs_synth_reads(codes.ctypes.data, nmask.ctypes.data if nmask is not None else None,
                          codes.size, C.byref(spec), seqs.ctypes.data, cap, offs.ctypes.data,
                          lens.ctypes.data, threads or (os.cpu_count() or 8))
    if rc:
        raise RuntimeError(f"gs_synth_reads failed: {rc}")
    total = int(offs[-1] + lens[-1]) if spec.n_reads else 0
    return seqs[:total], offs, lens


def write_fasta_reads(path, seqs, offs, lens):
    """One sequence line per read, as seed_gen reads them (seed_gen.cu:2955-2990)."""
    with open(path, "wb") as f:
        for i in range(lens.size):
            o, n = int(offs[i]), int(lens[i])
            f.write(b">r%d\n" % (i + 1))
            f.write(seqs[o:o + n].tobytes())
            f.write(b"\n")
