"""Seeding benchmark: reads/s of the batched GPU pipeline vs the plain kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 3] [--reads R] [--ref-len L]

Workload (default): the human-scale configuration the metric is quoted on --
a 3.1 Gbp synthetic reference (41% GC, segmental duplications, diverged
300 bp repeat families up to 45% repeats, 1% N blocks), index with SA ratio 7
built on the GPU, 10M reads of 50/75/100/150/250 bp with 1% substitutions and
0.05% indels, k = 19, SMEM mode.  Data is synthetic and seeded.

One step = one pass of the whole pipeline (search, filters, ordering, SA
walk) over all reads, inputs resident in HBM.  The inputs (1.25 GB of reads)
and the index (3.8 GB) are larger than L2, so no flush is needed between
steps.  `e2e` is the same pass through the C-ABI with host buffers: pinned
host -> device copies of the reads and device -> host copies of every seed and
position inside the timed region.

--impl reference times the reference's seeding semantics on the host cores:
the CPU restatement (oracle/, a "port") with every host thread, on a bounded
sample of the same reads per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "reads/sec SMEM (bit-exact) batched vs plain kernel on 1 GB300; p50/p99 latency"
CACHE = os.environ.get("GPUSEED_BENCH_CACHE", "/tmp/gpuseed_bench_cache")


def nvtx(name):
    """push an NVTX range (name) or pop the current one (None); no-op when
    torch was built without NVTX"""
    import torch
    try:
        if name is None:
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# workload

def workload(cfg, ref_len, n_reads, rank=0, load_gpu_index=True):
    """Reference + index files (built on the GPU, cached per box) + reads of this rank."""
    from gpuseed_gb300 import workloads as W
    spec = W.ref_spec(cfg, ref_len)
    rspec = W.read_spec(cfg, n_reads)
    rspec.seed += 7919 * rank
    tag = f"cfg{cfg}_L{spec.length}"
    d = os.path.join(CACHE, tag)
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "ref")
    t0 = time.time()
    codes, nmask = W.make_reference(spec)
    log(f"[bench] reference {spec.length:,} bp generated in {time.time() - t0:.1f}s")
    idx = None
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import build as gbuild
    gbuild.build()
    t0 = time.time()
    if os.path.exists(prefix + ".sa") and os.path.exists(prefix + ".bwt"):
        if load_gpu_index:
            idx = gs.Index(prefix)
        log(f"[bench] index files from cache, loaded in {time.time() - t0:.1f}s")
    else:
        # each rank writes its own files; the rename publishes them whole
        tmp = f"{prefix}.tmp{rank}.{os.getpid()}"
        idx = gs.build_index(codes, 7, prefix=tmp, load=load_gpu_index)
        for ext in (".bwt", ".sa"):
            os.replace(tmp + ext, prefix + ext)
        log(f"[bench] index built on GPU in {time.time() - t0:.1f}s")
    t0 = time.time()
    seqs, offs, lens = W.make_reads(codes, nmask, rspec)
    log(f"[bench] {lens.size:,} reads ({int(lens.sum()):,} bases) in {time.time() - t0:.1f}s")
    return dict(prefix=prefix, idx=idx, seqs=seqs, offs=offs, lens=lens, k=W.CONFIG_K[cfg],
                smem=W.CONFIG_SMEM[cfg], spec=spec, codes=codes, nmask=nmask)


# --------------------------------------------------------------------------
# clocks (nvidia-smi sampled during the timed region)

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


# --------------------------------------------------------------------------
# distributed helpers (one process per GPU, reads sharded by rank)

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# --------------------------------------------------------------------------
# CPU baseline (oracle port, all host threads, bounded sample)

def cpu_baseline(prefix, seqs, offs, lens, k, smem, table, target_s=12.0, threads=0):
    """The oracle's containment-stopped walk (the CPU port) on all host
    threads over the first reads of the workload, sized to ~target_s seconds.
    Returns the baseline record, the oracle's batch for those reads (the
    checker of the GPU result) and their count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    oidx = pyoracle.Index(prefix)
    threads = threads or len(os.sched_getaffinity(0))
    n_total = lens.size

    def run(n):
        t0 = time.perf_counter()
        b = oidx.seed(seqs, offs[:n], lens[:n], k=k, smem=smem, pruned=True, threads=threads,
                      table=table)
        return time.perf_counter() - t0, b

    n = min(20_000, n_total)
    dt, batch = run(n)
    n2 = int(min(n_total, max(n, n / max(dt, 1e-3) * target_s)))
    if n2 > n:
        del batch
        dt, batch = run(n2)
        n = n2
    rec = {"value": n / dt, "unit": "reads/s", "cores": threads, "kind": "port",
           "sample": f"first {n:,} reads of the workload, oracle containment-stopped walk, "
                     f"{threads} threads, {dt:.1f}s"}
    return rec, batch, n


def parity_check(batch, res, n):
    """reads among the first n whose GPU records (host result `res` of the
    whole batch) differ from the oracle's"""
    import pyoracle
    t0 = time.perf_counter()
    bad = pyoracle.mismatched_reads(batch, res.seeds, res.pos, res.read_seed_off,
                                    res.read_pos_off, cols=(0, 1, 2, 3, 6))
    log(f"[bench] parity: {n:,} reads checked against the oracle, {bad.size} differ "
        f"({time.perf_counter() - t0:.1f}s)")
    return int(bad.size)


# --------------------------------------------------------------------------
# serving: Poisson arrivals of config-5 requests against the resident index

def serving_sweep(idx, codes, nmask, k, smem, peak_reads_s, max_batch_reads=1 << 18, n_slots=12,
                  loads=(0.1, 0.5, 0.9, 1.2), modes=("continuous", "per_request"),
                  seconds=1.5, seed=0x5EED1005):
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    # request sizes: 1..4096 reads, log-uniform; reads 100-250 bp, 1% errors
    pool_spec = W.read_spec(5, 400_000)
    pseqs, poffs, plens = W.make_reads(codes, nmask, pool_spec)
    mean_reads = (4096 - 1) / np.log(4096)
    # load is a fraction of the batched throughput on these reads (one pass
    # over the whole pool, device-resident), not on the headline workload's
    import torch
    ctx = gs.Context(idx)
    d_s = torch.from_numpy(pseqs).cuda()
    d_o = torch.from_numpy(poffs.view(np.int64)).cuda()
    d_l = torch.from_numpy(plens.view(np.int32)).cuda()
    ts = []
    for _ in range(4):
        ctx.seed_device(d_s.data_ptr(), d_o.data_ptr(), d_l.data_ptr(), plens.size, fetch=False,
                        k=k, smem=smem)
        ts.append(ctx.last_timing()[1])
    ctx.close()
    del d_s, d_o, d_l
    peak_reads_s = plens.size / (min(ts[1:]) / 1e3)
    log(f"[bench] serving peak: batched pass over {plens.size:,} request reads at "
        f"{peak_reads_s:,.0f} reads/s")
    out = []
    for mode in modes:
        for load in loads:
            rate = load * peak_reads_s / mean_reads          # requests per second
            n_req = max(20, int(rate * seconds))
            if mode == "per_request":
                # one pass per request cannot keep up beyond low load: a bounded
                # stream still shows its latency and throughput
                n_req = min(n_req, 3000)
            sizes = np.exp(rng.uniform(0, np.log(4096), n_req)).astype(np.int64).clip(1, 4096)
            gaps = rng.exponential(1.0 / rate, n_req)
            starts = rng.integers(0, plens.size - 4096, n_req)
            if mode == "continuous":
                srv = gs.Server(idx, n_slots=n_slots, max_batch_reads=max_batch_reads, k=k, smem=smem)
            else:
                srv = gs.Server(idx, n_slots=1, max_batch_reads=1, k=k, smem=smem)
            # warm-up: the same arrival process for a third of the time, so that
            # the slots' workspaces reach their working size as in a running
            # server; then the measured stream (stats as differences)
            nw = max(10, n_req // 3)
            srv.replay(pseqs, poffs, plens, starts[:nw], sizes[:nw], gaps[:nw] * 1e3)
            st0 = srv.stats()
            lat, wall_ms, sub_ms = srv.replay(pseqs, poffs, plens, starts, sizes, gaps * 1e3)
            st1 = srv.stats()
            srv.stop()
            st = {n: st1[n] - st0[n] for n in ("passes", "submit_us", "merge_us", "seed_us",
                                                 "split_us")}
            out.append({"mode": mode, "load": load, "requests": n_req,
                        "max_batch_reads": max_batch_reads if mode == "continuous" else 1,
                        "peak_reads_s": float(peak_reads_s),
                        "offered_reads_s": float(sizes.sum() / gaps.sum()),
                        "submitted_reads_s": float(sizes.sum() / (sub_ms / 1e3)),
                        "achieved_reads_s": float(sizes.sum() / (wall_ms / 1e3)),
                        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                        "passes": int(st["passes"]),
                        "host_ms": {n: st[n + "_us"] / 1e3 for n in ("submit", "merge", "seed", "split")}})
            log(f"[bench] serving {mode} load {load:.0%}: p50 {out[-1]['p50_ms']:.1f} ms "
                f"p99 {out[-1]['p99_ms']:.1f} ms, {out[-1]['achieved_reads_s']:,.0f} reads/s "
                f"(submitted {out[-1]['submitted_reads_s']:,.0f}), {st['passes']} passes for "
                f"{n_req} requests; submit/merge/seed/split "
                + "/".join(f"{st[n + '_us'] / 1e3:.0f}" for n in ("submit", "merge", "seed", "split"))
                + " ms")
    return out


# --------------------------------------------------------------------------

def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfg = args.config
    w = workload(cfg, args.ref_len, args.reads, load_gpu_index=False)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    oidx = pyoracle.Index(w["prefix"])
    threads = len(os.sched_getaffinity(0))
    t0 = time.time()
    table = oidx.table13(threads)
    log(f"[bench] oracle 13-mer table in {time.time() - t0:.1f}s")
    # size one step's sample to ~args.ref_step_s seconds of CPU work
    lens, offs, seqs = w["lens"], w["offs"], w["seqs"]
    n = min(20_000, lens.size)
    t0 = time.perf_counter()
    oidx.seed(seqs, offs[:n], lens[:n], k=w["k"], smem=w["smem"], pruned=True, threads=threads,
              table=table)
    rate = n / (time.perf_counter() - t0)
    n_step = int(min(lens.size, max(n, rate * args.ref_step_s)))
    times = []
    for s in range(args.warmup + args.steps):
        lo = (s * n_step) % max(1, lens.size - n_step + 1)
        t0 = time.perf_counter()
        oidx.seed(seqs, offs[lo:lo + n_step], lens[lo:lo + n_step], k=w["k"], smem=w["smem"],
                  pruned=True, threads=threads, table=table)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    value = n_step * len(times) / tot
    sample = f"{n_step:,} reads per step (oracle containment-stopped walk, {threads} threads)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "reads/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * tot / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config_dict(args, w, sample_note=sample),
        "cpu_baseline": {"value": value, "unit": "reads/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def config_dict(args, w, sample_note=None):
    spec = w["spec"]
    if w.get("idx") is not None:
        info = w["idx"].info()
        index_gb = (f"{info.device_bytes / 1e9:.1f} GB on the device, "
                    f"text structures {'on' if info.text_min else 'off'}")
    else:
        index_gb = "files in host memory"
    d = {"workload": f"config {args.config}: {spec.length / 1e9:.2f} Gbp synthetic reference, "
                     f"{w['lens'].size:,} reads {'SMEM' if w['smem'] else 'MEM'} k={w['k']}",
         "ref_bp": int(spec.length), "reads": int(w["lens"].size), "bases": int(w["lens"].sum()),
         "k": w["k"], "mode": "smem" if w["smem"] else "mem", "sa_intv": 7,
         "l2": f"inputs larger than L2 (reads {w['lens'].sum() / 1e9:.2f} GB, index "
               f"{index_gb}); no flush"}
    if sample_note:
        d["sample"] = sample_note
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--reads", type=int, default=0)
    ap.add_argument("--ref-len", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--ref-step-s", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-text", action="store_true")
    ap.add_argument("--no-text-index", action="store_true",
                    help="seed without the full-SA / text structures")
    ap.add_argument("--no-sampled-sa", action="store_true",
                    help="skip the second timing without the text structures")
    ap.add_argument("--serve-slots", type=int, default=12)
    ap.add_argument("--serve-batch", type=int, default=1 << 18,
                    help="serving: most reads merged into one pass")
    ap.add_argument("--retune", action="store_true")
    ap.add_argument("--kernels-only", action="store_true",
                    help="profiling driver: default launch knobs, W + K uncaptured batched "
                         "passes (the K inside the NVTX range timed_batched), nothing else")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import gpuseed_gb300 as gs
    from gpuseed_gb300 import build as gbuild
    gbuild.build()
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = dist_init(ws, "nccl")
    dev = torch.device("cuda", local)

    w = workload(args.config, args.ref_len, args.reads, rank=rank)
    idx = w["idx"]
    if not args.no_text_index:
        t0 = time.time()
        idx.set_text(4)
        log(f"[bench] text structures (full SA, text, ISA samples) built in {time.time() - t0:.2f}s")
    seqs, offs, lens = w["seqs"], w["offs"], w["lens"]
    n_reads = int(lens.size)
    k, smem = w["k"], w["smem"]
    ctx = gs.Context(idx)
    st = torch.cuda.ExternalStream(ctx.stream())

    d_seqs = torch.from_numpy(seqs).to(dev)
    d_offs = torch.from_numpy(offs.view(np.int64)).to(dev)
    d_lens = torch.from_numpy(lens.view(np.int32)).to(dev)
    torch.cuda.synchronize()

    if args.kernels_only:
        # one kernel launch per pass stage, visible to a profiler by name
        for _ in range(args.warmup):
            ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                            fetch=False, k=k, smem=smem)
        torch.cuda.synchronize()
        nvtx("timed_batched")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                            fetch=False, k=k, smem=smem)
        e1.record(st)
        torch.cuda.synchronize()
        nvtx(None)
        walkers, text_jobs = ctx.last_walkers(), ctx.last_text_jobs()
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=False, k=k, smem=smem, count_work=True)
        torch.cuda.synchronize()
        executed = ctx.last_work()
        walk_counts = ctx.last_walk_counts()
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=False, k=k, smem=smem, count_work=True, kernel=gs.KERNEL_PLAIN)
        torch.cuda.synchronize()
        print(json.dumps({"kernels_only": True, "reads": n_reads, "ref_bp": int(w["spec"].length),
                          "kmer_start_len": idx.info().kmer_len,
                          "device_bytes_index": idx.info().device_bytes,
                          "ms_per_step": e0.elapsed_time(e1) / args.steps,
                          "work_executed_batched": executed, "work_canonical_own": ctx.last_work(),
                          "walkers": walkers, "text_jobs": text_jobs,
                          "walk_counts": walk_counts}),
              flush=True)
        return

    # autotuned launch knobs of the batched search (cached per GPU and workload)
    tag = f"{torch.cuda.get_device_name(local)}|cfg{args.config}|{w['spec'].length}|{n_reads}|{k}|{smem}"
    tune_path = os.path.join(CACHE, "autotune.json")
    cache = {}
    try:
        cache = json.load(open(tune_path))
    except Exception:
        pass
    if tag in cache and not args.retune:
        knobs = cache[tag]["knobs"]
    else:
        t0 = time.time()
        knobs, tms = ctx.autotune(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                                  sample=min(n_reads, 1 << 20), k=k, smem=smem)
        cache[tag] = {"knobs": knobs, "sample_search_ms": tms}
        try:
            tmp = f"{tune_path}.{os.getpid()}"
            with open(tmp, "w") as f:
                json.dump(cache, f, indent=1)
            os.replace(tmp, tune_path)
        except OSError:
            pass
        log(f"[bench] autotuned {knobs} ({tms:.1f} ms on the sample) in {time.time() - t0:.1f}s")

    def step(kernel, count=False, graph=False):
        kn = knobs if kernel == gs.KERNEL_BATCHED else {}
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=False, k=k, smem=smem, kernel=kernel, count_work=count, graph=graph,
                        **kn)

    def timed(kernel, steps, warmup, clocks=None, graph=False):
        for _ in range(warmup):
            step(kernel, graph=graph)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        search_ms = []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cm = clocks if clocks is not None else _Null()
        # NVTX range around the timed steps, so that a profiler can be limited
        # to them (ncu --nvtx --nvtx-include timed_batched/)
        rng = "timed_batched" if kernel == gs.KERNEL_BATCHED else "timed_plain"
        with cm:
            torch.cuda.synchronize()
            nvtx(rng)
            e0.record(st)
            for _ in range(steps):
                step(kernel, graph=graph)
                search_ms.append(ctx.last_timing()[0])
            e1.record(st)
            torch.cuda.synchronize()
            nvtx(None)
        if dist is not None:
            dist.barrier()
        return e0.elapsed_time(e1), search_ms

    # batched (the headline): the pass is captured once and replayed
    clocks = Clocks(local)
    ms, _ = timed(gs.KERNEL_BATCHED, args.steps, args.warmup, clocks, graph=True)
    # search-kernel time of the same pass, uncaptured (CUDA events around the
    # search launches on the context stream)
    search_ms = []
    for _ in range(3):
        step(gs.KERNEL_BATCHED)
        search_ms.append(ctx.last_timing()[0])
    search_ms = search_ms[1:]
    walkers, walker_cap = ctx.last_walkers()
    text_jobs, text_cap = ctx.last_text_jobs()
    # the lockstep form of the batched search, same pipeline otherwise
    lock_ms = []
    for _ in range(3):
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=False, k=k, smem=smem, kernel=gs.KERNEL_LOCKSTEP, queue_chunk=16,
                        handoff_lanes=2, handoff_steps=6)
        lock_ms.append(ctx.last_timing()[0])
    lock_ms = lock_ms[1:]
    log(f"[bench] lockstep search {statistics.mean(lock_ms):.1f} ms; batched walkers {walkers:,} "
        f"(buffer {walker_cap:,})")
    ms = max_over_ranks(dist, ms, dev)
    total_reads = sum_over_ranks(dist, n_reads * args.steps, dev)
    value = total_reads / (ms / 1e3)
    n_seeds, n_pos = ctx.device_counts()
    log(f"[bench] batched: {ms / args.steps:.1f} ms/step, {value:,.0f} reads/s, "
        f"search {statistics.mean(search_ms):.1f} ms, seeds {n_seeds:,} positions {n_pos:,}")

    # plain one-read-per-thread kernel, same pipeline otherwise
    pms, psearch = timed(gs.KERNEL_PLAIN, args.plain_steps, 1)
    pms = max_over_ranks(dist, pms, dev)
    plain_value = sum_over_ranks(dist, n_reads * args.plain_steps, dev) / (pms / 1e3)
    log(f"[bench] plain: {pms / args.plain_steps:.1f} ms/step, {plain_value:,.0f} reads/s, "
        f"search {statistics.mean(psearch):.1f} ms")

    # work the search executes with its own start table, counted on the whole
    # workload: the plain kernel's walk is the canonical containment-stopped
    # walk from that table; the batched search's own lookups beside it
    step(gs.KERNEL_PLAIN, count=True)
    torch.cuda.synchronize()
    work = ctx.last_work()
    step(gs.KERNEL_BATCHED, count=True)
    torch.cuda.synchronize()
    executed = ctx.last_work()
    walk_counts = ctx.last_walk_counts()
    own_bytes = 32 * (work["n_kmer"] + work["n_occ_blocks"])
    mean_search_s = statistics.mean(search_ms) / 1e3
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    traffic = None
    try:
        # "dram_bytes_per_read <float>" line of the committed ncu summary
        for ln in open(os.path.join(ROOT, "profiles", "search_traffic.txt")):
            if ln.startswith("dram_bytes_per_read "):
                traffic = float(ln.split()[1]) * n_reads
    except Exception:
        pass
    # random 32-byte gather roofline on a 16 GB buffer
    import ctypes as C
    L = gs.lib()
    L.gs_probe_random_gather.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_uint64,
                                         C.POINTER(C.c_double)]
    g32 = C.c_double()
    gs.check(L.gs_probe_random_gather(local, 16 << 30, 32, 1 << 30, C.byref(g32)))

    # e2e through the C-ABI with pinned host buffers
    h_seqs = torch.from_numpy(seqs).pin_memory()
    h_offs = torch.from_numpy(offs.view(np.int64)).pin_memory()
    h_lens = torch.from_numpy(lens.view(np.int32)).pin_memory()
    hs = h_seqs.numpy().view(np.uint8)
    ho = h_offs.numpy().view(np.uint64)
    hl = h_lens.numpy().view(np.uint32)
    p = ctx.params(k=k, smem=smem, **knobs)
    import ctypes as C2
    for _ in range(2):
        gs.check(L.gs_seed(ctx.h, C2.c_void_p(hs.ctypes.data), C2.c_void_p(ho.ctypes.data),
                           C2.c_void_p(hl.ctypes.data), n_reads, C2.byref(p)))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e2e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gs.check(L.gs_seed(ctx.h, C2.c_void_p(hs.ctypes.data), C2.c_void_p(ho.ctypes.data),
                           C2.c_void_p(hl.ctypes.data), n_reads, C2.byref(p)))
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(dist, e2e_s, dev)
    e2e_value = sum_over_ranks(dist, n_reads * e2e_steps, dev) / e2e_s
    res = ctx.result()
    h2d = int(seqs.nbytes + offs.nbytes + lens.nbytes)
    d2h = int(res.seeds.nbytes + res.pos.nbytes + res.read_seed_off.nbytes + res.read_pos_off.nbytes)
    log(f"[bench] e2e: {e2e_value:,.0f} reads/s")

    # the -o records of this result: GPU formatting vs the host writer, to /dev/null
    text = None
    if not args.no_text:
        # a device-resident pass leaves the result on both sides (gs_seed in
        # chunks keeps the host result only)
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=True, k=k, smem=smem, **knobs)
        fd = os.open(os.devnull, os.O_WRONLY)
        try:
            ctx.text_device(1, smem)
            t0 = time.perf_counter()
            _, text_bytes = ctx.text_device(1, smem)
            t_fmt = time.perf_counter() - t0
            t0 = time.perf_counter()
            ctx.write_text(fd, 1, smem)
            t_gpu = time.perf_counter() - t0
            t0 = time.perf_counter()
            ctx.write_text(fd, 1, smem, host=True)
            t_host = time.perf_counter() - t0
        finally:
            os.close(fd)
        text = {"bytes": text_bytes, "gpu_format_ms": t_fmt * 1e3,
                "gpu_write_ms": t_gpu * 1e3, "host_write_ms": t_host * 1e3,
                "sink": "/dev/null"}
        log(f"[bench] -o text {text_bytes / 1e9:.2f} GB: GPU format {t_fmt * 1e3:.1f} ms, "
            f"GPU format + copy-out + write {t_gpu * 1e3:.1f} ms, host writer {t_host * 1e3:.1f} ms")

    latency = None
    if rank == 0 and not args.no_serving:
        latency = serving_sweep(idx, w["codes"], w["nmask"], k, smem, value / ws,
                                max_batch_reads=args.serve_batch, n_slots=args.serve_slots)

    def device_pass_result():
        """host copy of one batched pass over the whole workload"""
        ctx.seed_device(d_seqs.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), n_reads,
                        fetch=True, k=k, smem=smem, **knobs)
        return ctx.result()

    # CPU baseline: the oracle on the first reads of the workload; its output
    # is also the checker of the GPU's records for those reads, and its work
    # counters give the canonical walk's lookups from the 13-mer table
    cpu, parity, canon = None, None, None
    oracle_batch, n_checked = None, 0
    if rank == 0 and not args.no_cpu_baseline:
        table = idx.kmer_table()
        cpu, oracle_batch, n_checked = cpu_baseline(w["prefix"], seqs, offs, lens, k, smem, table)
        del table
        log(f"[bench] cpu baseline: {cpu['value']:,.0f} reads/s on {cpu['cores']} threads")
        parity = {"reads_checked": n_checked,
                  "mismatches": parity_check(oracle_batch, device_pass_result(), n_checked),
                  "checker": "oracle containment-stopped walk, exact seeds (x, y, l, u, count) "
                             "and positions of the first reads of the workload"}
        # candidates of the sample and of the whole workload scale the counts
        cand = np.maximum(lens.astype(np.int64) - (k - 1), 0)
        scale = float(cand.sum()) / max(1.0, float(cand[:n_checked].sum()))
        ow = oracle_batch.work
        canon = {"n_kmer": ow["n_kmer"] * scale, "n_occ_blocks": ow["n_occ_blocks"] * scale,
                 "sample_reads": n_checked, "scale": scale}

    # roofline of the search pass.  achieved = the canonical walk's bytes from
    # the 13-mer table (32 B per table sector and per occurrence block, the
    # implementation-independent count; from the oracle's sample, scaled by
    # candidates) / the search kernels' CUDA-event time; the same from the
    # start table this index uses (the plain kernel's count over the whole
    # workload) beside it
    canon_bytes = 32 * (canon["n_kmer"] + canon["n_occ_blocks"]) if canon else None
    own_achieved = own_bytes / mean_search_s / 1e9
    achieved = canon_bytes / mean_search_s / 1e9 if canon_bytes else own_achieved
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_src} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": "gs_search_start + gs_search_walk + gs_search_text + gs_search_leftover (one search pass)",
                "algorithmic_bytes_per_launch": canon_bytes if canon_bytes else own_bytes,
                "algorithmic_count": ("canonical containment-stopped walk from the 13-mer table "
                                      "(oracle sample, scaled by candidates)") if canon_bytes else
                                     f"canonical walk from the {idx.info().kmer_len}-mer start table",
                "own_start_table": {"kmer_len": idx.info().kmer_len, "bytes": own_bytes,
                                    "achieved": own_achieved, "frac": own_achieved / peak},
                "random_32B_gather_gbs": g32.value,
                "frac_of_random_32B": achieved / g32.value if g32.value else None}
    log(f"[bench] search {achieved:.0f} GB/s algorithmic = {achieved / peak:.3f} of {peak:.0f} GB/s "
        f"({own_achieved:.0f} GB/s from the {idx.info().kmer_len}-mer start table); "
        f"random 32B gather {g32.value:.0f} GB/s")

    # the headline's index state, before the sampled-SA timing frees the
    # text structures
    cfg_d = config_dict(args, w)
    text_on = idx.info().text_min > 0

    # the sampled-SA walk (no text structures): locate by LF steps to a
    # sampled row, no text mode; same graph-replayed pass, timed the same way
    sampled = None
    if not args.no_text_index and not args.no_sampled_sa:
        idx.set_text(0)
        sms, _ = timed(gs.KERNEL_BATCHED, args.steps, args.warmup, None, graph=True)
        sms = max_over_ranks(dist, sms, dev)
        ssearch = []
        for _ in range(3):
            step(gs.KERNEL_BATCHED)
            ssearch.append(ctx.last_timing()[0])
        sampled = {"value": sum_over_ranks(dist, n_reads * args.steps, dev) / (sms / 1e3),
                   "unit": "reads/s",
                   "ms_per_step": sms / args.steps, "search_ms": statistics.mean(ssearch[1:]),
                   "index": "no text structures: locate walks LF steps to a sampled SA row"}
        if oracle_batch is not None:
            sampled["parity"] = {"reads_checked": n_checked,
                                 "mismatches": parity_check(oracle_batch, device_pass_result(),
                                                            n_checked)}
        log(f"[bench] sampled-SA walk: {sms / args.steps:.1f} ms/step, "
            f"{sampled['value']:,.0f} reads/s, search {sampled['search_ms']:.1f} ms")
    del oracle_batch

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": cfg_d,
            "plain": {"value": plain_value, "unit": "reads/s", "ms_per_step": pms / args.plain_steps,
                      "search_ms": statistics.mean(psearch)},
            "batched_over_plain": value / plain_value,
            "search_ms": statistics.mean(search_ms),
            "seeds_per_step": n_seeds, "positions_per_step": n_pos,
            "lockstep": {"search_ms": statistics.mean(lock_ms), "knobs": {"queue_chunk": 16,
                         "handoff_lanes": 2, "handoff_steps": 6}},
            "walkers": {"handed_to_walk_pass": walkers, "buffer": walker_cap,
                        "handed_to_text_pass": text_jobs, "text_buffer": text_cap},
            "text": text,
            "work": work,
            "work_canonical_13mer": canon,
            "walk_counts": walk_counts,
            "work_executed_batched": {"n_kmer": executed["n_kmer"],
                                      "n_occ_blocks": executed["n_occ_blocks"],
                                      "over_canonical": (executed["n_kmer"] + executed["n_occ_blocks"]) /
                                      max(1, work["n_kmer"] + work["n_occ_blocks"])},
            "e2e": {"value": e2e_value, "unit": "reads/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            # prepare, start, walk, (text), leftover, finalize count + emit, expand, locate
            "gpu_launches": (9 if text_on else 8) * args.steps,
            "graph": "each timed step replays one CUDA graph of the whole pass",
            "clocks": clocks.summary(),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "parity": parity,
            "sampled_sa": sampled,
            "latency": latency,
        }
        line["config"]["autotuned"] = knobs
        line["config"]["kmer_start_len"] = idx.info().kmer_len
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


if __name__ == "__main__":
    main()
