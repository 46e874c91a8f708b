#!/usr/bin/env python
"""Throughput benchmark of the exhaustive epistasis search on GB300.

One step = one complete scan (every combination of the workload, top-N
selection and FP64 re-score included) over the seeded synthetic data set of
the named workload; the default is order 3 over 2 000 SNPs x 8 000 samples
(4 000 cases / 4 000 controls), top-100.

Output: one JSON line (rank 0).  ``value`` is combinations x samples per second
with the data set resident in HBM; ``e2e`` is the same metric through the
public host-buffer call (``fiu_search``: pinned host data set -> device ->
search -> results to host, all inside the timed region).  ``roofline`` is the
roofline of the dominant (counting) kernel: for the tcgen05 kernel the tensor
bound (2^k multiply-adds per combination and sample, e4m3 peak = 2 x the
measured dense bf16 rate); for the CUDA-core kernels the HBM bound, with
``int_roofline`` their integer (AND+POPC) roofline against a peak measured
live on this GPU.
``cpu_baseline`` times the CPU oracle (a C restatement of the reference's
scalar search) on a bounded prefix sample of the same workload on the host
cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload order3_2000x8000]

With --gpus N > 1 (launched by torch.distributed.run), rank r searches shard r
of N of the whole search (equal ranges of the serving kernel's work units, so
every GPU keeps the whole-data-set kernels; no data-path collective), rank 0
gathers the top-N lists; value = all ranks' work / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k=3 combos×samples/s, batched/served vs plain, 1 GB300; scan p50/p99 latency"
UNIT = "combos*samples/s"


# ----------------------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def combos_of(n, k, step=1, offset=0):
    """Combinations owned by Distribution(n, k-1, step, offset): sum over owned prefixes of (n-1-last)."""
    if step == 1 and offset == 0:
        return math.comb(n, k)
    from oracle.oracle import Oracle  # exact count from the enumeration (small samples only)
    p = Oracle().prefixes(n, k - 1, step, offset)
    return int(np.sum(n - 1 - p[:, -1])) if len(p) else 0


def cpu_sample(spec, ds, seconds=10.0, threads=None):
    """The CPU oracle (C restatement of the reference's scalar search) on a
    uniform sample of the workload's prefixes, sized to about `seconds` of work."""
    from oracle.oracle import Oracle
    o = Oracle()
    threads = threads or os.cpu_count() or 1
    n_pref = math.comb(spec.snps, spec.order - 1)
    step = max(1, n_pref // (threads * 4))
    while True:
        t0 = time.perf_counter()
        _, _, _, done = o.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words,
                                 spec.order, spec.outputs, threads=threads, mi_mode=0, dist=(spec.snps, step, 0))
        dt = time.perf_counter() - t0
        if dt >= 0.5 or step == 1:
            break
        step = max(1, step // 8)
    # rescale the sample to ~`seconds`
    if dt < seconds and step > 1:
        step = max(1, int(step * dt / seconds))
        t0 = time.perf_counter()
        _, _, _, done = o.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words,
                                 spec.order, spec.outputs, threads=threads, mi_mode=0, dist=(spec.snps, step, 0))
        dt = time.perf_counter() - t0
    rate = done * spec.samples / dt
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "every %d-th (order-%d)-prefix of the workload (%d combinations, %.1f s)" %
                      (step, spec.order - 1, done, dt)}


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, spec):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from fiuncho_gb300 import Dataset, synth
    from oracle.oracle import Oracle
    geno, is_case, _ = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    o = Oracle()
    threads = os.cpu_count() or 1
    n_pref = math.comb(spec.snps, spec.order - 1)
    step = max(1, n_pref // (threads * 64))  # ~1/64 of the prefixes per thread-round, a few seconds
    times, done_all = [], 0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, _, done = o.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, spec.order,
                                 spec.outputs, threads=threads, mi_mode=0, dist=(spec.snps, step, it % step))
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            done_all += done
    total = sum(times)
    value = done_all * spec.samples / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": args.workload, "snps": spec.snps, "cases": spec.cases, "ctrls": spec.ctrls,
                       "order": spec.order, "outputs": spec.outputs,
                       "step_sample": "every %d-th prefix (offset rotates per step)" % step},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "every %d-th (order-%d)-prefix per step" % (step, spec.order - 1)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GB300 arm
def run_gpu(args, spec):
    ws, rank, local = dist_env()
    import ctypes as C

    import torch

    from fiuncho_gb300 import Context, Dataset, Distribution, GpuSearch, Resident, synth, _lib

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    geno, is_case, planted = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    gs = GpuSearch(local, kernel=args.kernel)
    ctx = gs.ctx
    lib = ctx.lib
    res = Resident(ctx, ds)
    # rank r of N searches shard r of the whole search's work units (the same
    # whole-data-set kernels on every GPU); N = 1 is the whole search
    total_combos = math.comb(ds.snps, spec.order)

    def search():
        return gs.run_shard(res, spec.order, rank, ws, spec.outputs)

    if args.profile_layer:
        # profiling case: two searches of one Distribution layer (the second one timed), no bench line
        step, off = (int(x) for x in args.profile_layer.split(","))
        layer = Distribution(ds.snps, spec.order - 1, step, off)
        gs.run(res, spec.order, layer, spec.outputs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = gs.run(res, spec.order, layer, spec.outputs)
        print(json.dumps({"profile_layer": [step, off], "workload": args.workload, "ms": 1e3 * (time.perf_counter() - t0),
                          "top1": list(out[0].combination) if out else None}))
        return
    stream = torch.cuda.ExternalStream(lib.fiu_stream(ctx.h), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 512 MB > L2 (129 MB)

    peak_rate = C.c_double(0)
    ctx.check(lib.fiu_probe_popc_rate(ctx.h, C.byref(peak_rate)))

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        out = search()
    # ---- timed region: resident data set, one event pair per step on the library's stream
    ctx.check(lib.fiu_set_kernel_timing(ctx.h, 1))
    launches0 = ctx.launches
    step_ms = []
    with ClockSampler(local) as clocks:
        barrier()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = search()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        barrier()
    launches = ctx.launches - launches0
    kms, klaunch, kcombos = C.c_double(0), C.c_uint64(0), C.c_uint64(0)
    ctx.check(lib.fiu_kernel_timing(ctx.h, C.byref(kms), C.byref(klaunch), C.byref(kcombos)))
    ctx.check(lib.fiu_set_kernel_timing(ctx.h, 0))
    my_time = sum(step_ms) / 1e3
    if ws > 1:
        t = torch.tensor([my_time], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        my_time = float(t.item())
        from fiuncho_gb300 import MPIEngine
        out = MPIEngine().gather(out, spec.outputs)
    value = total_combos * spec.samples * args.steps / my_time

    # ---- end to end through the public host-buffer call (pinned host data set)
    pinned = torch.empty(ds.data.size, dtype=torch.int64, pin_memory=True)
    pinned.numpy().view(np.uint64)[:] = ds.data
    hds = _lib.Dataset_t(C.cast(C.c_void_p(pinned.data_ptr()), C.POINTER(C.c_uint64)), ds.snps, ds.cases, ds.ctrls,
                         ds.cases_words, ds.ctrls_words)
    comb = np.zeros(spec.outputs * spec.order, np.int32)
    vals = np.zeros(spec.outputs, np.float32)
    cnt = C.c_uint(0)

    def e2e_call():
        ctx.check(lib.fiu_search_shard(ctx.h, C.byref(hds), spec.order, rank, ws, spec.outputs,
                                       _lib.ptr(comb, C.c_int32), _lib.ptr(vals, C.c_float), C.byref(cnt)))

    e2e_call()
    e2e_t = []
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_call()
        e2e_t.append(time.perf_counter() - t0)
    barrier()
    e2e_time = sum(e2e_t)
    if ws > 1:
        t = torch.tensor([e2e_time], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_time = float(t.item())
    e2e_value = total_combos * spec.samples * args.steps / e2e_time

    if rank != 0:
        return
    # ---- roofline of the dominant (counting) kernel
    k = spec.order
    kernel_id, kernel_tp = gs.last_tile()
    ops_per_combo = 3 ** k * (math.ceil(spec.cases / 32) + math.ceil(spec.ctrls / 32))
    avg_launch_s = (kms.value / 1e3) / max(1, klaunch.value)
    ops_per_launch = kcombos.value * ops_per_combo / max(1, klaunch.value)
    int_achieved = ops_per_launch / avg_launch_s if avg_launch_s > 0 else 0.0
    ds_bytes = ds.data.size * 8
    hbm_bytes_per_launch = ds_bytes / max(1, klaunch.value / args.steps)
    hbm_achieved = hbm_bytes_per_launch / avg_launch_s / 1e9 if avg_launch_s > 0 else 0.0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(args.workload)
    except (OSError, ValueError):
        pass
    if kernel_id == _lib.KERNEL_TENSOR:
        # 2^k core cells per combination, each a dot product over the samples of its class:
        # 2^k multiply-adds (2 * 2^k flops) per combination and sample, e4m3 operands.
        flops_per_launch = kcombos.value * 2 * 2 ** k * spec.samples / max(1, klaunch.value)
        tc_achieved = flops_per_launch / avg_launch_s / 1e12 if avg_launch_s > 0 else 0.0
        tc_peak = 2.0 * peaks.get("bf16_tflops", 1900.0)
        roofline = {"bound": "tensor", "achieved": tc_achieved, "peak": tc_peak, "unit": "TFLOP/s",
                    "frac": tc_achieved / tc_peak, "traffic": traffic,
                    "flops_per_combination_sample": 2 * 2 ** k,
                    "peak_source": "2 x measured dense bf16 (%s; e4m3 dense rate = 2 x bf16), of measured"
                                   % ("MEASURED_PEAKS.json" if "bf16_tflops" in peaks else "fallback 1.9 PF"),
                    "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                            "frac": hbm_achieved / hbm_peak}}
    else:
        roofline = {"bound": "hbm", "achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": hbm_achieved / hbm_peak, "traffic": traffic,
                    "note": "algorithmic bytes = the data set read once per scan; the kernel is integer-pipe "
                            "bound (int_roofline)"}
    top = out[0] if out else None
    planted_rank = planted_ranks(gs, res, ds, spec, planted) if ws == 1 else None
    cpu = cpu_sample(spec, ds, seconds=args.cpu_seconds) if args.cpu_seconds > 0 and ws == 1 else None
    batch = None if (args.no_batch or ws > 1) else run_batch_and_serve(args, gs, ctx)
    ingest_t = ingest_timing(ctx, os.cpu_count() or 1) if (not args.no_ingest and ws == 1) else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * my_time / args.steps, "step_ms": [round(x, 3) for x in step_ms],
        "higher_is_better": True, "scaling": "strong",  # the one scan's work units split over the ranks
        "vs_baseline": None, "dtype": "e4m3", "data": "synthetic",
        "arithmetic": "one-hot data: e4m3 0/1 operands on the tensor cores with FP32 accumulation (exact integer "
                      "counts below 2^24), derived cells in int32, MI keys in int64 fixed point, the kept candidates "
                      "re-scored in FP64; other data: uint64 AND + POPC",
        "config": {"workload": args.workload, "snps": spec.snps, "cases": spec.cases, "ctrls": spec.ctrls,
                   "order": spec.order, "outputs": spec.outputs, "combinations": total_combos,
                   "parallelism": "work-unit shards over %d rank(s)" % ws,
                   "l2": "flushed between steps (512 MB write); data set %.1f MB is L2-resident by design"
                         % (ds_bytes / 1e6),
                   "top1": (top.combination if top else None), "planted": [list(p) for p in planted],
                   "planted_rank": planted_rank},
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ds_bytes,
                "d2h_bytes_per_step": spec.outputs * (4 * spec.order + 4) + 8 * 2},
        "roofline": roofline,
        "int_roofline": {"bound": "int", "achieved": int_achieved / 1e12, "peak": peak_rate.value / 1e12,
                         "unit": "T word-ops/s", "frac": int_achieved / peak_rate.value if peak_rate.value else None,
                         "work": "3^k*(ceil(cases/32)+ceil(ctrls/32)) 32-bit AND+POPC per combination",
                         "peak_source": "fiu_probe_popc_rate on this GPU (AND+POPC+ADD microbenchmark)"},
        "kernel": {"requested": args.kernel or "auto", "ran": {1: "full", 2: "elided_popc", 3: "elided_hs",
                                                               4: "tensor"}.get(kernel_id, kernel_id),
                   "threads_per_prefix": kernel_tp, "one_hot": res.one_hot, "count_ms_total": kms.value,
                   "count_launches": klaunch.value, "combinations": kcombos.value},
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "batched": batch,
        "ingest": ingest_t,
    }
    print(json.dumps(line), flush=True)


def ingest_timing(ctx, threads):
    """Ingest of the 40 000 SNPs x 8 000 / 8 000 samples workload from PLINK text
    files (.tped 2.6 GB + .tfam, written first, outside the timing): the
    library's threaded parser to genotype codes, then packing on the device."""
    import tempfile

    from fiuncho_gb300 import ingest, synth
    spec = synth.WORKLOADS["order2_40000x16000"]
    g, c, _ = synth.simulate(spec)
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        tped, tfam = synth.write_tped(os.path.join(d, "x"), g, c)
        write_s = time.perf_counter() - t0
        del g, c
        size = os.path.getsize(tped)
        t0 = time.perf_counter()
        geno, is_case = ingest.read_genotypes([tped, tfam], threads=threads, ctx=ctx)
        parse_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    res = ingest.upload_genotypes(ctx, geno, is_case)
    pack_s = time.perf_counter() - t0
    res.free()
    return {"workload": "order2_40000x16000 as .tped/.tfam", "file_bytes": size, "threads": threads,
            "parse_s": parse_s, "parse_gb_per_s": size / parse_s / 1e9,
            "device_pack_and_prepare_s": pack_s, "write_s_untimed": write_s}


def planted_ranks(gs, res, ds, spec, planted):
    """Rank of each planted interaction (of the scan's order) among all combinations by
    exact MI: its FP64 MI from its tables, against the search's top FIU_MAX_OUTPUTS
    (outside the timed region)."""
    from fiuncho_gb300 import Distribution, _lib
    mine = [p for p in planted if len(p) == spec.order]
    if not mine:
        return None
    _, v64 = gs.run(res, spec.order, Distribution(ds.snps, spec.order - 1), _lib.FIU_MAX_OUTPUTS, with_fp64=True)
    out = []
    for p in mine:
        cc, tt = gs.tables(res, spec.order, np.array([p], np.int32))
        _, mi = gs.mi(cc, tt, ds.cases, ds.ctrls, mode=1)
        mi = float(mi[0])
        rank = int(np.sum(v64 > mi)) + 1 if len(v64) and mi >= v64[-1] else None
        out.append({"combination": list(p), "mi": mi, "rank": rank,
                    "rank_note": None if rank else "below the top %d (MI of the %d-th: %.6g)"
                    % (len(v64), len(v64), float(v64[-1]) if len(v64) else float("nan"))})
    return out


def run_batch_and_serve(args, gs, ctx):
    """Batched vs plain on the uneven 64-scan batch, then a served Poisson stream.

    The batch is the configuration as stated (synth.batch_specs(): SNPs
    log-uniform in [500, 20 000], order-4 scans capped at 400 SNPs, samples
    log-uniform in [1 000, 32 000], case fraction U(0.3, 0.7), order U{2,3,4}),
    with each scan's data set at full size.  The whole batch is ~1.2e16
    combinations x samples (~90 s per pass, 64 % of it one scan), so every scan
    is searched over a fixed leading range of its combinations: shard 0 of N_i
    of its work units, N_i the smallest with at most `--batch-cap`
    combinations x samples per shard.  Both arms run exactly those shards;
    the combinations of each shard are counted by the library.  Timed passes:
    `--batch-passes` per arm (alternating), median reported.

    The served stream draws full-size scans (no truncation) from the same 64
    at Poisson(`--serve-rate`) for `--serve-seconds` against a 120 GB device
    budget, admitted and run in `--serve-policy` order (shortest-first by
    default: the offered load is far above the device's throughput); at the
    end of the arrival window the backlog is recorded and the server is
    destroyed (scans still running are cancelled)."""
    import ctypes as C
    import random

    import torch

    from fiuncho_gb300 import Dataset, Distribution, Resident, Server, synth
    lib = ctx.lib
    specs = synth.batch_specs()
    t0 = time.perf_counter()
    data = []
    for sp in specs:
        g, c, _ = synth.simulate(sp)
        data.append(Dataset.from_genotypes(g, c))
        del g
    gen_s = time.perf_counter() - t0
    full_work = sum(sp.combos() * sp.samples for sp in specs)
    t0 = time.perf_counter()
    res = [Resident(ctx, ds) for ds in data]
    shards = [max(1, math.ceil(sp.combos() * sp.samples / args.batch_cap)) for sp in specs]
    reqs = [(r, sp.order, Distribution(sp.snps, sp.order - 1), sp.outputs, 0, n)
            for r, sp, n in zip(res, specs, shards)]

    def plain():
        return [gs.run_shard(r, o, sh, n, k, with_fp64=True) for r, o, _, k, sh, n in reqs]

    def batched():
        return gs.run_batch(reqs, use_graph=True)

    # first pass of the plain loop: builds each data set's device tables, and counts the
    # combinations of each shard (the library's counter of evaluated combinations)
    combos = []
    for r, o, _, k, sh, n in reqs:
        ctx.check(lib.fiu_set_kernel_timing(ctx.h, 1))
        gs.run_shard(r, o, sh, n, k)
        cnt = C.c_uint64(0)
        ctx.check(lib.fiu_kernel_timing(ctx.h, None, None, C.byref(cnt)))
        combos.append(int(cnt.value))
    ctx.check(lib.fiu_set_kernel_timing(ctx.h, 0))
    prep_s = time.perf_counter() - t0
    work = sum(c * sp.samples for c, sp in zip(combos, specs))
    a, b = plain(), batched()
    same = all([x.combination for x in p[0]] == [x.combination for x in q[0]] and np.array_equal(p[1], q[1])
               for p, q in zip(a, b))
    launches0 = ctx.launches
    t_plain, t_batch = [], []
    for _ in range(args.batch_passes):
        torch.cuda.synchronize()
        t = time.perf_counter()
        plain()
        t_plain.append(time.perf_counter() - t)
        t = time.perf_counter()
        batched()
        t_batch.append(time.perf_counter() - t)
    batch_launches = ctx.launches - launches0
    mp, mb = statistics.median(t_plain), statistics.median(t_batch)
    out = {"workload": "64 uneven scans as configured (synth.batch_specs): SNPs log-uniform [500, 20000], order-4 "
                       "capped at 400, samples log-uniform [1000, 32000], case fraction U(0.3, 0.7), order U{2,3,4}, "
                       "top-50 each; full-size data sets, each scan searched over shard 0 of N_i of its work units "
                       "(<= %.0e combinations x samples per scan)" % args.batch_cap,
           "combos_samples": work, "combos_samples_full_batch": full_work, "scans_truncated": sum(n > 1 for n in shards),
           "plain_s": t_plain, "batched_s": t_batch, "plain_median_s": mp, "batched_median_s": mb,
           "plain": work / mp, "batched": work / mb, "speedup": mp / mb, "passes": args.batch_passes,
           "identical_results": bool(same), "graph": True, "data_gen_s": gen_s, "device_prep_s": prep_s,
           "gpu_launches_timed": batch_launches, "unit": UNIT}
    for r in res:
        r.free()
    del res
    torch.cuda.empty_cache()
    # ---- served stream: full-size scans drawn from the same 64, Poisson arrivals
    rng = random.Random(7)
    rate, duration = args.serve_rate, args.serve_seconds
    arrivals, tnow = [], 0.0
    while True:
        tnow += rng.expovariate(rate)
        if tnow >= duration:
            break
        arrivals.append((tnow, rng.randrange(len(data))))
    policy = Server.SHORTEST_FIRST if args.serve_policy == "shortest" else Server.FIFO
    srv = Server(ctx.device, budget_bytes=120 * 1000 ** 3, policy=policy)
    lat, done_idx, pending = [], [], []
    try:
        t0 = time.perf_counter()

        def collect():
            keep = []
            for tk, i in pending:
                r = srv.result(tk, 0)
                if r is None:
                    keep.append((tk, i))
                else:
                    lat.append(r[2])
                    done_idx.append((i, r))
            pending[:] = keep

        for at, i in arrivals:
            while True:
                delay = t0 + at - time.perf_counter()
                if delay <= 0:
                    break
                collect()
                time.sleep(min(delay, 0.005))
            pending.append((srv.submit(data[i], specs[i].order, specs[i].outputs), i))
        while time.perf_counter() - t0 < duration:
            collect()
            time.sleep(0.005)
        collect()
        window = time.perf_counter() - t0
        st = srv.stats()
    finally:
        t1 = time.perf_counter()
        srv.close()
        close_s = time.perf_counter() - t1
    # each completed served result equals the same scan searched alone
    checked, same_served = 0, True
    alone = {}
    for i, (r, v64, _) in done_idx:
        if i not in alone:
            rr = Resident(ctx, data[i])
            alone[i] = gs.run(rr, specs[i].order, Distribution(specs[i].snps, specs[i].order - 1), specs[i].outputs,
                              with_fp64=True)
            rr.free()
        ar, av = alone[i]
        same_served &= [x.combination for x in r] == [x.combination for x in ar] and np.array_equal(v64, av)
        checked += 1
    lat.sort()
    offered_work = sum(specs[i].combos() * specs[i].samples for _, i in arrivals)
    out["served"] = {
        "workload": "Poisson arrivals of full-size scans drawn uniformly from the 64 above (configuration 5), "
                    "120 GB device budget",
        "policy": "shortest-first (least combinations x samples taken first)" if policy == Server.SHORTEST_FIRST
                  else "fifo (submission order)",
        "offered_scans_per_s": rate, "duration_s": duration, "requests": len(arrivals),
        "offered_combos_samples_per_s": offered_work / duration,
        "completed": int(st["completed"]), "completed_scans_per_s": st["completed"] / window,
        "completed_combos_samples_per_s": st["combos_samples"] / window,
        "backlog_at_end": int(st["queued"] + st["active"]), "queued_at_end": int(st["queued"]),
        "admitted_at_end": int(st["active"]), "peak_device_bytes": int(st["peak_bytes"]),
        "p50_ms": lat[len(lat) // 2] if lat else None,
        "p99_ms": lat[min(len(lat) - 1, int(0.99 * (len(lat) - 1) + 0.5))] if lat else None,
        "latency_of": "completed scans (submit -> result)",
        "rounds": int(st["rounds"]), "solo": int(st["solo"]), "overlapped": int(st["overlapped"]),
        "rounds_note": "every scan of this distribution is one-hot over its whole data set, so each runs on a "
                       "tensor-core (or pair-major order-4) kernel on a solo lane; the rounds serve the other scans",
        "identical_to_alone": bool(same_served), "checked": checked, "destroy_s": close_s, "unit": UNIT}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="order3_2000x8000")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--snps", type=int, default=0, help="override the SNP count (small profiling cases)")
    ap.add_argument("--kernel", type=int, default=0, help="force a counting kernel (0 = automatic choice)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched / served measurements")
    ap.add_argument("--no-ingest", action="store_true", help="skip the file ingest timing")
    ap.add_argument("--profile-layer", default="", metavar="STEP,OFFSET",
                    help="profiling case: search Distribution(snps, order-1, STEP, OFFSET) twice and exit")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="served stream: Poisson arrivals per second")
    ap.add_argument("--serve-policy", default="shortest", choices=["shortest", "fifo"],
                    help="served stream: order in which queued scans are admitted and run")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="served stream: arrival window (60 s, the served configuration's loop)")
    ap.add_argument("--batch-cap", type=float, default=2e12,
                    help="batched form: combinations x samples searched per scan (a leading shard of larger scans)")
    ap.add_argument("--batch-passes", type=int, default=3, help="batched form: timed passes per arm (median)")
    args = ap.parse_args()
    import dataclasses

    from fiuncho_gb300 import synth
    spec = synth.WORKLOADS[args.workload]
    if args.snps:
        spec = dataclasses.replace(spec, snps=args.snps)
        args.workload = "%s@%dsnps" % (args.workload, args.snps)
    if args.impl == "reference":
        run_reference(args, spec)
    else:
        run_gpu(args, spec)


if __name__ == "__main__":
    main()
