#!/usr/bin/env python3
"""Benchmark of the WRS hot path on GB300 (one JSON line on stdout, rank 0).

Workload (the single-large-distribution configuration): N = 2^26 FP32 weights in three
seeded distributions -- uniform(0,1], Zipf-like (i+1)^-1.1 randomly permuted, log-normal
(0, 2).  One step = PSA alias-table build (total mass -> fused prefix-partition ->
split+pack) of one distribution (cycling through the three) + S = 2^28 alias samples
(Philox4x32-10, key = seed, counter = sample index, uint32 indices).  Inputs (256 MB of
weights, a 512 MB table, 1 GB of samples) are larger than the 126 MB L2, so no flush is
needed between steps.

  value   samples/s over the timed steps (build included), inputs resident in HBM
  e2e     the same through the C ABI with host buffers: pinned H2D of the weights and D2H
          of the samples inside every timed step
  roofline  the dominant kernel (alias sampling): algorithmic 12 B/sample (8 B entry + 4 B
          index) / its mean CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU port of the same path (oracle/, single thread) on a bounded sample

Extra keys measure the rest of the configuration with the same events: per-kernel times
and bandwidths, the decoupled scan (weights scanned/s) and ITS sampling (samples/s); and
"batched", the mixed-size configuration (4096 distributions, N log-uniform in [64, 2^20],
2^30 samples in total) as one CUDA graph against 4096 per-call build + sample pairs; and
"served", a Poisson stream of 200k build+sample requests through the continuous-batching
server (p50/p99 latency, samples/s, alone-vs-mix equality).

`--impl reference` times the reference path's CPU implementation (the oracle port of
the reference's CPU code; its own compiled CPU code when that loads here) on all host
cores, on the same workload, and prints the same line with "impl": "reference".
Multi-GPU runs are independent replicas (the path does not shard one distribution).
"""
from __future__ import annotations

import argparse
import dataclasses
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LOG2_N = 26
LOG2_S = 28
SEEDS = (2, 3, 4)  # the workloads' HEADLINE_SEEDS
DISTS = ("uniform(0,1]", "zipf(s=1.1, permuted)", "lognormal(0,2)")
WORKLOAD = ("single large distribution: N=2^26 FP32 weights x 3 seeded distributions "
            "(uniform(0,1], Zipf s=1.1 permuted, log-normal(0,2)); step = PSA alias build + "
            "S=2^28 alias samples (Philox4x32-10, uint32 indices)")
METRIC = "samples/s"
# PSA split size of the single-distribution configuration, fixed so that the line's config is
# the same in every run: 12 is the autotuner's pick on GB300 at N = 2^26 (split+pack 0.70 ms
# uniform / 0.60 ms log-normal at 12, 0.72 / 0.67 at 8, 1.11 / 1.04 at 4, 0.88 / 0.85 at 24;
# float-float table accuracy does not depend on it).  The batched configuration tunes its
# split size live.
SPLIT_SIZE = 12
# end-to-end: the samples of a step leave the device in this many pieces
E2E_CHUNKS = 8
E2E_PASSES = 5
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "alias_sample_n26_s28.md")


def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over the ranks of the job (the job's time is its slowest replica's); x
    itself without a process group."""
    if dist is None or not dist.is_initialized():
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def headline_config(n: int, s: int, world: int) -> dict:
    """The headline configuration, the same for both arms (other sizes, from --log2n /
    --log2s, are named as what they are)."""
    workload = WORKLOAD
    l2 = "inputs larger than L2 (256 MB weights, 512 MB table, 1 GB samples)"
    if (n, s) != (1 << LOG2_N, 1 << LOG2_S):
        workload = WORKLOAD.replace("N=2^26", f"N=2^{n.bit_length() - 1}").replace(
            "S=2^28", f"S=2^{s.bit_length() - 1}")
        l2 = (f"{4 * n >> 20} MB weights, {8 * n >> 20} MB table, {4 * s >> 20} MB samples "
              "(L2: 129 MB)")
    return {"workload": workload, "N": n, "S": s, "split_size": SPLIT_SIZE,
            "rng": "philox4x32-10", "precision": "float-float partition prefix",
            "split": "float-float residual, light cap fixed", "l2": l2,
            "parallelism": f"replicas x{world}"}


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--log2n", type=int, default=LOG2_N)
    p.add_argument("--log2s", type=int, default=LOG2_S)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--l2-fetch", type=int, default=None,
                   help="set the context's L2 fetch granularity (bytes) instead of tuning it")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the per-distribution rows, statistics and per-kernel breakdown")
    p.add_argument("--no-batched", action="store_true",
                   help="skip the batched mixed-size configuration (4096 distributions)")
    p.add_argument("--no-served", action="store_true",
                   help="skip the served request-stream configuration (200k requests)")
    p.add_argument("--no-small", action="store_true",
                   help="skip the plain small configuration (N = 65,536)")
    p.add_argument("--no-precision", action="store_true",
                   help="skip the precision study (N = 2^28, S = 2^30)")
    p.add_argument("--batched-only", action="store_true",
                   help="only run the batched configuration and print its object (profiling)")
    p.add_argument("--small-only", action="store_true",
                   help="only run the plain small configuration and print its object")
    p.add_argument("--probe-gather", action="store_true",
                   help="only measure the random-gather rate per load width and exit")
    return p.parse_args()


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def launches_per_step(n: int) -> int:
    """The library's kernel launches in one headline step (wrs_build + wrs_sample): total mass,
    partition, the split descent (split-pack grids of >= 512 CTAs of 479 subproblems), the
    split-pack, the coin filter (2^22 < N <= 2^26) and the sampler."""
    blocks = -(-(n // SPLIT_SIZE) // 479)
    return 4 + (blocks >= 512) + ((1 << 22) < n <= (1 << 26))


def profiled_traffic(l2_fetch: int) -> float | None:
    """DRAM bytes of one headline alias-sampling launch (with the tables' coin filters, the
    mean over the three distributions' launches) at the given L2 fetch granularity, from the
    committed ncu summary (a line `dram_bytes_per_launch_coin_filter[l2=B]: X` per captured
    granularity), if it holds that granularity."""
    if not os.path.exists(PROFILE_TRAFFIC):
        return None
    key = f"dram_bytes_per_launch_coin_filter[l2={l2_fetch}]:"
    for line in open(PROFILE_TRAFFIC):
        if line.strip().startswith(key):
            return float(line.split(":", 1)[1].split()[0])
    return None


# ------------------------------------------------------------------ inputs ---

def make_weights(dist: int, n: int, seed: int, device):
    """Seeded synthetic weights of the configuration's three shapes (generated on the GPU;
    the CPU legs copy them back)."""
    from importlib import import_module
    return import_module("merian-wrs_gb300.workloads").headline(dist, n, seed, device)


# ------------------------------------------------------------------ clocks ---

class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.2)
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


# ------------------------------------------------------------------ CPU legs ---

def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_step(w_host, n: int, s: int, nthreads: int) -> tuple[float, dict]:
    """One whole step of the CPU path, nothing extrapolated: PSA build of n weights (the
    headline's split size and float-float split) + s alias samples (Philox4x32-10), on
    nthreads threads.  Returns (seconds, description)."""
    from oracle.oracle import RNG_PHILOX4X32_10, SPLIT_FLOAT_FLOAT, SPLIT_FULL_LIGHT, Oracle
    orc = Oracle()
    t0 = time.perf_counter()
    table, _, _ = orc.psa_build(w_host, SPLIT_SIZE, nthreads=nthreads,
                                flags=SPLIT_FLOAT_FLOAT | SPLIT_FULL_LIGHT)
    t1 = time.perf_counter()
    orc.alias_sample(table, s, 7, rng=RNG_PHILOX4X32_10, nthreads=nthreads)
    t2 = time.perf_counter()
    return t2 - t0, {"build_s": t1 - t0, "sample_s": t2 - t1}


def cpu_scan_its(w_host, nthreads: int, s: int = 1 << 24) -> dict:
    """The large configuration's other two CPU paths beside the GPU's: the Kahan inclusive
    prefix sum of the N weights on one thread (the oracle's restatement of the reference's
    host prefix_sum, src/host/reference/prefix_sum.hpp:17-74) and the lower-bound ITS sampler
    (Philox4x32-10) over that CMF on all threads, on a bounded sample of s draws."""
    from oracle.oracle import RNG_PHILOX4X32_10, Oracle
    orc = Oracle()
    n = w_host.size
    t0 = time.perf_counter()
    cmf = orc.prefix_kahan(w_host)
    t1 = time.perf_counter()
    orc.its_sample(cmf.astype("float32"), s, 7, rng=RNG_PHILOX4X32_10, nthreads=nthreads)
    t2 = time.perf_counter()
    return {"kind": "port", "scan_cores": 1, "its_cores": nthreads,
            "sample": f"the whole N-weight scan; {s} ITS draws (a bounded sample of the 2^28)",
            "scan_s": t1 - t0, "weights_scanned_per_s": n / (t1 - t0),
            "its_sample_s": t2 - t1, "its_samples_per_s": s / (t2 - t1)}


def reference_cpu(w_host, split_size: int = 32) -> dict:
    """The reference's own CPU code (oracle/_ref, compiled from its sources where the
    reference checkout is present), single-threaded as it is written: the PSA alias table
    host::reference::pmr::psa_alias_table at split size 32 (src/host/reference/
    psa_alias_table.hpp:23-67) and the Kahan prefix_sum (src/host/reference/prefix_sum.hpp:
    17-74), beside the oracle port's single-thread PSA build of the same weights at the same
    split size.  The reference has no sampler on the host, so samples/s is the port's only."""
    from oracle.oracle import Oracle, Reference
    if not Reference.available():
        return {"unavailable": "oracle/_ref (the reference's CPU code, compiled from the "
                               "reference checkout) is not built on this machine; the "
                               "reference checkout is not present here"}
    ref, orc = Reference(), Oracle()
    n = w_host.size
    t0 = time.perf_counter()
    ref.psa_alias_table(w_host, max(1, n // split_size))
    t1 = time.perf_counter()
    ref.prefix_sum(w_host)
    t2 = time.perf_counter()
    orc.psa_build(w_host, split_size, nthreads=1)
    t3 = time.perf_counter()
    return {"kind": "reference", "cores": 1, "N": n, "split_size": split_size,
            "psa_alias_table_s": t1 - t0, "alias_builds_per_s": 1.0 / (t1 - t0),
            "kahan_prefix_sum_s": t2 - t1, "weights_scanned_per_s": n / (t2 - t1),
            "port_psa_build_s_1thread": t3 - t2}


def run_reference(args) -> None:
    """--impl reference: the reference path's CPU implementation on all host cores; every step
    is one whole step of the workload (PSA build of N weights + S samples), timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    n, s = 1 << args.log2n, 1 << args.log2s
    nthreads = cpu_threads()
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    hosts = [make_weights(d, n, SEEDS[d], dev).cpu().numpy() for d in range(3)]
    for k in range(args.warmup):
        cpu_step(hosts[k % 3], n, s, nthreads)
    times, descs = [], []
    t_run = time.perf_counter()
    for k in range(args.steps):
        t, d = cpu_step(hosts[k % 3], n, s, nthreads)
        times.append(t)
        descs.append(d)
    t_run = time.perf_counter() - t_run
    total = sum(times)
    value = args.steps * s / total
    # the timed step is the oracle's port: the reference's own CPU code (reference_cpu below,
    # where it is built) has a PSA build and a scan but no sampler
    kind = "port"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": headline_config(n, s, args.gpus),
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": nthreads, "kind": kind,
                         "sample": f"every step whole: PSA build of N=2^{args.log2n} (split "
                                   f"{SPLIT_SIZE}, float-float split) + S=2^{args.log2s} "
                                   f"Philox4x32-10 alias samples, the three distributions in "
                                   f"turn; {nthreads} threads (the oracle's threaded port of "
                                   "the path: the reference's CPU code has no sampler)"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "cpu_build_s_mean": statistics.mean(d["build_s"] for d in descs),
        "cpu_sample_s_mean": statistics.mean(d["sample_s"] for d in descs),
        "timed_wall_s": t_run,
        "reference_cpu": reference_cpu(hosts[0]),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU ---

def probe_gather(args) -> None:
    """--probe-gather: random-gather rate per load width (4 .. 128 B) from a 512 MB buffer,
    one JSON line (the calibration behind the alias sampler's roofline)."""
    import torch
    pkg = importlib.import_module("merian-wrs_gb300")
    pkg.build()
    W = pkg.wrs
    nbytes, acc = 512 << 20, 1 << 26
    buf = torch.zeros(nbytes // 4, dtype=torch.int32, device="cuda")
    sink = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    out = {}
    for width in (4, 8, 16, 32, 64, 128):
        def launch():
            W.check(W.lib().wrs_probe_random_gather(stream.cuda_stream, buf.data_ptr(), nbytes,
                                                    acc, width, sink.data_ptr()))
        for _ in range(3):
            launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch()
        e1.record(stream)
        torch.cuda.synchronize()
        out[str(width)] = acc / (e0.elapsed_time(e1) / 1e3)
    print(json.dumps({"probe": "random gathers/s by load width (bytes), 512 MB buffer",
                      "gathers_per_s": out}), flush=True)


def main() -> None:
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.probe_gather:
        probe_gather(args)
        return
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    pkg = importlib.import_module("merian-wrs_gb300")
    pkg.build()
    W = pkg.wrs
    n, s = 1 << args.log2n, 1 << args.log2s
    cfg = W.AliasTableConfig(split_size=SPLIT_SIZE, rng=W.RNG_PHILOX4X32_10,
                             scan_precision=W.SCAN_FLOAT_FLOAT, split_residual_f64=True,
                             split_full_light=True)
    wrs = W.WRS(cfg)
    stream = torch.cuda.current_stream()
    dev = torch.device("cuda", local)
    if args.small_only:
        print(json.dumps({"small": small_leg(W, dev)}))
        return
    if args.batched_only:
        print(json.dumps({"batched": batched_leg(W, cfg, dev, stream, max(3, args.steps // 2),
                                                 max(3, args.warmup),
                                                 cpu=not args.no_cpu_baseline)}))
        return
    weights = [make_weights(d, n, SEEDS[d] + 1000 * rank, dev) for d in range(3)]
    internals = W.Internals(wrs.handle, n)
    samples = torch.empty(s, dtype=torch.int32, device=dev)
    bufs = [W.WRSBuffers(weights[d], samples, internals) for d in range(3)]

    # the context's L2 fetch granularity, tuned live on the first distribution (the split
    # size stays fixed); it changes no result
    if args.l2_fetch is None:
        tune = W.autotune_alias(cfg, stream, weights[0], n, s, samples, split_sizes=[],
                                l2_fetch=None, warmup=1, reps=2)
    else:
        W.set_l2_fetch_granularity(args.l2_fetch)
        tune = {"l2_fetch": W.get_l2_fetch_granularity(), "trials": []}

    def step(k: int, ev=None):
        b = bufs[k % 3]
        if ev is not None:
            ev[0].record(stream)
        wrs.build(stream, b, n)
        if ev is not None:
            ev[1].record(stream)
        wrs.sample(stream, b, n, s, seed=1234 + k)
        if ev is not None:
            ev[2].record(stream)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    dev_status = internals.status()
    assert not dev_status & W.DEVICE_TIMEOUT, "a lookback wait gave up during warm-up"

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timed region
    clocks = Clocks(local)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    clocks.start()
    e_start.record(stream)
    for k in range(args.steps):
        step(k, evs[k])
    e_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    elapsed_ms = e_start.elapsed_time(e_end)
    build_ms = [e[0].elapsed_time(e[1]) for e in evs]
    sample_ms = [e[1].elapsed_time(e[2]) for e in evs]
    elapsed_ms = max_over_ranks(elapsed_ms, dist, dev)
    value = world * args.steps * s / (elapsed_ms / 1e3)
    dev_status |= internals.status()
    assert not dev_status & W.DEVICE_TIMEOUT, "a lookback wait gave up in the timed region"

    # ---- end to end through the C ABI with host buffers.  Every step copies its weights from
    # pinned host memory (cudaMemcpyAsync on a copy stream, into one of two device buffers, so
    # the next step's copy overlaps this step's work), builds, and samples in E2E_CHUNKS
    # pieces (wrs_sample_at with the piece's offset) into one of two device sample buffers;
    # each piece's device-to-host copy into pinned host memory starts on an output stream as
    # soon as the piece is drawn, so the host link carries the samples while the device draws
    # the rest and builds the next step.  The last step's copies end inside the timed region.
    # e2e_kernel_to_host: the sampling kernel writes straight into pinned host memory;
    # e2e_serial: one device buffer, copies and work all on one stream.
    host_w = [weights[d].cpu().pin_memory() for d in range(3)]
    host_s = torch.empty(s, dtype=torch.int32).pin_memory()
    dev_w2 = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(2)]
    dev_s2 = [samples, torch.empty(s, dtype=torch.int32, device=dev)]
    cstream = torch.cuda.Stream(device=dev)
    ostream = torch.cuda.Stream(device=dev)
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    drawn = [[torch.cuda.Event() for _ in range(E2E_CHUNKS)] for _ in range(2)]
    L = W.lib()

    def load_build(k: int) -> int:
        b = k % 2
        cstream.wait_event(free[b])
        with torch.cuda.stream(cstream):
            dev_w2[b].copy_(host_w[k % 3], non_blocking=True)
        ready[b].record(cstream)
        stream.wait_event(ready[b])
        wrs.build(stream, W.WRSBuffers(dev_w2[b], None, internals), n)
        free[b].record(stream)
        return b

    def e2e_step(k: int):
        b = load_build(k)
        stream.wait_event(copied[b])  # the buffer's previous samples have left the device
        piece = s // E2E_CHUNKS
        for c in range(E2E_CHUNKS):
            off = c * piece
            W.check(L.wrs_sample_at(wrs.handle.ptr, stream.cuda_stream, internals.ptr, n, piece,
                                    1234 + k, off, dev_s2[b].data_ptr() + 4 * off))
            drawn[b][c].record(stream)
            ostream.wait_event(drawn[b][c])
            with torch.cuda.stream(ostream):
                host_s[off:off + piece].copy_(dev_s2[b][off:off + piece], non_blocking=True)
        copied[b].record(ostream)

    def e2e_kernel_to_host_step(k: int):
        b = load_build(k)
        wrs.sample(stream, W.WRSBuffers(dev_w2[b], host_s.data_ptr(), internals), n, s,
                   seed=1234 + k)

    def e2e_serial_step(k: int):
        dev_w2[0].copy_(host_w[k % 3], non_blocking=True)
        wrs.build(stream, W.WRSBuffers(dev_w2[0], samples, internals), n)
        wrs.sample(stream, W.WRSBuffers(dev_w2[0], samples, internals), n, s, seed=1234 + k)
        host_s.copy_(samples, non_blocking=True)

    def e2e_time(fn) -> float:
        for e in free + copied:
            e.record(stream)
        for k in range(min(args.warmup, 2)):
            fn(k)
        stream.wait_stream(ostream)
        barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        cstream.wait_stream(stream)  # no copy starts before t0
        ostream.wait_stream(stream)
        for k in range(args.steps):
            fn(k)
        stream.wait_stream(ostream)  # the last samples are in host memory
        t1.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(t0.elapsed_time(t1), dist, dev)

    # five timed passes of the pipelined loop, the median reported: run alone the loop repeats
    # to 0.1 % (16 passes in two processes, 41.28-41.36 G samples/s on one box), but inside
    # the benchmark one or two of three passes have fallen to 24-38 G while the others ran at
    # 41.3 G, so one or two disturbed passes do not set the figure; all passes are in the
    # line, in the order they ran
    e2e_order = [e2e_time(e2e_step) for _ in range(E2E_PASSES)]
    e2e_passes = sorted(e2e_order)
    e2e_ms = e2e_passes[len(e2e_passes) // 2]
    e2e_value = world * args.steps * s / (e2e_ms / 1e3)
    e2e_k2h_value = world * args.steps * s / (e2e_time(e2e_kernel_to_host_step) / 1e3)
    e2e_serial_value = world * args.steps * s / (e2e_time(e2e_serial_step) / 1e3)
    link = host_link_rates(host_s, samples, host_w[0], dev_w2[0], stream)
    check = host_s[:1024].numpy().view(np.uint32)
    assert int(check.max()) < n, "samples written to host memory out of range"

    # ---- roofline of the dominant kernel (alias sampling)
    pk = peaks()
    samp_s = statistics.mean(sample_ms) / 1e3
    achieved = 12.0 * s / samp_s / 1e9
    traffic = profiled_traffic(tune["l2_fetch"])
    gather_rate = random_gather_rate(W, internals, n, s, stream)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                "traffic_l2_fetch": tune["l2_fetch"],
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per "
                                  "headline launch (mean of the uniform, Zipf and log-normal "
                                  "launches, coin filters in use) at this run's L2 fetch "
                                  "granularity, null where none was captured at it "
                                  "(profiles/alias_sample_n26_s28.md)",
                "kernel": "k_alias_sample",
                "bytes_model": "12 B/sample (8 B entry + 4 B index), as without the coin "
                               "filter; with it the entry is read only where the coin does "
                               "not decide (plus 1 B of filter from L2)",
                "peak_source": pk["source"],
                "sector_model_frac": (36.0 * s / samp_s / 1e9) / pk["hbm_gbs"],
                "random_gather": {
                    "rate": gather_rate, "unit": "gathers/s",
                    "frac": (s / samp_s) / gather_rate,
                    "model": "random 8-byte loads from the same 512 MB table, one per thread "
                             "(wrs_probe_random_gather, CUDA events): the bound of sampling "
                             "from a table larger than L2, where each gather costs a DRAM burst "
                             "of ~107 B whatever its width"}}

    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": headline_config(n, s, world),
        "autotune": {"l2_fetch": tune["l2_fetch"], "trials": tune["trials"],
                     "method": "wrs_autotune_alias over L2 fetch granularity 32/64/128 B at "
                               f"split size {SPLIT_SIZE} (CUDA events, 1 warm-up + 2 timed "
                               "build+sample calls each), before the warm-up steps"},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * s,
                "method": "weights: pinned host -> device copy per step on a copy stream, "
                          "double-buffered (overlaps the previous step); samples: drawn in "
                          f"{E2E_CHUNKS} pieces into one of two device buffers, each piece "
                          "copied to pinned host memory on an output stream as soon as it is "
                          "drawn (overlaps the rest of the step and the next build); the median "
                          f"of {E2E_PASSES} timed passes of {args.steps} steps",
                "passes_samples_per_s": [world * args.steps * s / (ms / 1e3)
                                         for ms in e2e_order],
                "kernel_to_host_value": e2e_k2h_value,
                "serial_value": e2e_serial_value,
                "host_link": link},
        "roofline": roofline,
        "alias_builds_per_s": world / (statistics.mean(build_ms) / 1e3),
        "build_ms_mean": statistics.mean(build_ms),
        "sample_ms_mean": statistics.mean(sample_ms),
        "clocks": clk,
        "gpu_launches": launches_per_step(n) * args.steps,
        "device_status": {"timeout": bool(dev_status & W.DEVICE_TIMEOUT),
                          "split_overlap_beyond_window": bool(dev_status & W.DEVICE_NONMONOTONE_SPLIT)},
    }

    # every distribution of the configuration: its kernels timed alone and the statistics of
    # its alias and ITS samples
    if not args.no_extras:
        dists = per_distribution(W, wrs, internals, weights, samples, n, s, stream,
                                 pk["hbm_gbs"])
        line["statistics"] = {name: row["alias_statistics"] for name, row in dists.items()}
        line["per_distribution"] = dists
        line["kernels"] = kernel_breakdown(W, pkg, wrs, internals, weights, samples, n, s,
                                           stream, pk["hbm_gbs"], args)
    if not args.no_batched:
        line["batched"] = batched_leg(W, cfg, dev, stream, max(3, args.steps // 2),
                                      max(3, args.warmup), cpu=not args.no_cpu_baseline)
    if not args.no_served:
        line["served"] = served_leg(W, cfg, dev)
    if not args.no_small:
        line["small"] = small_leg(W, dev)
    if not args.no_precision:
        line["precision"] = precision_leg(W, dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        w0 = weights[0].cpu().numpy()
        nthreads = cpu_threads()
        t_step, desc = cpu_step(w0, n, s, nthreads)
        line["cpu_baseline"] = {
            "value": s / t_step, "unit": "samples/s", "cores": nthreads, "kind": "port",
            "sample": f"one whole step, nothing extrapolated: PSA build of N=2^{args.log2n} "
                      f"uniform weights ({desc['build_s']:.2f} s) + S=2^{args.log2s} "
                      f"Philox4x32-10 alias samples ({desc['sample_s']:.2f} s); {nthreads} "
                      "threads (the oracle's threaded port of the path)",
            "scan_and_its": cpu_scan_its(w0, nthreads),
            "reference_cpu": reference_cpu(w0)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


BATCH_DISTS = 4096
BATCH_LOG2_S = 30
BATCH_SEED = 6


CPU_SAMPLE_ITEMS = 256


def cpu_batch_baseline(items, total_s: int, what: str, reuse=None, seed: int = 60,
                       split_size: int = SPLIT_SIZE) -> dict:
    """The CPU port (oracle, float-float split, Philox4x32-10) on a seeded uniform sample of
    CPU_SAMPLE_ITEMS of the distributions / requests, all host cores in a thread pool over
    the items (one item per thread, as independent distributions shard); the time is scaled
    by items / sampled items.  items: (device weights, s, seed); reuse: items whose table is
    resident (sampled only)."""
    import concurrent.futures as cf
    import numpy as np
    from oracle.oracle import RNG_PHILOX4X32_10, SPLIT_FLOAT_FLOAT, SPLIT_FULL_LIGHT, Oracle
    orc = Oracle()
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(items), min(CPU_SAMPLE_ITEMS, len(items)), replace=False)
    host = [(items[i][0].cpu().numpy(), items[i][1], items[i][2],
             bool(reuse[i]) if reuse is not None else False) for i in pick]
    def one(k):
        """seconds of CPU work for item k: build + sampling, or sampling alone for a request
        whose table is resident (its build is done untimed)"""
        w, s, seed_k, reused = host[k]
        t0 = time.perf_counter()
        table, _, _ = orc.psa_build(w, split_size, nthreads=1,
                                    flags=SPLIT_FLOAT_FLOAT | SPLIT_FULL_LIGHT)
        t1 = time.perf_counter()
        orc.alias_sample(table, s, seed_k, rng=RNG_PHILOX4X32_10, nthreads=1)
        t2 = time.perf_counter()
        return (t2 - t1) if reused else (t2 - t0)

    nthreads = cpu_threads()
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        work = sum(ex.map(one, range(len(host))))
    elapsed = work / nthreads * len(items) / len(host)  # perfectly balanced over the threads
    return {"value": total_s / elapsed, "unit": "samples/s", "cores": nthreads, "kind": "port",
            "sample": f"{len(host)} of {len(items)} {what} (seeded uniform choice), one per "
                      f"thread on {nthreads} threads; CPU seconds summed, divided by the threads "
                      f"and scaled by {len(items) / len(host):.1f}" +
                      ("; requests on a resident table count their sampling only"
                       if reuse is not None else "")}


def batched_leg(W, cfg, dev, stream, steps: int, warmup: int, cpu: bool = True) -> dict:
    """The batched configuration: all 4096 distributions built and sampled by one CUDA graph
    (wrs_batch_build + wrs_batch_sample: 5 launches), against 4096 per-call wrs_build +
    wrs_sample pairs on the same stream, same inputs and seeds.  Both arms' samples are
    compared bit for bit and their per-distribution RMSE reported."""
    import numpy as np
    import torch
    wl = importlib.import_module("merian-wrs_gb300.workloads").batched(
        dev, BATCH_DISTS, BATCH_LOG2_S, BATCH_SEED)
    sizes, counts, w_off, s_off, w = wl["sizes"], wl["counts"], wl["w_off"], wl["s_off"], wl["w"]
    D = len(sizes)
    tables = torch.empty(2 * int(w_off[-1]), dtype=torch.int32, device=dev)
    out_b = torch.empty(int(s_off[-1]), dtype=torch.int32, device=dev)
    out_p = torch.empty_like(out_b)
    seeds = [77 + d for d in range(D)]
    wp, tp, bp, pp = w.data_ptr(), tables.data_ptr(), out_b.data_ptr(), out_p.data_ptr()
    dists = [(wp + 4 * int(w_off[d]), tp + 8 * int(w_off[d]), bp + 4 * int(s_off[d]),
              int(sizes[d]), int(counts[d]), seeds[d]) for d in range(D)]
    # autotuned: split size and L2 fetch granularity measured on this batch; both arms then
    # run the chosen configuration
    tune = W.autotune_batch(cfg, stream, dists, split_sizes=None, l2_fetch=None, warmup=1,
                            reps=2)
    cfg = dataclasses.replace(cfg, split_size=tune["split_size"])
    h = W.Handle(cfg)
    batch = W.Batch(h, D, int(sizes.sum()), int(counts.sum()))
    batch.set(stream, dists)
    batch.build(stream)
    batch.sample(stream)
    torch.cuda.synchronize()
    assert batch.status() == 0
    graph = torch.cuda.CUDAGraph()
    gs = torch.cuda.Stream()
    with torch.cuda.graph(graph, stream=gs):
        batch.build(torch.cuda.current_stream())
        batch.sample(torch.cuda.current_stream())
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / steps
    assert batch.status() == 0
    # the graph's two halves timed apart (the 4 build launches, the sampling launch)
    stages = {}
    for name, fn in (("build_ms", lambda: batch.build(stream)),
                     ("sample_ms", lambda: batch.sample(stream))):
        fn()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        stages[name] = e0.elapsed_time(e1) / steps
    assert batch.status() == 0

    # per call: one buffers object sized for the largest distribution, reused
    L = W.lib()
    wrs = W.WRS(cfg)
    internals = W.Internals(wrs.handle, int(sizes.max()))
    hp, ip, sp = wrs.handle.ptr, internals.ptr, stream.cuda_stream
    calls = [(wp + 4 * int(w_off[d]), int(sizes[d]), int(counts[d]), seeds[d],
              pp + 4 * int(s_off[d])) for d in range(D)]
    build, sample = L.wrs_build, L.wrs_sample_at

    def per_call_pass():
        for (wa, n, s, seed, oa) in calls:
            build(hp, sp, wa, n, ip)
            sample(hp, sp, ip, n, s, seed, 0, oa)

    for _ in range(warmup):
        per_call_pass()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        per_call_pass()
    e1.record(stream)
    torch.cuda.synchronize()
    per_call_py_ms = e0.elapsed_time(e1) / steps
    assert internals.status() == 0
    # the same per-call loop driven from C++ through include/wrs.hpp (libwrs_percall.so):
    # the primary per-call arm, with no interpreter between the calls
    import ctypes as C
    drv = C.CDLL(os.path.join(os.path.dirname(W.LIB_PATH), "libwrs_percall.so"))
    drv.wrs_percall_run.restype = C.c_int
    drv.wrs_percall_run.argtypes = [C.POINTER(W._Config), C.c_void_p, C.c_uint32, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.POINTER(C.c_float)]
    arr_w = (C.c_void_p * D)(*[c[0] for c in calls])
    arr_n = (C.c_uint32 * D)(*[c[1] for c in calls])
    arr_s = (C.c_uint64 * D)(*[c[2] for c in calls])
    arr_seed = (C.c_uint64 * D)(*[c[3] for c in calls])
    arr_out = (C.c_void_p * D)(*[c[4] for c in calls])
    ccfg = cfg.c()
    ms = C.c_float(0.0)
    args_c = (C.byref(ccfg), stream.cuda_stream, D, arr_w, arr_n, arr_s, arr_seed, arr_out)
    W.check(drv.wrs_percall_run(*args_c, warmup, C.byref(ms)))
    W.check(drv.wrs_percall_run(*args_c, steps, C.byref(ms)))
    per_call_ms = ms.value / steps

    # accuracy: both arms bit for bit, and the RMSE of each distribution's histogram
    identical = bool(torch.equal(out_b, out_p))
    # per distribution: the reference's chi-square over its items (df = items - 1) with its
    # p-value, the RMSE of the normalised histogram and the RMSE a multinomial draw has in
    # expectation; aggregated as the sum of the chi-squares over the sum of the dfs
    rmse, rmse_ratio, chi2s, dfs, pvals, bchi2, bdfs, bpvals = [], [], [], [], [], [], [], []
    vars_, pvals_m, bvars = [], [], []
    for d in range(D):
        n, s = int(sizes[d]), int(counts[d])
        if s == 0:
            continue
        smp = out_b[int(s_off[d]):int(s_off[d]) + s].long()
        o = torch.bincount(smp, minlength=n).double()
        wd = w[int(w_off[d]):int(w_off[d]) + n].double()
        p = wd / wd.sum()
        e = p * s
        pos = e > 0
        chi2 = float((((o - e) ** 2)[pos] / e[pos]).sum())
        r = float(torch.sqrt(torch.mean((o / s - p) ** 2)))
        rmse.append(r)
        rmse_ratio.append(r / float(torch.sqrt(torch.mean(p * (1 - p) / s))))
        chi2s.append(chi2)
        dfs.append(int(pos.sum()) - 1)
        vars_.append(multinomial_chi2_var(p, s))
        rep = chi2_report(chi2, dfs[-1], vars_[-1])
        pvals.append(rep["p_value"])
        pvals_m.append(rep.get("p_value_multinomial"))
        b = binned_chi2(o, e, 256.0)
        if b["df"] > 0:
            bchi2.append(b["chi2"])
            bdfs.append(b["df"])
            bvars.append(multinomial_chi2_var(p_binned(e, b["bin_items"]), s))
            bpvals.append(b["p_value"])
    pv = [x for x in pvals if x is not None]
    pvm = [x for x in pvals_m if x is not None]
    bpv = [x for x in bpvals if x is not None]
    total_s = int(counts.sum())
    return {
        "workload": f"batched mixed sizes: {D} distributions, N log-uniform in [64, 2^20] "
                    f"(sum {int(sizes.sum())}), uniform(0,1] or Zipf s=1.1 per distribution "
                    f"by seed; S_d proportional to N_d, sum 2^{BATCH_LOG2_S}; Philox4x32-10",
        "distributions": D, "weights": int(sizes.sum()), "samples": total_s,
        "autotune": {"split_size": tune["split_size"], "l2_fetch": tune["l2_fetch"],
                     "trials": tune["trials"],
                     "method": "wrs_autotune_batch: L2 fetch granularity 32/64/128 B at split "
                               f"size {SPLIT_SIZE}, then split sizes 4-32 at the best L2 value "
                               "(CUDA events, 1 warm-up + 2 timed batch build+sample each)"},
        "graph_ms": batched_ms, "stages": stages, "per_call_ms": per_call_ms,
        "samples_per_s": total_s / (batched_ms / 1e3),
        "per_call_samples_per_s": total_s / (per_call_ms / 1e3),
        "builds_per_s": D / (batched_ms / 1e3),
        "speedup_vs_per_call": per_call_ms / batched_ms,
        "per_call_python_ms": per_call_py_ms,
        "speedup_vs_per_call_python": per_call_py_ms / batched_ms,
        "graph_launches": 5, "per_call_launches": 5 * D,
        "samples_bitwise_equal": identical,
        "rmse_mean": statistics.mean(rmse), "rmse_max": max(rmse),
        "statistics": {
            **chi2_report(sum(chi2s), sum(dfs), sum(vars_)),
            "what": "sum over the distributions of the reference's chi-square (its items with "
                    "nonzero expectation, df = items - 1 each) and its p-value; per "
                    "distribution p-values summarised; *_multinomial: against the statistic's "
                    "exact multinomial variance (the sum over the distributions)",
            "rmse_mean": statistics.mean(rmse),
            "rmse_over_ideal_mean": statistics.mean(rmse_ratio),
            "rmse_over_ideal_max": max(rmse_ratio),
            "p_value_min": min(pv) if pv else None,
            "p_below_0.01_fraction": (sum(x < 0.01 for x in pv) / len(pv)) if pv else None,
            "p_multinomial_below_0.01_fraction": (sum(x < 0.01 for x in pvm) / len(pvm))
            if pvm else None,
            "distributions": len(chi2s),
            "binned": {**chi2_report(sum(bchi2), sum(bdfs), sum(bvars)),
                       "what": "per distribution the chi-square over bins of consecutive items "
                               "with a mean expectation of >= 256 samples (a distribution "
                               "that fills one bin has none), summed",
                       "distributions": len(bchi2),
                       "p_below_0.01_fraction": (sum(x < 0.01 for x in bpv) / len(bpv))
                       if bpv else None}},
        "per_call_driver": "C++ loop over the C++ facade of include/wrs.hpp (wrs::WRS::build + "
                           "sample per distribution, one reused wrs::WRSBuffers; "
                           "libwrs_percall.so, CUDA events around the loop); "
                           "per_call_python_ms: the same calls from a Python loop over the "
                           "C ABI",
        "cpu_baseline": cpu_batch_baseline(
            [(w[int(w_off[d]):int(w_off[d]) + int(sizes[d])], int(counts[d]), seeds[d])
             for d in range(D)], total_s, "distributions", split_size=cfg.split_size)
        if cpu else None,
    }


SERVED_REQUESTS = 200_000
SERVED_RATE = 50_000.0
SERVED_BUDGET = 16 << 30


def served_leg(W, cfg, dev, n_requests: int = SERVED_REQUESTS) -> dict:
    """The served configuration: a seeded Poisson stream of build+sample requests replayed in
    real time through wrs_server_run_trace (continuous batching over 3 stream slots, alias
    tables resident by id, 16 GiB device budget for tables and batch scratch).  Latency =
    completion seen by the host loop - arrival.  A seeded subset of requests is recomputed
    alone afterwards (a batch of one) and compared bit for bit with the served result."""
    import numpy as np
    import torch
    wl = importlib.import_module("merian-wrs_gb300.workloads").served(
        dev, n_requests, SERVED_RATE, seed=7)
    w, s_off = wl["w"], wl["s_off"]
    out = torch.zeros(int(s_off[-1]), dtype=torch.int32, device=dev)
    h = W.Handle(cfg)
    server = W.Server(h, memory_budget=SERVED_BUDGET)
    wp, op = w.data_ptr(), out.data_ptr()
    rows = [(int(wl["table_id"][i]), wp + 4 * int(wl["w_off"][i]), op + 4 * int(s_off[i]),
             int(wl["n"][i]), int(wl["s"][i]), int(wl["seeds"][i])) for i in range(n_requests)]
    reqs = W.Server.requests(rows)
    # warm-up: a short prefix of the stream, then a fresh server for the measured run
    server.run_trace(reqs, [0.0] * 64)
    torch.cuda.synchronize()
    del server
    server = W.Server(h, memory_budget=SERVED_BUDGET)
    comps = server.run_trace(reqs, [float(a) for a in wl["arrivals"]])
    torch.cuda.synchronize()
    st = server.stats()
    lat = np.array([comps[i].done_s - comps[i].submit_s for i in range(n_requests)])
    ok = all(comps[i].status == 0 for i in range(n_requests))
    t_first = min(comps[i].submit_s for i in range(n_requests))
    t_last = max(comps[i].done_s for i in range(n_requests))
    makespan = t_last - t_first
    total_s = int(wl["s"].sum())
    # alone vs in the mix
    rng = np.random.default_rng(70)
    pick = rng.choice(n_requests, 64, replace=False)
    batch = W.Batch(h, 1, int(wl["n"].max()), int(wl["s"].max()))
    tab = torch.empty(2 * int(wl["n"].max()), dtype=torch.int32, device=dev)
    alone = torch.empty(int(wl["s"].max()), dtype=torch.int32, device=dev)
    equal = 0
    chi2s, dfs, ratios, bchi2, bdfs, vars_, bvars = [], [], [], [], [], [], []
    for i in pick:
        n, s_i = int(wl["n"][i]), int(wl["s"][i])
        batch.set(None, [(wp + 4 * int(wl["w_off"][i]), tab, alone, n, s_i, int(wl["seeds"][i]))])
        batch.build(None)
        batch.sample(None)
        served_i = out[int(s_off[i]):int(s_off[i]) + s_i]
        equal += bool(torch.equal(alone[:s_i], served_i))
        # the served samples against the request's weights
        o = torch.bincount(served_i.long(), minlength=n).double()
        p = w[int(wl["w_off"][i]):int(wl["w_off"][i]) + n].double()
        p = p / p.sum()
        e = p * s_i
        pos = e > 0
        chi2s.append(float((((o - e) ** 2)[pos] / e[pos]).sum()))
        dfs.append(int(pos.sum()) - 1)
        vars_.append(multinomial_chi2_var(p, s_i))
        b = binned_chi2(o, e, 64.0)
        if b["df"] > 0:
            bchi2.append(b["chi2"])
            bdfs.append(b["df"])
            bvars.append(multinomial_chi2_var(p_binned(e, b["bin_items"]), s_i))
        ratios.append(float(torch.sqrt(torch.mean((o / s_i - p) ** 2))) /
                      float(torch.sqrt(torch.mean(p * (1 - p) / s_i))))
    return {
        "workload": f"served request stream: {n_requests} build+sample requests, Poisson "
                    f"arrivals at {SERVED_RATE:.0f} req/s, N log-uniform in [256, 2^22] "
                    f"log-normal(1.5) weights, S log-uniform in [1, 65536], 30% reuse a "
                    f"recent table by id; 16 GiB budget; 3 stream slots",
        "requests": n_requests, "samples": total_s, "all_ok": ok,
        "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)),
                       "p99": 1e3 * float(np.percentile(lat, 99)),
                       "mean": 1e3 * float(lat.mean()), "max": 1e3 * float(lat.max())},
        "samples_per_s": total_s / makespan, "requests_per_s": n_requests / makespan,
        "offered_requests_per_s": SERVED_RATE, "makespan_s": makespan,
        "batches": st["batches"], "builds": st["builds"], "resident_reuses": st["reuses"],
        "evictions": st["evictions"], "table_bytes_peak": st["table_bytes_peak"],
        "scratch_bytes": st["scratch_bytes"], "device_status": st["device_status"],
        "alone_vs_mix_equal": f"{equal}/{len(pick)}",
        "statistics": {
            **chi2_report(sum(chi2s), sum(dfs), sum(vars_)),
            "what": f"the {len(pick)} alone-vs-mix requests' served samples: sum of the "
                    "reference's chi-squares over their items (df = items - 1 each) and its "
                    "p-value; most requests draw far fewer samples than they have items, where "
                    "the chi-square distribution does not describe the statistic: "
                    "*_multinomial holds it against its exact multinomial variance (summed "
                    "over the requests) instead",
            "rmse_over_ideal_mean": statistics.mean(ratios),
            "rmse_over_ideal_max": max(ratios),
            "binned": {**chi2_report(sum(bchi2), sum(bdfs), sum(bvars)),
                       "what": "per request the chi-square over bins of consecutive items with "
                               "a mean expectation of >= 64 samples (requests of fewer samples "
                               "fill one bin and have none), summed",
                       "requests": len(bchi2)}},
        "cpu_baseline": cpu_batch_baseline(
            [(w[int(wl["w_off"][i]):int(wl["w_off"][i]) + int(wl["n"][i])], int(wl["s"][i]),
              int(wl["seeds"][i])) for i in range(n_requests)], total_s, "requests",
            reuse=[bool(wl["table_id"][i] != i) for i in range(n_requests)]),
    }


def _dev_copy(dst, src_ptr: int, nbytes: int) -> None:
    """Device-to-device copy from a raw device address (an internals view) into a tensor."""
    import ctypes
    import torch
    torch.cuda.synchronize()
    rt = ctypes.CDLL("libcudart.so." + torch.version.cuda.split(".")[0])
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(dst.data_ptr(), src_ptr, nbytes, 3) == 0


def _implied(table, n: int):
    """Probability mass (in mean units) an alias table gives each index, on the device:
    p_i + sum over buckets j aliasing to i of (1 - p_j)."""
    import torch
    t = table.view(torch.int32).view(-1, 2)
    p = t[:, 0].contiguous().view(torch.float32).double()
    a = t[:, 1].long()
    return p.index_add(0, a, 1.0 - p)


def precision_leg(W, dev, log2n: int = 28, log2s: int = 30) -> dict:
    """The precision study: N = 2^28 log-normal(0, 3) weights with 1% forced to 0 and 0.01%
    scaled by 1e6.  Scans (plain FP32 carry, compensated carry) against an FP64 scan of the
    same weights (torch.cumsum in FP64); alias tables of the three precisions against
    w / mean (FP64); RMSE of S = 2^30 ITS and alias draws against w / sum(w); zero-weight
    indices must never be drawn."""
    import torch
    n, s = 1 << log2n, 1 << log2s
    w = importlib.import_module("merian-wrs_gb300.workloads").precision(n, dev)
    ref = torch.cumsum(w.double(), 0)
    pos = ref > 0
    total = float(ref[-1])
    target = w.double() / total
    out = {"workload": f"precision study: N=2^{log2n} log-normal(0,3), 1% zeros, 0.01% x1e6; "
                       f"S=2^{log2s} draws per sampler", "N": n, "S": s,
           "statistics": "wrs_histogram + wrs_sample_statistics on the device"}
    stats = W.Statistics(n)
    cmf = torch.empty(n, dtype=torch.float32, device=dev)
    scans = {}
    for name, prec in (("fp32", W.SCAN_FP32), ("compensated", W.SCAN_COMPENSATED)):
        its = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=prec))
        internals = W.Internals(its.handle, n)
        its.prefix_sum(None, w, n, cmf, internals)
        torch.cuda.synchronize()
        rel = ((cmf.double() - ref).abs() / ref.clamp_min(1e-300))[pos]
        scans[name] = {"max_rel_prefix_err": float(rel.max()),
                       "max_rel_err_last": float(abs(float(cmf[-1]) - total) / total)}
        if prec == W.SCAN_COMPENSATED:
            samples = torch.empty(s, dtype=torch.int32, device=dev)
            its.its_sample(None, cmf, n, s, 11, 0, samples)
            r = sample_statistics(stats, samples, s, w, n, bin_target=8192.0)
            scans[name]["its_rmse"] = r["rmse"]
            scans[name]["its_zero_weight_draws"] = r["zero_weight_draws"]
            scans[name]["its_statistics"] = r
            del samples
        del internals
    out["scan"] = scans
    tables = {}
    mean_units = w.double() / (total / n)
    for name, prec in (("fp32", W.SCAN_FP32), ("compensated", W.SCAN_COMPENSATED),
                       ("float-float", W.SCAN_FLOAT_FLOAT)):
        cfg = W.AliasTableConfig(split_size=SPLIT_SIZE, rng=W.RNG_PHILOX4X32_10,
                                 scan_precision=prec, split_residual_f64=True,
                                 split_full_light=True)
        wrs = W.WRS(cfg)
        internals = W.Internals(wrs.handle, n)
        samples = torch.empty(s, dtype=torch.int32, device=dev)
        wrs.build(None, W.WRSBuffers(w, samples, internals), n)
        wrs.sample(None, W.WRSBuffers(w, samples, internals), n, s, seed=11)
        torch.cuda.synchronize()
        table_t = torch.empty(2 * n, dtype=torch.int32, device=dev)
        _dev_copy(table_t, internals.views()["alias_table"], 8 * n)
        imp = _implied(table_t, n)
        err = (imp - mean_units).abs()
        r = sample_statistics(stats, samples, s, w, n, bin_target=8192.0)
        tables[name] = {"max_abs_err_mean_units": float(err.max()),
                        "max_rel_err_w_ge_mean": float((err / mean_units)[mean_units >= 1].max()),
                        "alias_rmse": r["rmse"], "chi2": r["chi2"], "df": r["df"],
                        "p_value": r["p_value"], "z_score": r["z_score"],
                        "z_multinomial": r.get("z_multinomial"),
                        "p_value_multinomial": r.get("p_value_multinomial"), "binned": r["binned"],
                        "zero_weight_draws": r["zero_weight_draws"],
                        "zero_weight_mass": float(imp[w == 0].sum()),
                        "status": internals.status()}
        del internals, samples, table_t, imp, err
        torch.cuda.empty_cache()
    out["alias"] = tables
    out["rmse_ideal"] = float(torch.sqrt(torch.mean(target * (1 - target) / s)))
    return out


def small_leg(W, dev, steps: int = 20) -> dict:
    """The plain small configuration: N = 65,536 uniform(0,1] weights (seed 1), PSA build +
    S = 2^20 Philox4x32-10 samples (seed 1); builds/s and samples/s over `steps` repetitions,
    chi-square (df = N - 1) p-value and RMSE of the histogram against w / sum(w)."""
    import numpy as np
    import torch
    n, s = 65536, 1 << 20
    cfg = W.AliasTableConfig(split_size=2, rng=W.RNG_PHILOX4X32_10)
    wrs = W.WRS(cfg)
    w = make_weights(0, n, 1, dev)
    samples = torch.empty(s, dtype=torch.int32, device=dev)
    bufs = W.WRSBuffers(w, samples, W.Internals(wrs.handle, n))
    stream = torch.cuda.current_stream()
    for _ in range(3):
        wrs.build(stream, bufs, n)
        wrs.sample(stream, bufs, n, s, seed=1)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record(stream)
    for _ in range(steps):
        wrs.build(stream, bufs, n)
    e[1].record(stream)
    for _ in range(steps):
        wrs.sample(stream, bufs, n, s, seed=1)
    e[2].record(stream)
    torch.cuda.synchronize()
    build_s = e[0].elapsed_time(e[1]) / steps / 1e3
    sample_s = e[1].elapsed_time(e[2]) / steps / 1e3
    # the same builds with the host out of the loop: 8 builds captured in one CUDA graph
    per_graph = 8
    graph = torch.cuda.CUDAGraph()
    gs = torch.cuda.Stream()
    gs.wait_stream(stream)
    with torch.cuda.graph(graph, stream=gs):
        for _ in range(per_graph):
            wrs.build(torch.cuda.current_stream(), bufs, n)
    graph.replay()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(steps):
        graph.replay()
    e[1].record(stream)
    torch.cuda.synchronize()
    graph_build_s = e[0].elapsed_time(e[1]) / (steps * per_graph) / 1e3
    assert bufs.internals.status() == 0
    st = sample_statistics(W.Statistics(n), samples, s, w, n)  # histogram etc. on the device
    cpu = small_cpu_path(w.cpu().numpy(), samples.cpu().numpy().view(np.uint32), s)
    return {"workload": "plain path, small: N=65,536 uniform(0,1] (seed 1), PSA build (split 2) "
                        "+ S=2^20 Philox4x32-10 samples (seed 1)",
            "builds_per_s": 1.0 / build_s, "samples_per_s": s / sample_s,
            "build_us": build_s * 1e6, "sample_us": sample_s * 1e6,
            "graph_builds_per_s": 1.0 / graph_build_s, "graph_build_us": graph_build_s * 1e6,
            "graph_note": "per-call builds from a Python loop over the C ABI include the host's "
                          "launch gaps; graph_* replays 8 builds captured in one CUDA graph",
            "chi2": st["chi2"], "df": st["df"], "p_value": st["p_value"],
            "z_score": st["z_score"], "z_multinomial": st.get("z_multinomial"),
            "p_value_multinomial": st.get("p_value_multinomial"),
            "rmse": st["rmse"], "rmse_ideal": st["rmse_ideal"],
            "zero_weight_draws": st["zero_weight_draws"], "binned": st["binned"],
            "statistics": "wrs_histogram + wrs_sample_statistics on the device",
            "cpu_baseline": cpu}


def small_cpu_path(w_host, gpu_samples, s: int) -> dict:
    """The small configuration's CPU path on the host: the oracle's port of the PSA build at
    split size 2 (FP32, as the GPU's) and its Philox4x32-10 alias sampler (seed 1), on one
    thread as the reference's CPU code runs; builds/s and samples/s, the chi-square / RMSE of
    its histogram against the weights, and the RMSE between the GPU's and the CPU's normalised
    histograms (the same Philox stream over nearly the same table -- the FP32 prefix sums run
    in different orders, so a few entries differ in their last bits -- hence far below the
    RMSE of two independent draws)."""
    import numpy as np
    from oracle.oracle import RNG_PHILOX4X32_10, Oracle
    orc = Oracle()
    n = w_host.size
    t0 = time.perf_counter()
    table, _, _ = orc.psa_build(w_host, 2, nthreads=1)
    t1 = time.perf_counter()
    cs = orc.alias_sample(table, s, 1, rng=RNG_PHILOX4X32_10, nthreads=1)
    t2 = time.perf_counter()
    p = w_host.astype(np.float64) / float(np.sum(w_host.astype(np.float64)))
    hc = np.bincount(cs, minlength=n).astype(np.float64)
    hg = np.bincount(gpu_samples, minlength=n).astype(np.float64)
    e = p * s
    nz = e > 0
    out = {"kind": "port", "cores": 1,
           "sample": "the whole configuration: one PSA build of the 65,536 weights and all "
                     "2^20 samples, one thread",
           "build_s": t1 - t0, "builds_per_s": 1.0 / (t1 - t0),
           "sample_s": t2 - t1, "samples_per_s": s / (t2 - t1)}
    out.update(chi2_report(float(np.sum((hc[nz] - e[nz]) ** 2 / e[nz])), int(nz.sum()) - 1,
                           multinomial_chi2_var(p, s)))
    out["rmse"] = float(np.sqrt(np.mean((hc / s - p) ** 2)))
    out["rmse_gpu_vs_cpu_histogram"] = float(np.sqrt(np.mean((hg / s - hc / s) ** 2)))
    return out


def multinomial_chi2_var(p, s: int) -> float:
    """The exact variance of Pearson's chi-square over the k cells with p > 0 when s samples are
    drawn from the probabilities p (a numpy array or torch tensor): 2 (k - 1) + (sum 1/p - k^2
    - 2 k + 2) / s; its mean is k - 1 exactly.  Where the expected counts s p are small the
    sum of 1/p dominates, and the chi-square distribution's variance 2 (k - 1) understates the
    statistic's spread many times over."""
    q = p[p > 0]
    k = float(q.shape[0])
    inv = float((1.0 / q).sum())
    return 2.0 * (k - 1.0) + (inv - k * k - 2.0 * k + 2.0) / float(s)


def chi2_report(chi2: float, df: int, var: float | None = None) -> dict:
    """The chi-square statistic with its degrees of freedom, upper-tail p-value (scipy) and the
    reference's z-score (chi2 - df) / sqrt(2 df) (src/host/statistics/chi_square.hpp:11-15).
    With `var`, the statistic's exact multinomial variance (multinomial_chi2_var, summed over
    independent draws), also the z-score against that spread and its normal upper-tail
    p-value: the check that stays valid where items' expected counts are far below 5."""
    try:
        from scipy.stats import chi2 as chi2_dist
        p = float(chi2_dist.sf(chi2, df)) if df > 0 else None
    except ImportError:
        p = None
    out = {"chi2": chi2, "df": df, "p_value": p,
           "z_score": (chi2 - df) / math.sqrt(2.0 * df) if df > 0 else None}
    if var is not None and var > 0 and df > 0:
        z = (chi2 - df) / math.sqrt(var)
        out.update({"z_multinomial": z, "p_value_multinomial": 0.5 * math.erfc(z / math.sqrt(2.0))})
    return out


def binned_chi2(o, e, target: float) -> dict:
    """Chi-square over bins of G consecutive items (device tensors o: observed counts, e:
    expected counts), G the smallest power of two whose mean expected count per bin is at
    least `target`: the chi-square distribution describes the statistic only where expected
    counts are large, which item by item they are not for skewed weights.  Bins with no
    expectation are left out; df = bins - 1."""
    n = int(e.numel())
    mean_e = float(e.sum()) / max(n, 1)
    G = 1
    while G < n and G * mean_e < target:
        G *= 2
    O = bin_sums(o, G)
    E = bin_sums(e, G)
    keep = E > 0
    chi2 = float((((O - E) ** 2)[keep] / E[keep]).sum())
    bins = int(keep.sum())
    total = float(E.sum())
    var = multinomial_chi2_var(E / total, round(total)) if bins > 1 else None
    return {**chi2_report(chi2, bins - 1, var), "bin_items": G,
            "min_expected": float(E[keep].min()) if bins else None}


def bin_sums(x, G: int):
    """Sums of G consecutive entries of the device tensor x (the last bin zero-padded)."""
    import torch
    pad = (-int(x.numel())) % G
    if pad:
        x = torch.cat([x, x.new_zeros(pad)])
    return x.view(-1, G).sum(1)


def p_binned(e, G: int):
    """The bin probabilities of binned_chi2's bins of G items, from expected counts e."""
    E = bin_sums(e, G)
    return E / E.sum()


def sample_statistics(stats, samples, s: int, w, n: int, bin_target: float = 1024.0) -> dict:
    """Statistics of s samples of the n weights w (device tensors): the on-device histogram,
    chi-square and RMSE (wrs_histogram + wrs_sample_statistics) -- the reference's chi_square
    over the items with nonzero expectation (src/host/statistics/chi_square.hpp:17-37), df =
    those items - 1, and its RMSE of the normalised histogram (src/dep/eval/rms.hpp:44-63) --
    with the RMSE a multinomial draw of s samples has in expectation (rmse_ideal), and the
    binned chi-square (binned_chi2), whose p-value holds where items' expected counts are
    small."""
    import torch
    r = stats(None, samples, s, w)
    w64 = w[:n].double()
    total = w64.sum()
    p = w64 / total
    out = chi2_report(r["chi2"], int((w64 > 0).sum()) - 1, multinomial_chi2_var(p, s))
    out.update({"rmse": r["rmse"], "rmse_ideal": float(torch.sqrt(torch.mean(p * (1 - p) / s))),
                "zero_weight_draws": r["zero_weight_draws"],
                "binned": binned_chi2(stats.hist[:n].double(), p * s, bin_target)})
    return out


def host_link_rates(host_s, dev_s, host_w, dev_w, stream) -> dict:
    """Pinned host <-> device copy rates (cudaMemcpyAsync, CUDA events, 3 copies each after
    one warm-up): the bound of the end-to-end figure, which moves 4 B per sample off the
    device and 4 B per weight onto it every step."""
    import torch
    out = {}
    for name, dst, src in (("d2h_GBs", host_s, dev_s), ("h2d_GBs", dev_w, host_w)):
        dst.copy_(src, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = 3 * src.numel() * src.element_size() / (e0.elapsed_time(e1) / 1e3) / 1e9
    out["e2e_bound_samples_per_s"] = out["d2h_GBs"] * 1e9 / 4.0
    return out


def random_gather_rate(W, internals, n: int, s: int, stream) -> float:
    """Random 8-byte gathers per second from the alias table itself (wrs_probe_random_gather),
    mean of 3 timed launches of s gathers after 2 warm-up launches."""
    import torch
    sink = torch.zeros(1, dtype=torch.int32, device="cuda")
    table = internals.views()["alias_table"]

    def launch():
        W.check(W.lib().wrs_probe_random_gather(stream.cuda_stream, table, 8 * n, s, 8,
                                                sink.data_ptr()))

    for _ in range(2):
        launch()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        launch()
    e1.record(stream)
    torch.cuda.synchronize()
    return s / (e0.elapsed_time(e1) / 3 / 1e3)


def _timed(stream, fn, reps: int = 5) -> float:
    """Seconds per call of fn: CUDA events on `stream` around reps calls after 2 warm-up
    calls."""
    import torch
    for _ in range(2):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps / 1e3


def per_distribution(W, wrs, internals, weights, samples, n: int, s: int, stream,
                     peak: float) -> dict:
    """The single large distribution on each of its three shapes: the headline step's PSA
    build and alias sampling, the decoupled scan (exact and FP32 carries), ITS (build = scan +
    cell blocks; compensated CMF, and the FP32 CMF of the reference's precision) and Cutpoint
    (entry 128, compensated CMF), each timed alone (CUDA events, mean of 5 calls after 2
    warm-up calls), with the statistics of the alias and ITS samples against the weights."""
    import torch
    stats = W.Statistics(n)
    its = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=W.SCAN_COMPENSATED))
    its32 = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10))
    cp = W.WRS(W.CutpointConfig(128, rng=W.RNG_PHILOX4X32_10,
                                scan_precision=W.SCAN_COMPENSATED))
    its_int, its32_int, cp_int = (W.Internals(h.handle, n) for h in (its, its32, cp))
    cmf = torch.empty(n, dtype=torch.float32, device=weights[0].device)
    out = {}
    for d, name in enumerate(DISTS):
        w = weights[d]
        row = {}
        ab = W.WRSBuffers(w, samples, internals)
        row["alias_build_ms"] = _timed(stream, lambda: wrs.build(stream, ab, n)) * 1e3
        row["alias_builds_per_s"] = 1e3 / row["alias_build_ms"]
        row["alias_build_frac"] = 32.0 * n / (row["alias_build_ms"] / 1e3) / 1e9 / peak
        row["alias_sample_ms"] = _timed(stream, lambda: wrs.sample(stream, ab, n, s,
                                                                   seed=1234 + d)) * 1e3
        row["alias_samples_per_s"] = s / (row["alias_sample_ms"] / 1e3)
        row["alias_statistics"] = sample_statistics(stats, samples, s, w, n)
        for key, h, hi in (("scan", its, its_int), ("scan_fp32", its32, its32_int)):
            sec = _timed(stream, lambda: h.prefix_sum(stream, w, n, cmf, hi))
            row[f"{key}_ms"] = sec * 1e3
            row[f"{key}_weights_per_s"] = n / sec
            row[f"{key}_frac"] = 8.0 * n / sec / 1e9 / peak
        for key, h, hi in (("its", its, its_int), ("its_fp32", its32, its32_int),
                           ("cutpoint", cp, cp_int)):
            b = W.WRSBuffers(w, samples, hi)
            row[f"{key}_build_ms"] = _timed(stream, lambda: h.build(stream, b, n)) * 1e3
            sec = _timed(stream, lambda: h.sample(stream, b, n, s, seed=99))
            row[f"{key}_sample_ms"] = sec * 1e3
            row[f"{key}_samples_per_s"] = s / sec
            if key == "its":
                row["its_statistics"] = sample_statistics(stats, samples, s, w, n)
        for hi in (internals, its_int, its32_int, cp_int):
            assert not hi.status() & W.DEVICE_TIMEOUT
        out[name] = row
    return out


def kernel_breakdown(W, pkg, wrs, internals, weights, samples, n, s, stream, peak, args):
    """Each kernel of the path timed alone (CUDA events, mean of 5 launches after 2 warm-up
    launches) with its algorithmic bytes."""
    import torch
    v = internals.views()
    reps = 5
    out = {}

    def timed(fn):
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    w = weights[0]
    idx, prefix, elems, table, lo = (v["partition_indices"], v["partition_prefix"],
                                     v["partition_elements"], v["alias_table"],
                                     v["partition_prefix_lo"])

    def rec(name, sec, nbytes, units, unit_name):
        out[name] = {"ms": sec * 1e3, "GB/s": nbytes / sec / 1e9, "frac": nbytes / sec / 1e9 / peak,
                     f"{unit_name}/s": units / sec, "bytes_per_unit": nbytes / units}

    rec("total_mass", timed(lambda: wrs.total_mass(stream, w, n, internals)), 4 * n, n, "weights")
    # read w 4 + write index 4 + prefix 4 + element 4 + prefix low word 4
    rec("prefix_partition",
        timed(lambda: wrs.prefix_partition(stream, w, n, idx, prefix, elems, internals, lo)),
        20 * n, n, "weights")
    # the FP32-carry partition, decoupled lookback against the block-wise (reduce-then-scan)
    # baseline, which reads the weights twice (24 B / weight against 16)
    fp32 = W.WRS(dataclasses.replace(wrs.config, scan_precision=W.SCAN_FP32))
    rec("prefix_partition_fp32",
        timed(lambda: fp32.prefix_partition(stream, w, n, idx, prefix, elems, internals)),
        16 * n, n, "weights")
    rec("prefix_partition_blockwise",
        timed(lambda: fp32.prefix_partition_blockwise(stream, w, n, idx, prefix, elems,
                                                      internals)), 16 * n, n, "weights")
    wrs.prefix_partition(stream, w, n, idx, prefix, elems, internals, lo)  # the FF arrays again
    # read index 4 + element 4 + write entry 8 (split probes assumed L2-resident)
    rec("split_pack",
        timed(lambda: wrs.split_pack(stream, w, idx, prefix, elems, n, table, internals, lo)),
        16 * n, n, "weights")
    rec("alias_sample",
        timed(lambda: wrs.alias_sample(stream, table, n, s, 99, 0, samples)), 12 * s, s,
        "samples")
    # the same draws through the buffers after a build, i.e. with the table's coin filter
    ab = W.WRSBuffers(w, samples, internals)
    wrs.build(stream, ab, n)
    rec("alias_sample_coin_filter",
        timed(lambda: wrs.sample(stream, ab, n, s, seed=99)), 12 * s, s, "samples")
    # serial split-pack (split records + pack from them), the two pack strategies, against the
    # inline split-pack at the same split size
    serial = {}
    records = torch.empty(3 * (n // 2 + 1), dtype=torch.int32, device=w.device)
    for split in (SPLIT_SIZE, 256, 1024):
        row = {}
        for name, mode in (("inline", W.SPLITPACK_INLINE), ("scalar", W.SPLITPACK_SERIAL),
                           ("warp", W.SPLITPACK_SERIAL_SUBGROUP)):
            h = W.WRS(dataclasses.replace(wrs.config, split_size=split, split_pack_mode=mode))
            if mode == W.SPLITPACK_INLINE:
                row[name] = timed(lambda: h.split_pack(stream, w, idx, prefix, elems, n, table,
                                                       internals, lo)) * 1e3
            else:
                row["split_records"] = timed(lambda: h.split(stream, prefix, n, records,
                                                             internals, prefix_lo=lo)) * 1e3
                row[name] = timed(lambda: h.pack(stream, w, idx, elems, records, n, table,
                                                 internals)) * 1e3
        serial[split] = row
    out["split_pack_modes_ms"] = serial
    wrs.split_pack(stream, w, idx, prefix, elems, n, table, internals, lo)  # the inline table
    its = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=W.SCAN_COMPENSATED))
    cmf = torch.empty(n, dtype=torch.float32, device=w.device)
    rec("scan", timed(lambda: its.prefix_sum(stream, w, n, cmf, internals)), 8 * n, n, "weights")
    its32 = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10))
    rec("scan_fp32", timed(lambda: its32.prefix_sum(stream, w, n, cmf, internals)), 8 * n, n,
        "weights")
    rec("scan_blockwise", timed(lambda: its32.prefix_sum_blockwise(stream, w, n, cmf, internals)),
        8 * n, n, "weights")
    rec("its_sample", timed(lambda: its.its_sample(stream, cmf, n, s, 99, 0, samples)), 4 * s, s,
        "samples")
    # FP32 ITS through the buffers API (the same samples as its_sample on that CMF): with cell
    # size 0 the build stores the probe tree as blocks and the tree sampler reads them; with
    # the default cell size 4 the build also makes the cells and marks those the FP32 CMF's
    # decreases can reach, the cell search serves the others and the marked ones bisect
    tree32 = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10, guiding_entry_size=0))
    bufs32 = W.WRSBuffers(w, samples, W.Internals(tree32.handle, n))
    rec("its_build_fp32", timed(lambda: tree32.build(stream, bufs32, n)), 8 * n, n,
        "weights")
    rec("its_sample_stored_levels",
        timed(lambda: tree32.sample(stream, bufs32, n, s, seed=99)), 4 * s, s, "samples")
    del bufs32
    bufs32 = W.WRSBuffers(w, samples, W.Internals(its32.handle, n))
    rec("its_build_fp32_cells", timed(lambda: its32.build(stream, bufs32, n)), 8 * n, n,
        "weights")
    rec("its_sample_fp32_cells", timed(lambda: its32.sample(stream, bufs32, n, s, seed=99)),
        4 * s, s, "samples")
    del bufs32
    # through the buffers API: the compensated build also makes the guiding table, and
    # sampling runs the guided search (same samples as the bisection)
    its_bufs = W.WRSBuffers(w, samples, W.Internals(its.handle, n))
    rec("its_build", timed(lambda: its.build(stream, its_bufs, n)), 8 * n, n, "weights")
    rec("its_sample_cells", timed(lambda: its.sample(stream, its_bufs, n, s, seed=99)), 4 * s,
        s, "samples")
    # the ITS sector model: the 4-byte output plus one 32-byte sector per bisection level
    # whose probes fall outside L2, ceil(log2(4 N / L2 bytes)) levels; the cell-block search
    # reads one random 32-byte block instead
    l2 = getattr(torch.cuda.get_device_properties(w.device), "L2_cache_size", 126 << 20)
    outside = max(0, math.ceil(math.log2(4 * n / l2)))
    for name, b in (("its_sample", 4 + 32 * outside),
                    ("its_sample_stored_levels", 4 + 32 * outside),
                    ("its_sample_fp32_cells", 4 + 32),
                    ("its_sample_cells", 4 + 32)):
        sec = out[name]["ms"] / 1e3
        out[name]["sector_model"] = {"bytes_per_sample": b, "levels_outside_l2": outside,
                                     "GB/s": b * s / sec / 1e9, "frac": b * s / sec / 1e9 / peak}
    # guiding-table granularity of the guided search: build (scan + table) and sampling time
    sweep = {}
    for entry in (2, 3, 4, 6, 8):
        h = W.WRS(W.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=W.SCAN_COMPENSATED,
                              guiding_entry_size=entry))
        bufs = W.WRSBuffers(w, samples, W.Internals(h.handle, n))
        sweep[entry] = {"build_ms": timed(lambda: h.build(stream, bufs, n)) * 1e3,
                        "sample_ms": timed(lambda: h.sample(stream, bufs, n, s, seed=99)) * 1e3}
    out["its_guide_entry_sweep"] = sweep
    cp = W.WRS(W.CutpointConfig(128))
    G = (n + 127) // 128
    guide = torch.empty(G, dtype=torch.int32, device=w.device)
    # guiding table: one lower-bound search per entry (reads ~1 sector per level, writes 4 B)
    rec("cutpoint_guide", timed(lambda: cp.cutpoint_guide(stream, cmf, n, guide)), 4 * G, G,
        "entries")
    rec("cutpoint_sample",
        timed(lambda: cp.cutpoint_sample(stream, cmf, n, guide, s, 99, 0, samples)), 4 * s, s,
        "samples")
    # the reference's PRNG operator (wrs_philox): S uniform floats into the samples buffer,
    # 4 B written per element
    prng = W.PRNG()
    floats = samples.view(torch.float32)
    rec("philox_uniform", timed(lambda: prng.run(stream, floats, s, 7)), 4 * s, s, "elements")
    assert not internals.status() & W.DEVICE_TIMEOUT
    return out


if __name__ == "__main__":
    main()
