"""GPU tests of the autotuner (wrs_autotune_alias / wrs_autotune_batch) and of the L2
fetch-granularity knob it tunes.

Bar: the tuner returns one of its candidates with positive timings and the trial count its
coordinate search implies, leaves the context's L2 limit at the chosen value, and the knob
changes no result: tables and samples are bit-for-bit the same under every L2 setting, and
a build with the tuned split size matches the oracle as any other split size does.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform, weights_zipf
from gpu_util import d2h, h2d, t2h
from oracle.oracle import ENTRY_DTYPE
from test_gpu_parity import Built, same_table

pytestmark = pytest.mark.gpu


def _cfg(pkg, split):
    W = pkg.wrs
    return pkg.AliasTableConfig(split_size=split, rng=W.RNG_PHILOX4X32_10,
                                scan_precision=W.SCAN_FLOAT_FLOAT, split_residual_f64=True,
                                split_full_light=True)


def _build_sample(pkg, cfg, w, S, seed):
    W = pkg.wrs
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(w.size, S, cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, w.size)
    wrs.sample(None, bufs, w.size, S, seed)
    assert bufs.internals.status() == 0
    tab = d2h(W.lib().wrs_buffers_alias_table(bufs.internals.ptr), w.size, ENTRY_DTYPE)
    return tab, t2h(bufs.samples, np.uint32)[:S]


def test_autotune_alias_returns_a_measured_candidate(pkg, cuda, oracle):
    import torch
    W = pkg.wrs
    n, S = 1 << 20, 1 << 22
    w = weights_lognormal(n, 31)
    dw = h2d(w)
    out = torch.zeros(S, dtype=torch.int32, device="cuda")
    before = W.get_l2_fetch_granularity()
    try:
        r = W.autotune_alias(_cfg(pkg, 8), None, dw, n, S, out, split_sizes=[4, 8, 12],
                             l2_fetch=[64, 128], warmup=1, reps=2)
        # 2 L2 candidates at split 8, then splits 4 and 12 at the best L2 value
        assert len(r["trials"]) == 4
        assert r["split_size"] in (4, 8, 12) and r["l2_fetch"] in (64, 128)
        assert all(t["build_ms"] > 0 and t["sample_ms"] > 0 for t in r["trials"])
        best = min(t["build_ms"] + t["sample_ms"] for t in r["trials"])
        assert r["build_ms"] + r["sample_ms"] == pytest.approx(best)
        assert W.get_l2_fetch_granularity() == r["l2_fetch"]
        # the tuned configuration builds the oracle's table
        b = Built(pkg, w, _cfg(pkg, r["split_size"]))
        assert b.status == 0
        ref = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, r["split_size"], flags=3,
                             elems=b.elems, prefix_lo=b.prefix_lo, mean64=b.mean64)
        assert same_table(b.table, ref)
    finally:
        W.set_l2_fetch_granularity(before)


def test_autotune_build_only_and_fixed_split(pkg, cuda):
    W = pkg.wrs
    n = 300_000
    dw = h2d(weights_uniform(n, 32))
    before = W.get_l2_fetch_granularity()
    try:
        r = W.autotune_alias(_cfg(pkg, 12), None, dw, n, 0, None, split_sizes=[],
                             l2_fetch=[], warmup=1, reps=1)
        assert len(r["trials"]) == 1 and r["split_size"] == 12 and r["l2_fetch"] == 0
        assert r["sample_ms"] >= 0 and r["build_ms"] > 0
        assert W.get_l2_fetch_granularity() == before  # not tuned, not touched
    finally:
        W.set_l2_fetch_granularity(before)


@pytest.mark.parametrize("gran", [32, 64, 128])
def test_l2_fetch_granularity_changes_no_result(pkg, cuda, gran):
    W = pkg.wrs
    n, S = 1 << 21, 1 << 22
    w = weights_zipf(n, 33)
    before = W.get_l2_fetch_granularity()
    try:
        W.set_l2_fetch_granularity(128)
        tab0, smp0 = _build_sample(pkg, _cfg(pkg, 12), w, S, 5)
        W.set_l2_fetch_granularity(gran)
        assert W.get_l2_fetch_granularity() == gran
        tab1, smp1 = _build_sample(pkg, _cfg(pkg, 12), w, S, 5)
    finally:
        W.set_l2_fetch_granularity(before)
    assert np.array_equal(tab0.view(np.uint64), tab1.view(np.uint64))
    assert np.array_equal(smp0, smp1)


def test_autotune_batch_then_batch_matches_per_call(pkg, cuda):
    import torch
    W = pkg.wrs
    sizes = [64, 4097, 70001, 300000, 1 << 20]
    gens = (weights_uniform, weights_zipf, weights_lognormal)
    ws = [gens[k % 3](n, 40 + k) for k, n in enumerate(sizes)]
    dws = [h2d(w) for w in ws]
    tabs = [torch.zeros(2 * n, dtype=torch.int32, device="cuda") for n in sizes]
    counts = [max(1, n // 4) for n in sizes]
    outs = [torch.zeros(s, dtype=torch.int32, device="cuda") for s in counts]
    dists = [(dws[k], tabs[k], outs[k], sizes[k], counts[k], 7 + k) for k in range(len(sizes))]
    before = W.get_l2_fetch_granularity()
    try:
        r = W.autotune_batch(_cfg(pkg, 8), None, dists, split_sizes=[6, 8, 16],
                             l2_fetch=[64], warmup=1, reps=1)
        assert len(r["trials"]) == 3 and r["split_size"] in (6, 8, 16)
        cfg = _cfg(pkg, r["split_size"])
        b = W.Batch(W.Handle(cfg), len(sizes), sum(sizes), sum(counts))
        b.set(None, dists)
        b.build(None)
        b.sample(None)
        assert b.status() == 0
        for k in range(len(sizes)):
            tab, smp = _build_sample(pkg, cfg, ws[k], counts[k], 7 + k)
            got = t2h(tabs[k], np.uint32).view(ENTRY_DTYPE)
            assert np.array_equal(got.view(np.uint64), tab.view(np.uint64)), sizes[k]
            assert np.array_equal(t2h(outs[k], np.uint32)[:counts[k]], smp), sizes[k]
    finally:
        W.set_l2_fetch_granularity(before)
