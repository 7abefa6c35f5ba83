"""GPU tests of the batched path (wrs_batch_*): many distributions built and sampled with
one launch per stage.

Bar: in the compensated precisions every distribution's alias table and samples are
bit-for-bit those of a per-call wrs_build + wrs_sample on the same weights, seed and
configuration, whatever else the batch holds; tables built in a batch also encode the
weights (implied distribution vs w / mean) as the per-call path does.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform, weights_zipf
from gpu_util import h2d, t2h
from oracle.oracle import ENTRY_DTYPE

pytestmark = pytest.mark.gpu

SIZES = [64, 100, 4095, 4096, 4097, 12289, 70001, 300000, 1 << 20]


def _configs(pkg):
    W = pkg.wrs
    return {
        "ff-philox-s8": pkg.AliasTableConfig(split_size=8, rng=W.RNG_PHILOX4X32_10,
                                             scan_precision=W.SCAN_FLOAT_FLOAT,
                                             split_residual_f64=True, split_full_light=True),
        "comp-ref-s2": pkg.AliasTableConfig(split_size=2, scan_precision=W.SCAN_COMPENSATED),
        "comp-ref-s32-gather": pkg.AliasTableConfig(split_size=32,
                                                    scan_precision=W.SCAN_COMPENSATED,
                                                    use_partition_elements=False,
                                                    split_full_light=True),
    }


def _weights(k: int, n: int) -> np.ndarray:
    g = (weights_uniform, weights_zipf, weights_lognormal)[k % 3]
    return g(n, 100 + k)


class Case:
    """Distributions in device memory: weights, tables and sample buffers."""

    def __init__(self, sizes, seeds, counts):
        import torch
        self.sizes = list(sizes)
        self.w = [_weights(k, n) for k, n in enumerate(self.sizes)]
        self.dw = [h2d(w) for w in self.w]
        self.tables = [torch.zeros(2 * n, dtype=torch.int32, device="cuda") for n in self.sizes]
        self.out = [torch.zeros(max(1, s), dtype=torch.int32, device="cuda") for s in counts]
        self.seeds = list(seeds)
        self.counts = list(counts)

    def descs(self, which=None, build=True, sample=True):
        which = range(len(self.sizes)) if which is None else which
        return [(self.dw[k] if build else None, self.tables[k], self.out[k] if sample else None,
                 self.sizes[k], self.counts[k] if sample else 0, self.seeds[k]) for k in which]

    def table(self, k):
        return t2h(self.tables[k], np.uint32).view(ENTRY_DTYPE)

    def samples(self, k):
        return t2h(self.out[k], np.uint32)[: self.counts[k]]


def _per_call(pkg, cfg, w, S, seed):
    W = pkg.wrs
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(w.size, max(1, S), cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, w.size)
    if S:
        wrs.sample(None, bufs, w.size, S, seed)
    assert bufs.internals.status() == 0
    tab = W.lib().wrs_buffers_alias_table(bufs.internals.ptr)
    from gpu_util import d2h
    return d2h(tab, w.size, ENTRY_DTYPE), t2h(bufs.samples, np.uint32)[:S]


@pytest.mark.parametrize("name", ["ff-philox-s8", "comp-ref-s2", "comp-ref-s32-gather"])
def test_batch_matches_per_call(pkg, cuda, name):
    """Tables and samples of a mixed-size batch equal per-call builds bit for bit."""
    cfg = _configs(pkg)[name]
    W = pkg.wrs
    counts = [3 * n + 5 for n in SIZES]
    case = Case(SIZES, [7 + k for k in range(len(SIZES))], counts)
    h = W.Handle(cfg)
    batch = W.Batch(h, 64, sum(SIZES), sum(counts))
    batch.set(None, case.descs())
    assert batch.count() == len(SIZES)
    batch.build(None)
    batch.sample(None)
    assert batch.status() == 0
    for k, n in enumerate(SIZES):
        tab, smp = _per_call(pkg, cfg, case.w[k], counts[k], case.seeds[k])
        assert np.array_equal(case.table(k).view(np.uint32), tab.view(np.uint32)), (name, n)
        assert np.array_equal(case.samples(k), smp), (name, n)


def test_batch_alone_equals_in_mix(pkg, cuda):
    """Each distribution built and sampled alone in a batch equals the same distribution
    inside a batch of all of them (the serving loop's equality)."""
    import torch
    cfg = _configs(pkg)["ff-philox-s8"]
    W = pkg.wrs
    sizes = [4097, 64, 250000, 9000, 1 << 19]
    counts = [1000, 1, 70000, 4096, 12345]
    mix = Case(sizes, [3, 1, 4, 1, 5], counts)
    h = W.Handle(cfg)
    batch = W.Batch(h, 16, sum(sizes), sum(counts))
    batch.set(None, mix.descs())
    batch.build(None)
    batch.sample(None)
    assert batch.status() == 0
    alone = Case(sizes, [3, 1, 4, 1, 5], counts)
    for k in range(len(sizes)):
        batch.set(None, alone.descs([k]))
        batch.build(None)
        batch.sample(None)
    assert batch.status() == 0
    torch.cuda.synchronize()
    for k in range(len(sizes)):
        assert np.array_equal(mix.table(k).view(np.uint32), alone.table(k).view(np.uint32))
        assert np.array_equal(mix.samples(k), alone.samples(k))


def test_batch_sample_only_and_build_only(pkg, cuda):
    """A distribution with no weights samples its resident table; one with no samples only
    builds; both in one batch with an ordinary one."""
    cfg = _configs(pkg)["ff-philox-s8"]
    W = pkg.wrs
    sizes = [5000, 20000, 777]
    counts = [4000, 0, 999]
    case = Case(sizes, [11, 12, 13], counts)
    h = W.Handle(cfg)
    batch = W.Batch(h, 8, sum(sizes), sum(counts) + 10000)
    batch.set(None, case.descs())
    batch.build(None)
    batch.sample(None)
    first = [case.table(k) for k in range(3)]
    # resample distribution 0 only (table resident, no rebuild) with another seed, and
    # rebuild distribution 1 without sampling
    descs = case.descs()
    descs[0] = (None, case.tables[0], case.out[0], sizes[0], counts[0], 99)
    descs[1] = (case.dw[1], case.tables[1], None, sizes[1], 0, 12)
    batch.set(None, descs[:2])
    assert batch.count() == 2
    batch.build(None)
    batch.sample(None)
    assert batch.status() == 0
    assert np.array_equal(case.table(1).view(np.uint32), first[1].view(np.uint32))
    _, smp = _per_call(pkg, cfg, case.w[0], counts[0], 99)
    assert np.array_equal(case.samples(0), smp)


def test_batch_graph_replay(pkg, cuda):
    """wrs_batch_build + wrs_batch_sample captured once into a CUDA graph: every replay
    reproduces the eager result (the lookback and mass counters clean up after themselves)."""
    import torch
    cfg = _configs(pkg)["ff-philox-s8"]
    W = pkg.wrs
    sizes = [64, 4097, 100000, 33333, 1 << 18]
    counts = [64, 5000, 200000, 1, 300000]
    case = Case(sizes, [21, 22, 23, 24, 25], counts)
    h = W.Handle(cfg)
    batch = W.Batch(h, 8, sum(sizes), sum(counts))
    batch.set(None, case.descs())
    batch.build(None)
    batch.sample(None)
    assert batch.status() == 0
    ref_t = [case.table(k).copy() for k in range(len(sizes))]
    ref_s = [case.samples(k).copy() for k in range(len(sizes))]
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        batch.build(torch.cuda.current_stream())
        batch.sample(torch.cuda.current_stream())
    for rep in range(3):
        for t in case.tables + case.out:
            t.zero_()
        g.replay()
        torch.cuda.synchronize()
        for k in range(len(sizes)):
            assert np.array_equal(case.table(k).view(np.uint32), ref_t[k].view(np.uint32)), rep
            assert np.array_equal(case.samples(k), ref_s[k]), rep
    assert batch.status() == 0


def test_batch_tables_encode_weights(pkg, cuda, oracle):
    """Batched tables encode their weights: the implied distribution matches w / mean to
    the per-call float-float path's bound (1e-3 mean units)."""
    cfg = _configs(pkg)["ff-philox-s8"]
    W = pkg.wrs
    sizes = [64, 4096, 50000, 1 << 20]
    case = Case(sizes, [1, 2, 3, 4], [0, 0, 0, 0])
    h = W.Handle(cfg)
    batch = W.Batch(h, 8, sum(sizes), 1)
    batch.set(None, case.descs(sample=False))
    batch.build(None)
    assert batch.status() == 0
    for k, n in enumerate(sizes):
        w = case.w[k]
        implied = oracle.alias_to_weights(case.table(k))
        target = w / w.astype(np.float64).mean()
        assert np.all(np.abs(implied - target) <= 1e-3 + 1e-7 * target), n


def test_batch_argument_checks(pkg, cuda):
    W = pkg.wrs
    h = W.Handle(pkg.AliasTableConfig())
    batch = W.Batch(h, 2, 10000, 10000)
    dw = h2d(weights_uniform(6000, 1))
    import torch
    t = torch.zeros(2 * 6000, dtype=torch.int32, device="cuda")
    with pytest.raises(W.WRSError) as e:  # three distributions > max_dists
        batch.set(None, [(dw, t, None, 10, 0, 1)] * 3)
    assert e.value.status == 6
    with pytest.raises(W.WRSError) as e:  # weights beyond max_weights
        batch.set(None, [(dw, t, None, 6000, 0, 1), (dw, t, None, 6000, 0, 1)])
    assert e.value.status == 6
    with pytest.raises(W.WRSError) as e:  # s > 0 without a sample buffer
        batch.set(None, [(dw, t, None, 6000, 5, 1)])
    assert e.value.status == 1
    other = W.Handle(pkg.AliasTableConfig(split_size=4))  # not the batch's split size
    assert W.lib().wrs_batch_build(other.ptr, None, batch.ptr) == 1
    its = W.Handle(pkg.ITSConfig())
    assert W.lib().wrs_batch_sample(its.ptr, None, batch.ptr) == 5  # alias method only
