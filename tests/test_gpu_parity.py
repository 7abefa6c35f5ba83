"""GPU parity tests: the CUDA path, driven through the C ABI, against the oracle.

Bar (stated per test):
  * integer / index outputs -- partition indices, heavy count, split points, alias indices
    and samples -- are bit-exact against the oracle given the same upstream values (the
    GPU's own mean, partition prefix, alias table or CMF, as "given the same scanned
    weights" in the reference's test strategy);
  * FP32 values computed by the same operations (alias probabilities p) are bit-exact too;
  * scans and the total mass are within stated relative tolerances of an FP64 oracle.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import (weights_lognormal, weights_precision, weights_uniform, weights_zipf)
from gpu_util import d2h, empty, h2d, t2h
from oracle.oracle import ENTRY_DTYPE, RNG_PHILOX4X32_10, RNG_REFERENCE

pytestmark = pytest.mark.gpu

GENS = {"uniform": weights_uniform, "zipf": weights_zipf, "lognormal": weights_lognormal}
EDGE_N = [1, 2, 3, 31, 32, 33, 4095, 4096, 4097]


class Built:
    """wrs_build through the public API, with the internals read back."""

    def __init__(self, pkg, w: np.ndarray, cfg):
        W = pkg.wrs
        self.wrs = W.WRS(cfg)
        self.N = w.size
        self.buffers = W.WRSBuffers.allocate(self.N, 1, cfg, handle=self.wrs.handle)
        self.buffers.weights.copy_(h2d(w))
        self.wrs.build(None, self.buffers, self.N)
        v = self.buffers.internals.views()
        self.status = self.buffers.internals.status()
        if cfg.method == W.METHOD_ALIAS_TABLE:
            self.mean = float(d2h(v["mean"], 1, np.float32)[0])
            self.total = float(d2h(v["total"], 1, np.float64)[0])
            self.mean64 = float(d2h(v["mean64"], 1, np.float64)[0])
            self.hc = int(d2h(v["heavy_count"], 1, np.uint32)[0])
            self.idx = d2h(v["partition_indices"], self.N, np.uint32)
            self.prefix = d2h(v["partition_prefix"], self.N, np.float32)
            self.elems = (d2h(v["partition_elements"], self.N, np.float32)
                          if cfg.use_partition_elements else None)
            self.prefix_lo = (d2h(v["partition_prefix_lo"], self.N, np.float32)
                              if cfg.scan_precision == W.SCAN_FLOAT_FLOAT else None)
            self.table = d2h(v["alias_table"], self.N, ENTRY_DTYPE)
        else:
            self.cmf = d2h(v["cmf"], self.N, np.float32)

    def sample(self, S, seed, offset=0):
        import torch
        out = torch.empty(S, dtype=torch.int32, device="cuda")
        self.buffers.samples = out
        self.wrs.sample(None, self.buffers, self.N, S, seed, offset=offset)
        return t2h(out, np.uint32)


def same_table(a: np.ndarray, b: np.ndarray) -> bool:
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


# ------------------------------------------------------------------ total mass ---

@pytest.mark.parametrize("N", [1, 5, 4097, 1 << 20, (1 << 22) + 3])
@pytest.mark.parametrize("gen", ["uniform", "lognormal"])
def test_total_mass(pkg, cuda, oracle, N, gen):
    """FP64 total mass: relative error <= 1e-12 against a sequential FP64 sum; the mean
    (rounded once to FP32) equals the oracle's."""
    w = GENS[gen](N, N)
    b = Built(pkg, w, pkg.AliasTableConfig())
    ref = oracle.total_mass(w)
    assert abs(b.total - ref) <= 1e-12 * ref
    assert np.float32(b.mean) == np.float32(oracle.mean(w))


def test_total_mass_unaligned_view(pkg, cuda, oracle):
    """A weights pointer that is not 16-byte aligned (a view into a larger array)."""
    W = pkg.wrs
    w = weights_uniform(100003, 1)
    dw = h2d(w)
    wrs = W.WRS(pkg.AliasTableConfig())
    internals = W.Internals(wrs.handle, w.size)
    wrs.total_mass(None, dw[1:], w.size - 1, internals)
    total = d2h(internals.views()["total"], 1, np.float64)[0]
    assert abs(total - oracle.total_mass(w[1:])) <= 1e-12 * total


# ------------------------------------------------------------- prefix partition ---

@pytest.mark.parametrize("N", EDGE_N + [65536, (1 << 20) + 77])
@pytest.mark.parametrize("gen", list(GENS))
@pytest.mark.parametrize("comp", [False, True])
def test_prefix_partition(pkg, cuda, oracle, N, gen, comp):
    """Partition indices, elements and heavy count bit-exact against the stable partition
    of shader.comp:329-361 at the GPU's mean; heavy / light prefixes within 1e-6
    (compensated carry) or 1e-4 (FP32 carry) relative to the FP64 prefix."""
    w = GENS[gen](N, 7 * N + 1)
    cfg = pkg.AliasTableConfig(scan_precision=1 if comp else 0)
    b = Built(pkg, w, cfg)
    assert b.status == 0
    idx, elems, hc = oracle.partition(w, b.mean)
    assert b.hc == hc
    assert np.array_equal(b.idx, idx)
    assert np.array_equal(b.elems.view(np.uint32), elems.view(np.uint32))
    ref = oracle.partition_prefix_f64(w, b.mean)
    err = np.abs(b.prefix.astype(np.float64) - ref) / np.maximum(np.abs(ref), 1e-30)
    assert err.max() <= (1e-6 if comp else 1e-4), err.max()


# --------------------------------------------------------------- split + pack ---

@pytest.mark.parametrize("split_size", [1, 2, 3, 16, 24, 32])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
@pytest.mark.parametrize("gen", list(GENS))
def test_split_pack_bit_exact(pkg, cuda, oracle, split_size, flags, gen):
    """The GPU alias table equals the oracle's split+pack (shader.comp:81-223) fed the GPU's
    own partition, prefix, heavy count and mean: p bits and alias indices identical (split
    sizes up to 24 stage their walks in shared memory sized by the split size; 32 writes its
    entries directly)."""
    N = 65536 + 123
    w = GENS[gen](N, split_size * 10 + flags)
    cfg = pkg.AliasTableConfig(split_size=split_size, split_residual_f64=bool(flags & 1),
                               split_full_light=bool(flags & 2))
    b = Built(pkg, w, cfg)
    assert b.status == 0
    ref = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, split_size, flags=flags,
                            elems=b.elems)
    assert same_table(b.table, ref)


@pytest.mark.parametrize("N", [(1 << 20) + 5, (1 << 22) + 17])
@pytest.mark.parametrize("gen", list(GENS))
@pytest.mark.parametrize("split_size", [2, 16, 32])
def test_float_float_prefix_mode(pkg, cuda, oracle, N, gen, split_size):
    """WRS_SCAN_FLOAT_FLOAT: high + low words of the partition prefix carry only the
    tile-local FP32 rounding (<= 4096 * max w * 2^-20 absolute), the table equals the oracle's
    float-float split+pack given the GPU's arrays, no overlap escapes the ownership window,
    and the table encodes w/mean to 1e-3 (FP32 prefixes alone give ~1e-2 at 2^20 and whole
    mean-units at 2^26)."""
    W = pkg.wrs
    w = GENS[gen](N, 5 * split_size)
    cfg = pkg.AliasTableConfig(split_size=split_size, scan_precision=W.SCAN_FLOAT_FLOAT,
                               split_full_light=True)
    b = Built(pkg, w, cfg)
    assert b.status == 0
    ref64 = oracle.partition_prefix_f64(w, b.mean)
    got64 = b.prefix.astype(np.float64) + b.prefix_lo.astype(np.float64)
    assert np.abs(got64 - ref64).max() <= 4096 * float(w.max()) * 2.0 ** -20
    assert b.mean64 == b.total / N
    ref = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, split_size, flags=2,
                            elems=b.elems, prefix_lo=b.prefix_lo, mean64=b.mean64)
    assert same_table(b.table, ref)
    implied = oracle.alias_to_weights(b.table)
    target = w / w.astype(np.float64).mean()
    assert np.all(np.abs(implied - target) <= 1e-3 + 1e-7 * target)


@pytest.mark.parametrize("gen", list(GENS))
@pytest.mark.parametrize("comp", [False, True])
def test_split_pack_overlapping_subproblems(pkg, cuda, oracle, gen, comp):
    """At N ~ 2^22 with split size 2, FP32 rounding makes some splits step back so that two
    subproblems pack the same items; the table still equals the oracle's sequential
    subproblem order (the later subproblem's write stands) and no unresolved overlap is
    reported."""
    N = (1 << 22) + 17
    w = GENS[gen](N, 99)
    b = Built(pkg, w, pkg.AliasTableConfig(scan_precision=1 if comp else 0))
    assert b.status == 0
    ref, (si, sj, _) = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, 2, elems=b.elems,
                                         return_splits=True)
    steps_back = np.count_nonzero((np.diff(si.astype(np.int64)) < 0) |
                                  (np.diff(sj.astype(np.int64)) < 0))
    assert same_table(b.table, ref), f"{steps_back} splits step back"


@pytest.mark.parametrize("use_elems", [False, True])
def test_split_pack_partition_elements_switch(pkg, cuda, oracle, use_elems):
    """PSAConfig::usePartitionElements changes where pack reads weights, not the result."""
    w = weights_lognormal(200001, 3)
    b = Built(pkg, w, pkg.AliasTableConfig(use_partition_elements=use_elems))
    ref = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, 2)
    assert same_table(b.table, ref)


@pytest.mark.parametrize("full_light", [False, True])
@pytest.mark.parametrize("split_size", [4, 12])
def test_split_pack_table_end(pkg, cuda, oracle, full_light, split_size):
    """wrs_split_pack on prefixes summed sequentially in FP32 (coarse enough that the last PSA
    subproblem runs out of heavy items first) with a zero weight at the item past the heavy
    range: the table equals the oracle's with and without the table-end rule of the full
    light cap, and with it no entry aliases a light item."""
    W = pkg.wrs
    w = weights_precision(1 << 20, 5)
    w[-1] = 0.0
    mean = np.float32(oracle.mean(w))
    idx, elems, hc = oracle.partition(w, mean)
    prefix = np.concatenate([np.cumsum(elems[:hc], dtype=np.float32),
                             np.cumsum(elems[hc:][::-1], dtype=np.float32)[::-1]])
    wrs = W.WRS(pkg.AliasTableConfig(split_size=split_size, split_full_light=full_light))
    internals = W.Internals(wrs.handle, w.size)
    W.check(W.lib().wrs_buffers_set_partition_info(internals.ptr, None, float(mean),
                                                   oracle.total_mass(w) / w.size, hc))
    table = empty(2 * w.size, "i32")
    wrs.split_pack(None, h2d(w), h2d(idx), h2d(prefix), h2d(elems), w.size, table, internals)
    got = t2h(table, np.uint32).view(ENTRY_DTYPE)
    assert internals.status() == 0
    ref = oracle.split_pack(w, idx, prefix, hc, mean, split_size, flags=2 if full_light else 0,
                            elems=elems)
    assert same_table(got, ref)
    heavy = np.zeros(w.size, bool)
    heavy[idx[:hc]] = True
    assert heavy[got["a"][got["p"] < 1]].all() == full_light


def test_split_pack_primitive_on_oracle_inputs(pkg, cuda, oracle):
    """wrs_split_pack on inputs made entirely by the oracle (FP64-rounded prefix)."""
    W = pkg.wrs
    w = weights_zipf(30001, 9)
    mean = np.float32(oracle.mean(w))
    idx, elems, hc = oracle.partition(w, mean)
    prefix = oracle.partition_prefix_f64(w, mean).astype(np.float32)
    wrs = W.WRS(pkg.AliasTableConfig(split_size=4))
    internals = W.Internals(wrs.handle, w.size)
    W.check(W.lib().wrs_buffers_set_partition_info(internals.ptr, None, float(mean),
                                                   oracle.total_mass(w) / w.size, hc))
    table = empty(2 * w.size, "i32")
    wrs.split_pack(None, h2d(w), h2d(idx), h2d(prefix), h2d(elems), w.size, table, internals)
    got = t2h(table, np.uint32).view(ENTRY_DTYPE)
    assert same_table(got, oracle.split_pack(w, idx, prefix, hc, mean, 4, elems=elems))


@pytest.mark.parametrize("N", EDGE_N)
def test_edge_sizes_build_and_sample(pkg, cuda, oracle, N):
    w = weights_uniform(N, 5)
    b = Built(pkg, w, pkg.AliasTableConfig())
    idx, _, hc = oracle.partition(w, b.mean)
    assert np.array_equal(b.idx, idx) and b.hc == hc
    assert same_table(b.table, oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, 2))
    S = 1000 + N
    assert np.array_equal(b.sample(S, 77), oracle.alias_sample(b.table, S, 77))


@pytest.mark.parametrize("case", ["all_equal", "zeros", "single_nonzero", "two_values"])
def test_degenerate_weights(pkg, cuda, oracle, case):
    N = 10000
    w = {"all_equal": np.full(N, 0.3, np.float32),
         "zeros": np.where(np.arange(N) % 3 == 0, 0.0, weights_uniform(N, 2)).astype(np.float32),
         "single_nonzero": np.where(np.arange(N) == 4321, 2.5, 0.0).astype(np.float32),
         "two_values": np.where(np.arange(N) % 2 == 0, 1.0, 3.0).astype(np.float32)}[case]
    cfg = pkg.AliasTableConfig(split_full_light=True)
    b = Built(pkg, w, cfg)
    idx, _, hc = oracle.partition(w, b.mean)
    assert np.array_equal(b.idx, idx) and b.hc == hc
    assert same_table(b.table, oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, 2, flags=2))
    s = b.sample(200000, 3)
    assert np.array_equal(s, oracle.alias_sample(b.table, 200000, 3))
    if case in ("zeros", "single_nonzero"):
        assert np.all(w[s] > 0), "a zero-weight item was sampled"
    if case == "single_nonzero":
        assert np.all(s == 4321)


# ------------------------------------------------------------------- sampling ---

@pytest.mark.parametrize("rng,coop", [(RNG_REFERENCE, 0), (RNG_REFERENCE, 128),
                                      (RNG_REFERENCE, 32), (RNG_PHILOX4X32_10, 0)])
@pytest.mark.parametrize("offset", [0, 12345])
def test_alias_sample_bit_exact(pkg, cuda, oracle, rng, coop, offset):
    """Alias samples equal the oracle's restatement of alias/sampling/shader.comp:68-111
    (reference streams) or of the Philox4x32-10 mode, given the GPU's table."""
    w = weights_zipf(100000, 4)
    b = Built(pkg, w, pkg.AliasTableConfig(rng=rng, coop_size=coop))
    S = (1 << 20) + 13
    got = b.sample(S, 0xDEADBEEF12345, offset)
    ref = oracle.alias_sample(b.table, S, 0xDEADBEEF12345, rng=rng, coop=coop, offset=offset,
                              nthreads=8)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("N", [(1 << 22) + 1, (1 << 23) + 6])
@pytest.mark.parametrize("rng,coop", [(RNG_REFERENCE, 0), (RNG_PHILOX4X32_10, 0),
                                      (RNG_REFERENCE, 64)])
@pytest.mark.parametrize("gen", ["uniform", "lognormal"])
def test_alias_sample_coin_filter(pkg, cuda, oracle, N, rng, coop, gen):
    """Tables of more than 2^22 entries are sampled through their coin filter (the table read
    only where the coin does not decide); the samples equal the oracle's full evaluation on
    the GPU's table in both generator modes, and the cooperative mode (no filter) too."""
    w = GENS[gen](N, 9)
    b = Built(pkg, w, pkg.AliasTableConfig(split_size=12, rng=rng, coop_size=coop,
                                           scan_precision=pkg.wrs.SCAN_FLOAT_FLOAT,
                                           split_residual_f64=True, split_full_light=True))
    S = (1 << 21) + 5
    got = b.sample(S, 77, offset=(1 << 20) + 3)
    ref = oracle.alias_sample(b.table, S, 77, rng=rng, coop=coop, offset=(1 << 20) + 3,
                              nthreads=16)
    assert np.array_equal(got, ref)


def test_coin_filter_follows_the_table(pkg, cuda, oracle):
    """A table rewritten in the buffers by the split-pack primitive (another split size) is
    sampled from its new entries, not through the coin filter of the table the build made."""
    W = pkg.wrs
    N = (1 << 22) + 9
    w = weights_uniform(N, 3)
    b = Built(pkg, w, pkg.AliasTableConfig(split_size=12, rng=RNG_PHILOX4X32_10))
    other = W.WRS(pkg.AliasTableConfig(split_size=2, rng=RNG_PHILOX4X32_10))
    v = b.buffers.internals.views()
    other.split_pack(None, b.buffers.weights, v["partition_indices"], v["partition_prefix"],
                     v["partition_elements"], N, v["alias_table"], b.buffers.internals)
    table = d2h(v["alias_table"], N, ENTRY_DTYPE)
    assert not same_table(table, b.table)
    S = 1 << 21
    got = b.sample(S, 5)
    assert np.array_equal(got, oracle.alias_sample(table, S, 5, rng=RNG_PHILOX4X32_10,
                                                   nthreads=16))


@pytest.mark.parametrize("n", [1, 3, 4, 1023, 1024, 1025, (1 << 20) + 3, (1 << 24) + 1])
@pytest.mark.parametrize("seed", [0, 12345, 0xFFFFFFFF])
@pytest.mark.parametrize("shift", [0, 1])
def test_philox_operator_bit_exact(pkg, cuda, oracle, n, seed, shift):
    """The PRNG operator (PRNG::run with PhiloxConfig) equals the oracle's restatement of
    prng/philox/shader.comp:47-55 bit for bit, into aligned and unaligned (shift 1) views,
    and writes nothing past element n - 1."""
    W = pkg.wrs
    buf = empty(n + 8)
    buf.fill_(-7.0)
    W.PRNG().run(None, buf[shift:], n, seed)
    got = t2h(buf, np.float32)
    assert np.array_equal(got[shift:shift + n].view(np.uint32),
                          oracle.philox_uniform(seed, n).view(np.uint32))
    assert np.all(got[:shift] == -7.0) and np.all(got[shift + n:] == -7.0)


@pytest.mark.parametrize("N", [1, 3, 4097, (1 << 20) + 1, 1 << 22])
@pytest.mark.parametrize("comp", [False, True])
def test_scan_precision(pkg, cuda, oracle, N, comp):
    """Inclusive scan against FP64: max relative error <= 1e-6 with the compensated carry,
    <= 1e-4 with the FP32 carry; the reference's own prefix checker accepts it."""
    w = weights_lognormal(N, N)
    b = Built(pkg, w, pkg.ITSConfig(scan_precision=1 if comp else 0))
    assert b.status == 0
    ref = oracle.prefix_f64(w)
    err = np.abs(b.cmf.astype(np.float64) - ref) / np.maximum(ref, 1e-30)
    assert err.max() <= (1e-6 if comp else 1e-4), err.max()


@pytest.mark.parametrize("case", ["dips", "deep_dips", "nan"])
@pytest.mark.parametrize("rng", [RNG_REFERENCE, RNG_PHILOX4X32_10])
def test_its_fp32_cells_on_a_decreasing_cmf(pkg, cuda, oracle, case, rng):
    """The cell search on an FP32 CMF that really decreases (weights outside the contract):
    small negative weights (dips the marks cover cell by cell), large ones (intervals over
    more cells than the marking takes, so every cell bisects), NaN weights (every cell
    bisects).  Samples equal those of the primitive that bisects the CMF, and the oracle's."""
    import torch
    W = pkg.wrs
    N = 300001
    w = weights_lognormal(N, 21)
    r = np.random.default_rng(5)
    pick = r.random(N) < 0.01
    if case == "dips":
        w[pick] = -w[pick] * np.float32(0.01)
    elif case == "deep_dips":
        w[pick] = -w[pick] * np.float32(50.0)
    else:
        w[r.integers(N // 2, N, 3)] = np.float32("nan")
    wrs = W.WRS(pkg.ITSConfig(rng=rng))
    bufs = W.WRSBuffers.allocate(N, 1, wrs.config, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, N)
    S = (1 << 20) + 3
    out = torch.empty(S, dtype=torch.int32, device="cuda")
    bufs.samples = out
    wrs.sample(None, bufs, N, S, 17, offset=2)
    cmf = bufs.internals.views()["cmf"]
    plain = torch.empty(S, dtype=torch.int32, device="cuda")
    wrs.its_sample(None, cmf, N, S, 17, 2, plain)
    torch.cuda.synchronize()
    assert torch.equal(out, plain)
    if case != "nan":  # (a NaN total makes every target NaN-derived; the primitive is the bar)
        got = t2h(out, np.uint32)
        ref = oracle.its_sample(d2h(cmf, N, np.float32), S, 17, rng=rng, offset=2, nthreads=8)
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("N", [8191, 8192, 8193, 3 * 8192 + 5])
@pytest.mark.parametrize("comp", [False, True])
@pytest.mark.parametrize("shift_in,shift_out", [(0, 0), (1, 0), (0, 1), (3, 2)])
def test_scan_tiles_and_unaligned_views(pkg, cuda, oracle, N, comp, shift_in, shift_out):
    """The scan primitive around its tile size (8192 weights per bulk-copied tile in FP32
    mode) and on views whose pointers are not 16-byte aligned (input read with plain loads,
    output written element by element): within the precision's bound of the FP64 prefix."""
    W = pkg.wrs
    w = weights_lognormal(N + shift_in, N)
    wrs = W.WRS(pkg.ITSConfig(scan_precision=1 if comp else 0))
    internals = W.Internals(wrs.handle, N)
    dw = h2d(w)
    out = empty(N + shift_out)
    wrs.prefix_sum(None, dw[shift_in:], N, out[shift_out:], internals)
    assert internals.status() == 0
    got = t2h(out, np.float32)[shift_out:].astype(np.float64)
    ref = oracle.prefix_f64(w[shift_in:])
    err = np.abs(got - ref) / np.maximum(ref, 1e-30)
    assert err.max() <= (1e-6 if comp else 1e-4), err.max()


@pytest.mark.parametrize("N", [4097, (1 << 22) + 5])
def test_compensated_cmf_is_exactly_monotone(pkg, cuda, oracle, N):
    """The compensated CMF is non-decreasing, equal across every zero weight (also at thread
    and tile boundaries), bit-identical across builds, and the Philox ITS sampler never draws
    a zero-weight index."""
    w = weights_precision(N, 9)
    w[::4096] = 0.0                   # zero weights at every tile start
    w[16::4096] = 0.0                 # ... and at a thread boundary inside every tile
    w[0] = 1.0
    cfg = pkg.ITSConfig(scan_precision=1, rng=RNG_PHILOX4X32_10)
    a = Built(pkg, w, cfg)
    b = Built(pkg, w, cfg)
    assert np.array_equal(a.cmf.view(np.uint32), b.cmf.view(np.uint32))
    d = np.diff(a.cmf.astype(np.float64))
    assert np.all(d >= 0)
    zero = np.nonzero(w[1:] == 0)[0]
    assert np.all(d[zero] == 0)
    s = a.sample(1 << 22, 3)
    assert not np.any(w[s] == 0)
    ref = oracle.prefix_f64(w)
    assert np.abs(a.cmf.astype(np.float64) - ref).max() <= 1e-6 * ref[-1]


def _fx(x: np.float32, g: int) -> int:
    """An FP32 value >= 0 on the fixed-point grid 2^g (bits below the grid dropped)."""
    b = int(np.float32(x).view(np.uint32))
    e, m = b >> 23, b & 0x7FFFFF
    ex = -149
    if e:
        m |= 1 << 23
        ex = e - 150
    sh = ex - g
    return m << sh if sh >= 0 else m >> -sh


def _round_f32(k: int, g: int) -> np.float32:
    """k * 2^g rounded to nearest FP32 (ties to even), for normal results."""
    if k == 0:
        return np.float32(0.0)
    nb = k.bit_length()
    q, e = k, g
    if nb > 24:
        sh = nb - 24
        q, rem, half = k >> sh, k & ((1 << sh) - 1), 1 << (sh - 1)
        if rem > half or (rem == half and q & 1):
            q += 1
        e = g + sh
    return np.float32(math.ldexp(q, e))


def exact_cmf(w: np.ndarray, total: float) -> np.ndarray:
    """The compensated CMF's definition: element i of thread t (16 consecutive weights per
    thread) is RN(K_t + r_i) -- K_t the exact fixed-point sum of the FP32 totals of all threads
    before t, r_i the thread's FP32 running sum through i, both on the grid 2^g that the
    distribution's FP64 total sets (its exponent minus 123)."""
    g = math.frexp(total)[1] - 123
    pad = (-w.size) % 16
    run = np.cumsum(np.concatenate([w, np.zeros(pad, np.float32)]).reshape(-1, 16), axis=1,
                    dtype=np.float32)
    out = np.empty(w.size, np.float32)
    K = 0
    for t in range(run.shape[0]):
        for c in range(16):
            i = 16 * t + c
            if i < w.size:
                out[i] = _round_f32(K + _fx(run[t, c], g), g)
        K += _fx(run[t, 15], g)
    return out


@pytest.mark.parametrize("N", [4097, 3 * 4096 + 5, 65536 + 77])
@pytest.mark.parametrize("gen", ["uniform", "lognormal", "precision"])
def test_compensated_cmf_bit_exact(pkg, cuda, N, gen):
    """Every element of the compensated CMF equals its definition computed on the CPU with
    exact integers (the GPU decides most roundings from a float-float evaluation and the
    rest in fixed point; both must give the correctly rounded sum)."""
    w = {"uniform": weights_uniform, "lognormal": weights_lognormal,
         "precision": weights_precision}[gen](N, 3 * N + 1)
    w[0] = max(w[0], np.float32(1e-3))  # keep the first values normal
    b = Built(pkg, w, pkg.ITSConfig(scan_precision=1))
    assert b.status == 0
    total = float(d2h(b.buffers.internals.views()["total"], 1, np.float64)[0])
    assert np.array_equal(b.cmf.view(np.uint32), exact_cmf(w, total).view(np.uint32))


@pytest.mark.parametrize("rng,coop,parray", [(RNG_REFERENCE, 0, False),
                                             (RNG_REFERENCE, 128, False),
                                             (RNG_REFERENCE, 4096, True),
                                             (RNG_REFERENCE, 64, True),
                                             (RNG_PHILOX4X32_10, 0, False)])
def test_its_sample_bit_exact(pkg, cuda, oracle, rng, coop, parray):
    """ITS samples equal the oracle's restatement of its/sampling/shader.comp:80-177 (or the
    Philox4x32-10 mode) given the GPU's CMF."""
    w = weights_uniform(300001, 8)
    b = Built(pkg, w, pkg.ITSConfig(coop_size=coop, parray=parray, rng=rng))
    S = (1 << 20) + 5
    got = b.sample(S, 4242, 99)
    ref = oracle.its_sample(b.cmf, S, 4242, rng=rng, coop=coop, parray=parray, offset=99,
                            nthreads=8)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("N", [1, 2, 33, 4097, 300001, (1 << 22) + 3])
@pytest.mark.parametrize("rng", [RNG_REFERENCE, RNG_PHILOX4X32_10])
@pytest.mark.parametrize("entry", [1, 4, 8, 32, 0])
def test_its_guided_sampling_on_the_compensated_cmf(pkg, cuda, oracle, N, rng, entry):
    """ITS on the compensated (non-decreasing) CMF runs the guided search (a guiding-table cell
    instead of the whole range, its values read with vector loads when the cell is short):
    samples equal the oracle's plain bisection for every guiding-table granularity (entry 0:
    no table), also with runs of zero weights and a heavy tail."""
    w = weights_precision(N, N)
    w[0] = max(w[0], np.float32(0.25))
    b = Built(pkg, w, pkg.ITSConfig(rng=rng, scan_precision=1, guiding_entry_size=entry))
    assert np.all(np.diff(b.cmf.astype(np.float64)) >= 0)
    S = (1 << 20) + 11
    got = b.sample(S, 4242, 7)
    ref = oracle.its_sample(b.cmf, S, 4242, rng=rng, offset=7, nthreads=8)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("gen", ["zipf", "lognormal"])
@pytest.mark.parametrize("entry", [3, 8])
def test_its_cells_heavy_heads_and_crowded_cells(pkg, cuda, oracle, gen, entry):
    """Cell blocks under skewed weights: heavy items span many one-item cells, light regions
    give crowded cells (more than a block holds) that take the bisection; samples equal the
    oracle's bisection."""
    N = (1 << 20) + 7
    w = GENS[gen](N, 77 + entry)
    b = Built(pkg, w, pkg.ITSConfig(rng=RNG_PHILOX4X32_10, scan_precision=1,
                                    guiding_entry_size=entry))
    S = (1 << 20) + 3
    got = b.sample(S, 99, 3)
    assert np.array_equal(got, oracle.its_sample(b.cmf, S, 99, rng=RNG_PHILOX4X32_10, offset=3,
                                                 nthreads=8))


def test_its_buffers_must_hold_the_handles_cells(pkg, cuda):
    """A compensated ITS handle refuses buffers made without cell blocks (an FP32 handle's
    with cell size 0) or with another cell size, instead of reading past them."""
    W = pkg.wrs
    N = 10000
    w = h2d(weights_uniform(N, 3))
    fp32 = W.WRS(pkg.ITSConfig(scan_precision=0, guiding_entry_size=0))
    comp8 = W.WRS(pkg.ITSConfig(scan_precision=1, guiding_entry_size=8))
    comp4 = W.WRS(pkg.ITSConfig(scan_precision=1, guiding_entry_size=4))
    b32 = W.WRSBuffers.allocate(N, 16, fp32.config, handle=fp32.handle)
    b8 = W.WRSBuffers.allocate(N, 16, comp8.config, handle=comp8.handle)
    for h, b in ((comp8, b32), (comp4, b8)):
        b.weights.copy_(w)
        with pytest.raises(W.WRSError) as e:
            h.build(None, b, N)
        assert e.value.status == 1
        with pytest.raises(W.WRSError):
            h.sample(None, b, N, 16, 1)
    b8.weights.copy_(w)
    comp8.build(None, b8, N)
    comp8.sample(None, b8, N, 16, 1)
    assert b8.internals.status() == 0


@pytest.mark.parametrize("N", [1, 2, 3, 7, 4095, 4096, 4097, 8191, 8193, 70001])
@pytest.mark.parametrize("rng", [RNG_REFERENCE, RNG_PHILOX4X32_10])
def test_its_sample_edge_sizes(pkg, cuda, oracle, N, rng):
    """The non-cooperative ITS sampler (probe tree cached in shared memory) at sizes around
    the cached depth, with runs of zero weights (equal CMF values), equals the oracle."""
    w = weights_uniform(N, N)
    w[np.random.default_rng(N).random(N) < 0.2] = 0.0
    w[0] = max(w[0], np.float32(0.5))
    b = Built(pkg, w, pkg.ITSConfig(rng=rng))
    S = 3 * 1024 + 77
    got = b.sample(S, 7, 5)
    ref = oracle.its_sample(b.cmf, S, 7, rng=rng, offset=5)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("rng", [RNG_REFERENCE, RNG_PHILOX4X32_10])
@pytest.mark.parametrize("entry", [0, 4])
def test_its_stored_tree_blocks(pkg, cuda, oracle, rng, entry):
    """The FP32 build stores the bisection's probe tree as blocks of three levels.  Cell size 0:
    the tree sampler (shared-memory top, block levels below); cell size 4: the cell search on
    the unmarked cells of the (not monotone) FP32 CMF, the bisection through the blocks on the
    marked ones.  Samples through the buffers equal those of the primitive that probes the CMF
    itself at 2^22 + 3, 2^19 + 1 and 2^16 + 1, the same buffers rebuilt for each smaller size;
    the last equals the oracle."""
    import torch
    W = pkg.wrs
    cfg = pkg.ITSConfig(rng=rng, guiding_entry_size=entry)
    wrs = W.WRS(cfg)
    sizes = ((1 << 22) + 3, (1 << 19) + 1, (1 << 16) + 1)
    bufs = W.WRSBuffers.allocate(sizes[0], 1, cfg, handle=wrs.handle)
    S = (1 << 21) + 9
    small = sizes[-1]
    for N in sizes:
        w = weights_lognormal(N, N)
        bufs.weights[:N].copy_(h2d(w))
        wrs.build(None, bufs, N)
        out = torch.empty(S, dtype=torch.int32, device="cuda")
        bufs.samples = out
        wrs.sample(None, bufs, N, S, 31, offset=4)
        plain = torch.empty(S, dtype=torch.int32, device="cuda")
        cmf = bufs.internals.views()["cmf"]
        wrs.its_sample(None, cmf, N, S, 31, 4, plain)
        torch.cuda.synchronize()
        assert bufs.internals.status() == 0
        assert torch.equal(out, plain)
    got = t2h(out, np.uint32)
    ref = oracle.its_sample(d2h(cmf, small, np.float32), S, 31, rng=rng, offset=4, nthreads=8)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("precision", [0, 1])
def test_its_sample_n_other_than_built(pkg, cuda, oracle, precision):
    """Sampling with an n other than the last build's: the cell blocks and probe-tree blocks
    were written for the built n and are not read; the samples equal the primitive's bisection
    of the first n CMF values (and the oracle's).  A sample call on buffers never built returns
    indices inside [0, n)."""
    import torch
    W = pkg.wrs
    cfg = pkg.ITSConfig(rng=RNG_PHILOX4X32_10, scan_precision=precision)
    wrs = W.WRS(cfg)
    N, n = (1 << 20) + 3, 70001
    fresh = W.WRSBuffers.allocate(N, 1, cfg, handle=wrs.handle)
    S = (1 << 18) + 5
    out = torch.empty(S, dtype=torch.int32, device="cuda")
    fresh.samples = out
    wrs.sample(None, fresh, n, S, 5, offset=2)
    assert int(t2h(out, np.uint32).max()) < n
    bufs = W.WRSBuffers.allocate(N, 1, cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(weights_lognormal(N, 17)))
    wrs.build(None, bufs, N)
    bufs.samples = out
    wrs.sample(None, bufs, n, S, 5, offset=2)
    plain = torch.empty(S, dtype=torch.int32, device="cuda")
    cmf = bufs.internals.views()["cmf"]
    wrs.its_sample(None, cmf, n, S, 5, 2, plain)
    torch.cuda.synchronize()
    assert bufs.internals.status() == 0
    assert torch.equal(out, plain)
    ref = oracle.its_sample(d2h(cmf, n, np.float32), S, 5, rng=RNG_PHILOX4X32_10, offset=2,
                            nthreads=8)
    assert np.array_equal(t2h(out, np.uint32), ref)


# ------------------------------------------------------------------- cutpoint ---

@pytest.mark.parametrize("N,entry", [(1, 32), (5, 1), (1000, 32), (4097, 128), (300001, 32),
                                     ((1 << 20) + 3, 7)])
@pytest.mark.parametrize("rng", [RNG_REFERENCE, RNG_PHILOX4X32_10])
@pytest.mark.parametrize("precision", [0, 1])
def test_cutpoint_bit_exact(pkg, cuda, oracle, N, entry, rng, precision):
    """Cutpoint (guiding table + guided sampling): the guiding table equals the oracle's
    restatement of cutpoint/guiding_table/shader.comp and the samples its restatement of
    cutpoint/sampling/shader.comp, given the GPU's CMF.  On the compensated (non-decreasing)
    CMF the table is built by galloping searches; it must still equal the bisections'."""
    W = pkg.wrs
    w = weights_uniform(N, N + entry)
    if precision:
        w[np.random.default_rng(N).random(N) < 0.3] = 0.0  # runs of equal CMF values
        w[0] = np.float32(0.5)
    cfg = pkg.CutpointConfig(entry, rng=rng, scan_precision=precision)
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(N, 1, cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, N)
    v = bufs.internals.views()
    cmf = d2h(v["cmf"], N, np.float32)
    G = (N + entry - 1) // entry
    guide = d2h(v["guide_table"], G, np.uint32)
    assert np.array_equal(guide, oracle.cutpoint_guide(cmf, entry))
    S = 100003
    import torch
    out = torch.empty(S, dtype=torch.int32, device="cuda")
    bufs.samples = out
    wrs.sample(None, bufs, N, S, 4242, offset=17)
    got = t2h(out, np.uint32)
    assert np.array_equal(got, oracle.cutpoint_sample(cmf, guide, S, 4242, rng=rng, offset=17))
    assert got.max() < N
    assert bufs.internals.status() == 0


def test_cutpoint_primitives(pkg, cuda, oracle):
    """wrs_cutpoint_guide / wrs_cutpoint_sample on a caller's CMF (an oracle prefix sum)."""
    W = pkg.wrs
    N, entry = 77777, 64
    w = weights_lognormal(N, 3)
    cmf = oracle.prefix_kahan(w)
    wrs = W.WRS(pkg.CutpointConfig(entry))
    G = (N + entry - 1) // entry
    dcmf = h2d(cmf)
    guide = empty(G, "i32")
    wrs.cutpoint_guide(None, dcmf, N, guide)
    g = t2h(guide, np.uint32)
    assert np.array_equal(g, oracle.cutpoint_guide(cmf, entry))
    out = empty(5000, "i32")
    wrs.cutpoint_sample(None, dcmf, N, guide, 5000, 99, 0, out)
    assert np.array_equal(t2h(out, np.uint32), oracle.cutpoint_sample(cmf, g, 5000, 99))


# ----------------------------------------------------------------- statistics ---

@pytest.mark.parametrize("gen", list(GENS))
def test_sampling_statistics(pkg, cuda, oracle, gen):
    """Two separate claims (Philox4x32-10 streams):
    (1) the samplers are unbiased for the distribution their build encodes -- a binned
        chi-square test of S = 2^24 samples against the table's (alias) or the CMF's (ITS)
        implied probabilities gives p > 1e-4;
    (2) the build encodes the target: alias-table weights within 0.05 mean-units of w/mean
        (FP32 partition prefixes quantise the split residuals), CMF steps within two ulps of
        the total of w."""
    N, S = 65536, 1 << 24
    w = GENS[gen](N, 21)
    target = w / w.astype(np.float64).mean()
    b = Built(pkg, w, pkg.AliasTableConfig(rng=RNG_PHILOX4X32_10, split_full_light=True,
                                           scan_precision=1, split_residual_f64=True))
    implied = oracle.alias_to_weights(b.table)
    st = oracle.sample_stats(b.sample(S, 31337), implied.astype(np.float32))
    assert st["p_value"] > 1e-4, ("alias", st)
    assert np.abs(implied - target).max() < 0.05
    b = Built(pkg, w, pkg.ITSConfig(rng=RNG_PHILOX4X32_10, scan_precision=1))
    steps = np.diff(np.concatenate([[0.0], b.cmf.astype(np.float64)]))
    st = oracle.sample_stats(b.sample(S, 31337), steps.astype(np.float32))
    assert st["p_value"] > 1e-4, ("its", st)
    ulp = np.spacing(np.float32(b.cmf[-1]))
    assert np.abs(steps - w).max() <= 2 * ulp


def test_precision_weights_never_sample_zero(pkg, cuda, oracle):
    """Log-normal(0,3) with 1% zeros and 0.01% scaled by 1e6: no zero-weight item is drawn
    (alias with the light-cap fix, and ITS with Philox4x32-10)."""
    N = 1 << 20
    w = weights_precision(N, 5)
    for cfg in (pkg.AliasTableConfig(rng=RNG_PHILOX4X32_10, split_full_light=True,
                                     scan_precision=1, split_residual_f64=True),
                pkg.ITSConfig(rng=RNG_PHILOX4X32_10, scan_precision=1)):
        b = Built(pkg, w, cfg)
        s = b.sample(1 << 22, 5)
        assert np.all(w[s] > 0), cfg.name()


@pytest.mark.parametrize("method", ["alias", "its"])
def test_sample_into_pinned_host_memory(pkg, cuda, method):
    """wrs_sample with a pinned host buffer as the output writes the same samples as with a
    device buffer."""
    import torch
    W = pkg.wrs
    w = weights_lognormal(100003, 4)
    cfg = (pkg.AliasTableConfig(split_size=8, rng=W.RNG_PHILOX4X32_10)
           if method == "alias" else pkg.ITSConfig(rng=W.RNG_PHILOX4X32_10))
    b = Built(pkg, w, cfg)
    S = (1 << 20) + 3
    dev = b.sample(S, 77)
    host = torch.zeros(S, dtype=torch.int32).pin_memory()
    b.wrs.sample(None, W.WRSBuffers(b.buffers.weights, host.data_ptr(), b.buffers.internals),
                 b.N, S, 77)
    torch.cuda.synchronize()
    assert np.array_equal(host.numpy().view(np.uint32), dev)


# ------------------------------------------------------------ determinism, status ---

@pytest.mark.parametrize("precision", [1, 2])
def test_build_is_deterministic(pkg, cuda, precision):
    """Repeated builds of one input give identical prefixes and tables: in the compensated
    precisions the lookback carries exact fixed-point sums, so a tile's carry does not
    depend on which predecessors the lookback saw."""
    w = weights_lognormal((1 << 22) + 9, 12)
    cfg = pkg.AliasTableConfig(scan_precision=precision, split_size=8)
    a = Built(pkg, w, cfg)
    for _ in range(3):
        b = Built(pkg, w, cfg)
        assert np.array_equal(a.prefix.view(np.uint32), b.prefix.view(np.uint32))
        if precision == 2:
            assert np.array_equal(a.prefix_lo.view(np.uint32), b.prefix_lo.view(np.uint32))
        assert same_table(a.table, b.table)


def test_repeated_builds_reuse_buffers(pkg, cuda, oracle):
    """One buffers object serves many builds of different sizes (self-cleaning lookback
    state), for both the partition and the scan kernels."""
    W = pkg.wrs
    cfg = pkg.AliasTableConfig()
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(1 << 20, 1, cfg, handle=wrs.handle)
    its = W.WRS(pkg.ITSConfig())
    for k, N in enumerate([1 << 20, 5000, 777777, 1 << 20, 4096, 123456]):
        w = weights_uniform(N, k)
        bufs.weights[:N].copy_(h2d(w))
        wrs.build(None, bufs, N)
        v = bufs.internals.views()
        idx = d2h(v["partition_indices"], N, np.uint32)
        mean = d2h(v["mean"], 1, np.float32)[0]
        assert np.array_equal(idx, oracle.partition(w, mean)[0])
        out = empty(N)
        its.prefix_sum(None, bufs.weights, N, out, bufs.internals)
        ref = oracle.prefix_f64(w)
        assert np.abs(t2h(out, np.float32) - ref).max() <= 1e-4 * ref[-1]
    assert bufs.internals.status() == 0


def test_lookback_wait_runs_out_and_reports(pkg, cuda):
    """A scan whose first tile is never scheduled: every other tile's lookback wait runs out
    of its budget, the kernel still ends, the status reports a timeout, and the context
    stays usable for a normal build afterwards."""
    import ctypes as C
    W = pkg.wrs
    N = 64 * 4096
    w = weights_uniform(N, 1)
    wrs = W.WRS(pkg.ITSConfig())
    internals = W.Internals(wrs.handle, N)
    dw, out = h2d(w), empty(N)
    W.check(W.lib().wrs_test_prefix_sum_stalled(wrs.handle.ptr, None, dw.data_ptr(), N,
                                                out.data_ptr(), internals.ptr, 2000))
    v = C.c_uint32(0)
    assert W.lib().wrs_buffers_status(internals.ptr, None, C.byref(v)) == 3  # WRS_ERR_TIMEOUT
    assert v.value & W.DEVICE_TIMEOUT
    # the context and the buffers are still good
    wrs.prefix_sum(None, dw, N, out, internals)
    assert internals.status() == 0
    got = t2h(out, np.float32).astype(np.float64)
    ref = np.cumsum(w.astype(np.float64))
    assert np.abs(got - ref).max() <= 1e-4 * ref[-1]
