"""GPU parity at the benchmark's own configurations and full sizes.

The headline configuration is the single large distribution: N = 2^26 weights of each of
its three seeded shapes (uniform(0,1], Zipf-like permuted, log-normal(0, 2)), built with the
benchmark's alias configuration -- split size 12, float-float partition prefix, FP64 split
residual, full light cap, Philox4x32-10 -- and sampled.  At that size the FP32 split
predicate stops being monotone and PSA subproblems can overlap, which the smaller parity
tests do not reach.  The precision configuration is N = 2^28 log-normal(0, 3) weights with
1% zeros and 0.01% scaled by 1e6.

Bar (as in the reference's test strategy, given the same upstream arrays):
  * partition indices, partition elements and heavy count bit-exact against the oracle's
    stable partition at the GPU's mean;
  * the whole alias table (p bits and alias indices) bit-exact against the oracle's
    split+pack fed the GPU's partition arrays;
  * 2^24 samples at a nonzero counter offset bit-exact against the oracle's sampler on the
    GPU's table;
  * no device status bit: no lookback timeout and no subproblem overlap beyond the
    ownership window.
"""
from __future__ import annotations

import importlib
import os

import numpy as np
import pytest

from gpu_util import t2h
from oracle.oracle import RNG_PHILOX4X32_10, SPLIT_F64, SPLIT_FULL_LIGHT
from test_gpu_parity import Built, same_table

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))
SPLIT_SIZE = 12
FLAGS = SPLIT_F64 | SPLIT_FULL_LIGHT


def workloads():
    return importlib.import_module("merian-wrs_gb300.workloads")


def headline_config(pkg, precision=None):
    W = pkg.wrs
    return pkg.AliasTableConfig(split_size=SPLIT_SIZE, rng=W.RNG_PHILOX4X32_10,
                                scan_precision=W.SCAN_FLOAT_FLOAT if precision is None
                                else precision,
                                split_residual_f64=True, split_full_light=True)


def check_build(pkg, oracle, w: np.ndarray, cfg, seed: int, offset: int, S: int = 1 << 24):
    W = pkg.wrs
    ff = cfg.scan_precision == W.SCAN_FLOAT_FLOAT
    b = Built(pkg, w, cfg)
    assert b.status == 0, f"device status {b.status}"
    N = w.size
    # against numpy's pairwise FP64 sum (error ~ log2(N) ulps; a sequential sum's grows with N)
    assert abs(b.total - float(np.sum(w, dtype=np.float64))) <= 1e-12 * b.total
    assert b.mean64 == b.total / N
    idx, elems, hc = oracle.partition(w, b.mean)
    assert b.hc == hc
    assert np.array_equal(b.idx, idx)
    assert np.array_equal(b.elems.view(np.uint32), elems.view(np.uint32))
    del idx, elems
    ref = oracle.split_pack(w, b.idx, b.prefix, b.hc, b.mean, SPLIT_SIZE, flags=FLAGS,
                            elems=b.elems, prefix_lo=b.prefix_lo if ff else None,
                            mean64=b.mean64, nthreads=THREADS)
    assert same_table(b.table, ref)
    del ref
    got = b.sample(S, seed, offset)
    assert np.array_equal(got, oracle.alias_sample(b.table, S, seed, rng=RNG_PHILOX4X32_10,
                                                   offset=offset, nthreads=THREADS))
    return b


@pytest.mark.parametrize("N", [1 << 26, (1 << 26) + 5])
@pytest.mark.parametrize("dist", [0, 1, 2], ids=["uniform", "zipf", "lognormal"])
def test_headline_alias_bit_exact(pkg, cuda, oracle, N, dist):
    """The benchmark's build of each of its three distributions at N = 2^26 (and a ragged
    2^26 + 5): partition, whole table and 2^24 samples at a counter offset inside the
    benchmark's 2^28-sample stream equal the oracle's."""
    wl = workloads()
    w = t2h(wl.headline(dist, N, wl.HEADLINE_SEEDS[dist], "cuda"), np.float32)
    check_build(pkg, oracle, w, headline_config(pkg), seed=1234,
                offset=(1 << 28) - (1 << 24) + 7)


@pytest.mark.parametrize("precision", ["float-float", "compensated"])
def test_precision_config_alias_bit_exact(pkg, cuda, oracle, precision):
    """The precision configuration at N = 2^28 (1% zero weights, 0.01% scaled by 1e6): the
    partition, the whole table and 2^24 samples equal the oracle's, for the float-float
    prefix and for the compensated (FP32 prefix, exact carries) precision, and no zero-weight
    item can be drawn."""
    W = pkg.wrs
    w = t2h(workloads().precision(1 << 28, "cuda"), np.float32)
    prec = W.SCAN_FLOAT_FLOAT if precision == "float-float" else W.SCAN_COMPENSATED
    b = check_build(pkg, oracle, w, headline_config(pkg, prec), seed=11, offset=12345)
    # zero-weight items get no probability at all: they keep p = 0, and with the table-end
    # rule of the full light cap every bucket that can send a draw to its alias aliases a
    # heavy item (in the compensated precision the last subproblem runs out of heavy items
    # first at this size; the reference's table end then aliases the light item past them)
    assert np.all(b.table["p"][w == 0] == 0)
    heavy = np.zeros(w.size, bool)
    heavy[b.idx[:b.hc]] = True
    assert heavy[b.table["a"][b.table["p"] < 1]].all()
