"""GPU tests of the block-wise (reduce-then-scan) baselines: the scan within the FP32 carry
bound of the FP64 prefix, the partition's indices, elements and heavy count bit-exact against
the oracle's stable partition (and the decoupled kernel's), its prefixes within the FP32
bound."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform, weights_zipf
from gpu_util import d2h, h2d, t2h

pytestmark = pytest.mark.gpu

GENS = {"uniform": weights_uniform, "zipf": weights_zipf, "lognormal": weights_lognormal}


def _bound(N, total):
    # FP32: one rounding per tile carry and per add inside a tile's thread/warp/CTA tree
    tiles = (N + 4095) // 4096
    return (tiles + 4096 + 64) * 2.0 ** -24 * total


@pytest.mark.parametrize("N", [1, 5, 4096, 4097, (1 << 20) + 3, 1 << 22])
@pytest.mark.parametrize("gen", ["uniform", "lognormal"])
def test_blockwise_scan(pkg, cuda, oracle, N, gen):
    import torch
    W = pkg.wrs
    w = GENS[gen](N, N + 1)
    its = W.WRS(pkg.ITSConfig())
    internals = W.Internals(its.handle, N)
    out = torch.empty(N, dtype=torch.float32, device="cuda")
    its.prefix_sum_blockwise(None, h2d(w), N, out, internals)
    got = t2h(out, np.float32).astype(np.float64)
    ref = oracle.prefix_f64(w)
    assert np.abs(got - ref).max() <= _bound(N, ref[-1])
    assert internals.status() == 0


@pytest.mark.parametrize("N", [1, 7, 4096, 4097, 100003, (1 << 22) + 17])
@pytest.mark.parametrize("gen", ["uniform", "zipf", "lognormal"])
def test_blockwise_partition(pkg, cuda, oracle, N, gen):
    import torch
    W = pkg.wrs
    w = GENS[gen](N, 2 * N + 3)
    wrs = W.WRS(pkg.AliasTableConfig())
    internals = W.Internals(wrs.handle, N)
    dw = h2d(w)
    wrs.total_mass(None, dw, N, internals)
    idx = torch.empty(N, dtype=torch.int32, device="cuda")
    prefix = torch.empty(N, dtype=torch.float32, device="cuda")
    elems = torch.empty(N, dtype=torch.float32, device="cuda")
    wrs.prefix_partition_blockwise(None, dw, N, idx, prefix, elems, internals)
    v = internals.views()
    mean = float(d2h(v["mean"], 1, np.float32)[0])
    hc = int(d2h(v["heavy_count"], 1, np.uint32)[0])
    ridx, _, rhc = oracle.partition(w, mean)
    assert hc == rhc
    gidx = t2h(idx, np.uint32)
    assert np.array_equal(gidx, ridx)
    assert np.array_equal(t2h(elems, np.float32).view(np.uint32), w[ridx].view(np.uint32))
    ref = oracle.partition_prefix_f64(w, mean)
    got = t2h(prefix, np.float32).astype(np.float64)
    assert np.abs(got - ref).max() <= _bound(N, float(w.astype(np.float64).sum()))
    # the decoupled FP32 kernel puts every item at the same position
    idx2 = torch.empty(N, dtype=torch.int32, device="cuda")
    prefix2 = torch.empty(N, dtype=torch.float32, device="cuda")
    wrs.prefix_partition(None, dw, N, idx2, prefix2, None, internals)
    assert np.array_equal(t2h(idx2, np.uint32), gidx)
    assert internals.status() == 0
