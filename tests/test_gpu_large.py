"""GPU tests at the largest sizes: N = 2^30 + 7 weights (4 GB, ragged against the tile, the
split size and the ITS cell size; 1% zero weights, log-normal(0, 2) otherwise) and S = 2^30
samples, built and sampled through the buffers API (alias float-float; ITS compensated with
cell blocks).  The full arrays are too large for the oracle at test speed, so the checks are
the size-independent properties, computed on the device: every sample in range, no draw on
a zero-probability bucket, and the RMSE of the histogram against the target distribution
within 2% of its ideal value sqrt(sum p (1 - p) / (S N)) (a bias of 1e-3 relative per bucket
would show as several times that).  The alias table's target is the weights themselves (the
float-float prefix resolves every weight).  ITS samples the stored FP32 CMF, whose ulp at a
total of ~8e9 is 1024 -- coarser than the weights (~1-50), as in the reference's FP32 ITS --
so its target is the CMF's steps p_i = (cmf[i] - cmf[i-1]) / total (exact FP32 differences of
neighbours); the test checks the sampler against exactly that."""
from __future__ import annotations

import math

import pytest

pytestmark = pytest.mark.gpu

N = (1 << 30) + 7
S = 1 << 30


def _weights(seed: int):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    w = torch.exp(2.0 * torch.randn(N, generator=g, device="cuda"))
    w[torch.rand(N, generator=g, device="cuda") < 0.01] = 0.0
    return w


@pytest.mark.parametrize("method", ["alias", "its"])
def test_max_size_build_and_sample(pkg, cuda, method):
    import torch
    W = pkg.wrs
    if method == "alias":
        cfg = pkg.AliasTableConfig(split_size=12, rng=W.RNG_PHILOX4X32_10,
                                   scan_precision=W.SCAN_FLOAT_FLOAT, split_residual_f64=True,
                                   split_full_light=True)
    else:
        cfg = pkg.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=W.SCAN_COMPENSATED)
    w = _weights(11 if method == "alias" else 12)
    samples = torch.empty(S, dtype=torch.int32, device="cuda")
    wrs = W.WRS(cfg)
    internals = W.Internals(wrs.handle, N)
    bufs = W.WRSBuffers(w, samples, internals)
    wrs.build(None, bufs, N)
    wrs.sample(None, bufs, N, S, seed=2024)
    assert internals.status() == 0
    if method == "its":
        # the build's CMF (exact carries: the primitive computes the same values) and its
        # steps, the distribution ITS samples
        cmf = torch.empty(N, dtype=torch.float32, device="cuda")
        wrs.prefix_sum(None, w, N, cmf, internals)
        w = torch.diff(cmf, prepend=torch.zeros(1, dtype=torch.float32, device="cuda"))
        del cmf
    del internals, bufs
    st = W.Statistics(N)(None, samples, S, w)
    assert not st["out_of_range"]
    assert st["zero_weight_draws"] == 0
    p = w.double() / st["total"]
    ideal = math.sqrt(float((p * (1.0 - p)).sum()) / (S * N))
    assert abs(st["rmse"] / ideal - 1.0) < 0.02, (st["rmse"], ideal)


@pytest.mark.parametrize("rng,entry", [("reference", 4), ("philox", 4), ("philox", 0)])
def test_max_size_its_fp32_stored_tree(pkg, cuda, rng, entry):
    """FP32 ITS at N = 2^30 + 7: the build stores the bisection's probe tree as blocks (tree
    levels 0 .. 26, 614 MB); cell size 0 samples with the tree sampler, cell size 4 with the
    cell search on the unmarked cells and the block bisection on the marked ones.  2^27 samples
    through the buffers equal those of the primitive that probes the CMF alone (same probe
    sequence), all in range."""
    import torch
    W = pkg.wrs
    cfg = pkg.ITSConfig(rng=W.RNG_PHILOX4X32_10 if rng == "philox" else W.RNG_REFERENCE,
                        guiding_entry_size=entry)
    w = _weights(13)
    S = 1 << 27
    samples = torch.empty(S, dtype=torch.int32, device="cuda")
    wrs = W.WRS(cfg)
    internals = W.Internals(wrs.handle, N)
    bufs = W.WRSBuffers(w, samples, internals)
    wrs.build(None, bufs, N)
    wrs.sample(None, bufs, N, S, seed=99, offset=1 << 33)
    plain = torch.empty_like(samples)
    wrs.its_sample(None, internals.views()["cmf"], N, S, 99, 1 << 33, plain)
    torch.cuda.synchronize()
    assert internals.status() == 0
    assert torch.equal(samples, plain)
    assert int(samples.min()) >= 0
    assert int(samples.max()) < N
