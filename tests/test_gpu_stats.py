"""GPU tests of the on-device statistics (wrs_histogram, wrs_sample_statistics): the
histogram equals numpy's bincount bit for bit; chi-square and RMSE agree with the oracle's
restatement of the reference's host statistics (src/host/statistics/chi_square.hpp, the RMSE
of src/dep/eval/rms.hpp) to 1e-6 relative; repeated runs are bit-identical."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform
from gpu_util import h2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,S", [(1, 100), (1000, 1 << 20), (70001, (1 << 22) + 7)])
def test_histogram_and_statistics(pkg, cuda, oracle, N, S):
    import torch
    W = pkg.wrs
    rng = np.random.default_rng(N)
    w = weights_lognormal(N, 3)
    if N > 1:
        w[rng.random(N) < 0.05] = 0.0
    samples = rng.integers(0, N, S, dtype=np.uint32)
    st = W.Statistics(N)
    dw, ds = h2d(w), h2d(samples)
    r = st(None, ds, S, dw)
    hist = st.hist.cpu().numpy().astype(np.uint64)
    assert np.array_equal(hist, np.bincount(samples, minlength=N).astype(np.uint64))
    assert not r["out_of_range"]
    ref_chi2 = oracle.chi_square(hist, w, S)
    ref_rmse = oracle.rmse(hist, w, S)
    assert abs(r["chi2"] - ref_chi2) <= 1e-6 * max(ref_chi2, 1.0)
    assert abs(r["rmse"] - ref_rmse) <= 1e-6 * ref_rmse + 1e-15
    assert r["zero_weight_draws"] == int(hist[w == 0].sum())
    assert abs(r["total"] - w.astype(np.float64).sum()) <= 1e-12 * w.astype(np.float64).sum()
    again = st(None, ds, S, dw)
    assert again == r


def test_statistics_of_the_sampler(pkg, cuda):
    """The alias sampler's draws pass the on-device chi-square (df = N - 1) and never land on
    a zero-weight item; an out-of-range sample index is reported."""
    import torch
    from scipy.stats import chi2 as chi2_dist
    W = pkg.wrs
    N, S = 4096, 1 << 24
    w = weights_uniform(N, 8)
    w[::97] = 0.0
    cfg = pkg.AliasTableConfig(split_size=8, rng=W.RNG_PHILOX4X32_10,
                               scan_precision=W.SCAN_FLOAT_FLOAT, split_full_light=True)
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(N, S, cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, N)
    wrs.sample(None, bufs, N, S, 5)
    r = W.Statistics(N)(None, bufs.samples, S, bufs.weights)
    assert r["zero_weight_draws"] == 0
    df = int((w > 0).sum()) - 1
    assert chi2_dist.sf(r["chi2"], df) > 1e-4
    bad = torch.tensor([0, N + 5, 1], dtype=torch.int32, device="cuda")
    assert W.Statistics(N)(None, bad, 3, bufs.weights)["out_of_range"]
