"""GPU tests of inputs outside the contract (weights must be finite and >= 0): NaN, +inf,
negative and all-zero weights.  The reference leaves these undefined; here every build ends
(no lookback wait runs out), every sample index is in range, and the calls report success:
the kernels' guards keep a corrupt partition or CMF from reading or writing out of bounds."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_uniform
from gpu_util import h2d, t2h

pytestmark = pytest.mark.gpu

N = 100_003
S = 1 << 18


def _cases():
    base = weights_uniform(N, 5)
    nan = base.copy()
    nan[::1000] = np.nan
    inf = base.copy()
    inf[777] = np.inf
    neg = base.copy()
    neg[::97] = -neg[::97]
    zero = np.zeros(N, np.float32)
    return {"nan": nan, "inf": inf, "negative": neg, "all_zero": zero}


@pytest.mark.parametrize("case", ["nan", "inf", "negative", "all_zero"])
@pytest.mark.parametrize("method", ["alias-ff", "alias-fp32", "its-comp", "its-fp32", "cutpoint"])
def test_out_of_contract_weights_stay_in_bounds(pkg, cuda, case, method):
    import torch
    W = pkg.wrs
    cfg = {
        "alias-ff": pkg.AliasTableConfig(split_size=12, rng=W.RNG_PHILOX4X32_10,
                                         scan_precision=W.SCAN_FLOAT_FLOAT,
                                         split_residual_f64=True, split_full_light=True),
        "alias-fp32": pkg.AliasTableConfig(),
        "its-comp": pkg.ITSConfig(rng=W.RNG_PHILOX4X32_10, scan_precision=W.SCAN_COMPENSATED),
        "its-fp32": pkg.ITSConfig(),
        "cutpoint": pkg.CutpointConfig(scan_precision=W.SCAN_COMPENSATED),
    }[method]
    w = _cases()[case]
    wrs = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(N, S, cfg, handle=wrs.handle)
    bufs.weights.copy_(h2d(w))
    wrs.build(None, bufs, N)
    wrs.sample(None, bufs, N, S, seed=3)
    status = bufs.internals.status()
    assert not status & W.DEVICE_TIMEOUT
    got = t2h(bufs.samples, np.uint32)[:S]
    assert int(got.max()) < N
