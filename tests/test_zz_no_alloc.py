"""GPU test of wrs_prefix_sum_noalloc, the prefix sum for callers that cannot allocate device
memory (for example code running under an application whose pool already holds all device
memory, or code that must avoid the device-wide synchronisation of cudaMalloc).

For both carries it runs the no-allocation scan several times in a row on different inputs
through the C ABI -- among them n = 2^26, the scratch's limit -- and checks each result
against the regular wrs_prefix_sum (which takes its scratch from a wrs_buffers object): bit
for bit with the compensated carry (exact fixed-point carries make the CMF a deterministic
function of the weights), within the scan tests' FP32-carry bound otherwise.  After the
first call (which may load the library's device module) the device's free memory must not
move across calls, and sizes beyond the limit are refused with a clear error.  This file is
collected last so that a run stopping at the first failure has already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform, weights_zipf
from gpu_util import empty, h2d, t2h

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "compensated"])
def test_prefix_sum_noalloc_matches_prefix_sum(pkg, cuda, precision):
    import torch
    W = pkg.wrs
    L = W.lib()
    prec = W.SCAN_COMPENSATED if precision == "compensated" else W.SCAN_FP32
    its = W.WRS(pkg.ITSConfig(scan_precision=prec))
    cases = [(weights_lognormal, (1 << 22) + 3), (weights_uniform, 1000003),
             (weights_zipf, 1 << 26), (weights_uniform, 1 << 26), (weights_lognormal, 8191)]
    nmax = max(n for _, n in cases)
    internals = W.Internals(its.handle, nmax)
    ref, out = empty(nmax), empty(nmax)
    status = empty(1, "i32")
    first = True
    for k, (gen, n) in enumerate(cases):
        w = gen(n, 40 + k)
        dw = h2d(w)
        # the regular entry point, scratch from a wrs_buffers object
        its.prefix_sum(None, dw, n, ref, internals)
        assert internals.status() == 0
        # the no-allocation entry point
        status.fill_(-1)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        W.check(L.wrs_prefix_sum_noalloc(None, dw.data_ptr(), n, out.data_ptr(), prec,
                                         status.data_ptr()))
        torch.cuda.synchronize()
        free = torch.cuda.mem_get_info()[0]
        if not first:
            assert free == free_before, f"call {k}: device memory moved"
        first = False
        assert int(t2h(status, np.uint32)[0]) == 0
        got = t2h(out[:n], np.float32)
        want = t2h(ref[:n], np.float32)
        exact = np.cumsum(w.astype(np.float64))
        if prec == W.SCAN_COMPENSATED:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"call {k}"
            assert np.all(np.abs(got - exact) <= 1e-6 * exact + 1e-30), f"call {k}"
        else:
            # FP32 carries: every element within the FP32 carry's bound of the exact scan
            assert np.all(np.abs(got - exact) <= 1e-4 * exact[-1]), f"call {k}"
            assert np.all(np.abs(got - want) <= 1e-4 * exact[-1]), f"call {k}"
        del dw

    # beyond the scratch's limit: refused before any GPU work
    rc = L.wrs_prefix_sum_noalloc(None, out.data_ptr(), (1 << 26) + 1, out.data_ptr(), prec,
                                  None)
    assert rc == 6  # WRS_ERR_CAPACITY
    assert b"2^26" in L.wrs_last_error()
