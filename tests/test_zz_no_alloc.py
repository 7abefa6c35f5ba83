"""GPU test of wrs_prefix_sum_noalloc, the prefix sum for callers that cannot allocate device
memory (for example code running under an application whose pool already holds all device
memory, or code that must avoid the device-wide synchronisation of cudaMalloc).

It runs the no-allocation scan twice in a row on different inputs through the C ABI and
checks each result against the regular wrs_prefix_sum (which takes its scratch from a
wrs_buffers object) with the scan tests' tolerance: relative 1e-6 with the compensated
carry.  It also checks that sizes beyond the scratch's 2^26-weight limit are refused with a
clear error.  This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform
from gpu_util import empty, h2d, t2h

pytestmark = pytest.mark.gpu


def test_prefix_sum_noalloc_matches_prefix_sum(pkg, cuda):
    W = pkg.wrs
    L = W.lib()
    its = W.WRS(pkg.ITSConfig(scan_precision=W.SCAN_COMPENSATED))
    cases = [(weights_lognormal, (1 << 22) + 3), (weights_uniform, 1000003)]
    for k, (gen, n) in enumerate(cases):
        w = gen(n, 40 + k)
        dw = h2d(w)
        # the regular entry point, scratch from a wrs_buffers object
        ref = empty(n)
        internals = W.Internals(its.handle, n)
        its.prefix_sum(None, dw, n, ref, internals)
        assert internals.status() == 0
        # the no-allocation entry point
        out = empty(n)
        status = empty(1, "i32")
        status.fill_(-1)
        W.check(L.wrs_prefix_sum_noalloc(None, dw.data_ptr(), n, out.data_ptr(),
                                         W.SCAN_COMPENSATED, status.data_ptr()))
        got = t2h(out, np.float32).astype(np.float64)
        want = t2h(ref, np.float32).astype(np.float64)
        assert int(t2h(status, np.uint32)[0]) == 0
        assert np.all(np.abs(got - want) <= 1e-6 * np.abs(want) + 1e-30), f"call {k}"
        exact = np.cumsum(w.astype(np.float64))
        assert np.all(np.abs(got - exact) <= 1e-6 * exact + 1e-30), f"call {k}"

    # beyond the scratch's limit: refused before any GPU work
    rc = L.wrs_prefix_sum_noalloc(None, dw.data_ptr(), (1 << 26) + 1, out.data_ptr(),
                                  W.SCAN_COMPENSATED, None)
    assert rc == 6  # WRS_ERR_CAPACITY
    assert b"2^26" in L.wrs_last_error()
