"""GPU tests of the served request loop (wrs_server_*): continuous batching with resident
tables under a device memory budget.

Bar: every request completes with WRS_OK, and its samples equal those of the same request
computed alone (a batch of one, itself equal to per-call wrs_build + wrs_sample) bit for
bit -- whatever ran beside it, whether its table was built for it, reused while resident,
or rebuilt after an eviction.
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(pkg, n_requests, rate, budget, n_max, seed=5, reuse=0.3, recent=64):
    import torch
    W = pkg.wrs
    wl = importlib.import_module("merian-wrs_gb300.workloads").served(
        "cuda", n_requests, rate, seed=seed, n_max=n_max, s_max=4096, reuse=reuse,
        recent=recent, pool_log2=22)
    cfg = pkg.AliasTableConfig(split_size=8, rng=W.RNG_PHILOX4X32_10,
                               scan_precision=W.SCAN_FLOAT_FLOAT, split_residual_f64=True,
                               split_full_light=True)
    h = W.Handle(cfg)
    server = W.Server(h, memory_budget=budget, slots=3, max_batch_dists=64,
                      max_batch_weights=1 << 20, max_batch_samples=1 << 18)
    out = torch.full((int(wl["s_off"][-1]),), -1, dtype=torch.int32, device="cuda")
    wp, op = wl["w"].data_ptr(), out.data_ptr()
    rows = [(int(wl["table_id"][i]), wp + 4 * int(wl["w_off"][i]), op + 4 * int(wl["s_off"][i]),
             int(wl["n"][i]), int(wl["s"][i]), int(wl["seeds"][i])) for i in range(n_requests)]
    return W, wl, h, server, out, W.Server.requests(rows)


class Alone:
    """Requests recomputed one at a time (a batch of one)."""

    def __init__(self, W, h, wl):
        import torch
        self.wl = wl
        n, s = int(wl["n"].max()), int(wl["s"].max())
        self.b = W.Batch(h, 1, n, s)
        self.tab = torch.empty(2 * n, dtype=torch.int32, device="cuda")
        self.smp = torch.empty(s, dtype=torch.int32, device="cuda")

    def __call__(self, i):
        wl = self.wl
        n, s = int(wl["n"][i]), int(wl["s"][i])
        self.b.set(None, [(wl["w"].data_ptr() + 4 * int(wl["w_off"][i]), self.tab, self.smp, n,
                           s, int(wl["seeds"][i]))])
        self.b.build(None)
        self.b.sample(None)
        assert self.b.status() == 0
        return self.smp[:s]


def test_server_trace_alone_equals_mix(pkg, cuda):
    """A compressed Poisson trace through a small budget (evictions and rebuilds happen):
    every request's samples equal the request computed alone."""
    import torch
    n_req = 600
    W, wl, h, server, out, reqs = _setup(pkg, n_req, 2e5, 64 << 20, 1 << 17)
    comps = server.run_trace(reqs, [float(a) for a in wl["arrivals"]])
    torch.cuda.synchronize()
    st = server.stats()
    assert all(comps[i].status == 0 for i in range(n_req))
    assert st["completed"] == n_req and st["batches"] >= 2
    assert st["builds"] + st["reuses"] == n_req
    assert st["reuses"] > 0 and st["evictions"] > 0, st
    assert st["device_status"] == 0
    assert sum(comps[i].built for i in range(n_req)) == st["builds"]
    alone = Alone(W, h, wl)
    for i in range(n_req):
        assert comps[i].done_s >= comps[i].submit_s
        s, off = int(wl["s"][i]), int(wl["s_off"][i])
        assert torch.equal(out[off:off + s], alone(i)), i


def test_server_submit_progress_drains(pkg, cuda):
    """The incremental API: submit everything at once, call progress until nothing is
    pending; completions come back once each."""
    import torch
    n_req = 200
    W, wl, h, server, out, reqs = _setup(pkg, n_req, 1e6, 256 << 20, 1 << 16, seed=9)
    tickets = [server.submit(reqs[i]) for i in range(n_req)]
    assert tickets == list(range(n_req))
    seen = []
    for _ in range(100000):
        seen += [c.ticket for c in server.progress()]
        if server.pending() == 0:
            break
    torch.cuda.synchronize()
    assert sorted(seen) == tickets
    alone = Alone(W, h, wl)
    for i in (0, 1, n_req // 2, n_req - 1):
        s, off = int(wl["s"][i]), int(wl["s_off"][i])
        assert torch.equal(out[off:off + s], alone(i))


def test_server_rejects_bad_requests(pkg, cuda):
    W, wl, h, server, out, reqs = _setup(pkg, 4, 1e5, 64 << 20, 1 << 12)
    bad = W.Request(1, wl["w"].data_ptr(), out.data_ptr(), 10, 1, 0, 0)  # n = 0
    with pytest.raises(W.WRSError) as e:
        server.submit(bad)
    assert e.value.status == 1
    big = W.Request(1, wl["w"].data_ptr(), out.data_ptr(), 10, 1, (1 << 20) + 1, 0)
    with pytest.raises(W.WRSError):
        server.submit(big)  # n beyond max_batch_weights
    many = W.Request(1, wl["w"].data_ptr(), out.data_ptr(), (1 << 18) + 1, 1, 100, 0)
    with pytest.raises(W.WRSError):
        server.submit(many)  # s beyond max_batch_samples
