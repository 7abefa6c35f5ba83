"""GPU tests of the serial split-pack (ScalarSplit records + ScalarPack, and the warp-cooperative
SubgroupPack strategy): records and tables bit-exact against the oracle's restatement of
split/scalar/shader.comp and pack/scalar/float.comp given the GPU's partition arrays, the warp
strategy's table bit-identical to the scalar one, the record primitives equal to the build."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import weights_lognormal, weights_uniform, weights_zipf
from gpu_util import d2h, h2d
from oracle.oracle import ENTRY_DTYPE, SPLIT_DTYPE

pytestmark = pytest.mark.gpu

GENS = {"uniform": weights_uniform, "zipf": weights_zipf, "lognormal": weights_lognormal}


def _cfg(pkg, precision, mode, split, elems=True):
    W = pkg.wrs
    kw = dict(split_size=split, split_pack_mode=mode, use_partition_elements=elems)
    if precision == "fp32":
        return pkg.AliasTableConfig(**kw)
    if precision == "comp64":
        return pkg.AliasTableConfig(scan_precision=W.SCAN_COMPENSATED, split_residual_f64=True,
                                    **kw)
    return pkg.AliasTableConfig(scan_precision=W.SCAN_FLOAT_FLOAT, split_residual_f64=True,
                                split_full_light=True, **kw)


class Serial:
    """A serial-mode build read back: partition arrays, records and table."""

    def __init__(self, pkg, w, cfg):
        W = pkg.wrs
        self.wrs = W.WRS(cfg)
        self.N = w.size
        self.bufs = W.WRSBuffers.allocate(self.N, 1, cfg, handle=self.wrs.handle)
        self.bufs.weights.copy_(h2d(w))
        self.wrs.build(None, self.bufs, self.N)
        v = self.bufs.internals.views()
        self.status = self.bufs.internals.status()
        self.mean = float(d2h(v["mean"], 1, np.float32)[0])
        self.mean64 = float(d2h(v["mean64"], 1, np.float64)[0])
        self.hc = int(d2h(v["heavy_count"], 1, np.uint32)[0])
        self.idx = d2h(v["partition_indices"], self.N, np.uint32)
        self.prefix = d2h(v["partition_prefix"], self.N, np.float32)
        self.elems = (d2h(v["partition_elements"], self.N, np.float32)
                      if cfg.use_partition_elements else None)
        self.lo = (d2h(v["partition_prefix_lo"], self.N, np.float32)
                   if cfg.scan_precision == W.SCAN_FLOAT_FLOAT else None)
        self.K = W.lib().wrs_split_records_count(self.N, cfg.split_size)
        self.records = d2h(v["split_records"], self.K, SPLIT_DTYPE)
        self.table = d2h(v["alias_table"], self.N, ENTRY_DTYPE)
        self.views = v


FLAGS = {"fp32": 0, "comp64": 1, "ff": 3}


@pytest.mark.parametrize("N", [4097, 100003, (1 << 20) + 5])
@pytest.mark.parametrize("split", [2, 5, 32, 256])
@pytest.mark.parametrize("precision", ["fp32", "comp64", "ff"])
def test_serial_records_and_table_bit_exact(pkg, cuda, oracle, N, split, precision):
    W = pkg.wrs
    w = GENS[("uniform", "zipf", "lognormal")[(N + split) % 3]](N, N + split)
    b = Serial(pkg, w, _cfg(pkg, precision, W.SPLITPACK_SERIAL, split))
    assert b.status == 0
    assert b.K == -(-N // split)
    ref = oracle.scalar_split(b.prefix, b.hc, b.mean, split, flags=FLAGS[precision],
                              prefix_lo=b.lo, mean64=b.mean64)
    assert np.array_equal(b.records.view(np.uint32), ref.view(np.uint32))
    table = oracle.scalar_pack(w, b.idx, b.hc, b.mean, split, b.records, elems=b.elems,
                               flags=FLAGS[precision])
    assert np.array_equal(b.table.view(np.uint64), table.view(np.uint64))


@pytest.mark.parametrize("N", [4097, 300001, (1 << 22) + 17])
@pytest.mark.parametrize("split", [2, 32, 1000])
@pytest.mark.parametrize("elems", [True, False])
@pytest.mark.parametrize("precision", ["fp32", "ff"])
def test_warp_pack_equals_scalar_pack(pkg, cuda, oracle, N, split, elems, precision):
    """The warp-cooperative strategy writes the scalar pack's table from the same records and
    arrays, with and without partition elements (then the lanes gather the weights), FP32
    prefixes included (where splits step back and later subproblems override), with and
    without the table-end rule of the full light cap ("ff"); a build in the warp mode matches
    the oracle's scalar pack of its own records."""
    import torch
    W = pkg.wrs
    w = weights_lognormal(N, split + N)
    a = Serial(pkg, w, _cfg(pkg, precision, W.SPLITPACK_SERIAL, split, elems))
    assert a.status == 0
    warp = W.WRS(_cfg(pkg, precision, W.SPLITPACK_SERIAL_SUBGROUP, split, elems))
    v = a.views
    table = torch.zeros(2 * N, dtype=torch.int32, device="cuda")
    warp.pack(None, a.bufs.weights, v["partition_indices"],
              v["partition_elements"] if elems else None, v["split_records"], N, table,
              a.bufs.internals)
    torch.cuda.synchronize()
    assert a.bufs.internals.status() == 0
    assert np.array_equal(table.cpu().numpy().view(np.uint64), a.table.view(np.uint64))
    b = Serial(pkg, w, _cfg(pkg, precision, W.SPLITPACK_SERIAL_SUBGROUP, split, elems))
    assert b.status == 0
    ref = oracle.scalar_pack(w, b.idx, b.hc, b.mean, split, b.records, elems=b.elems,
                             flags=FLAGS[precision])
    assert np.array_equal(b.table.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("mode", [1, 2])
def test_record_primitives_equal_the_build(pkg, cuda, mode):
    """wrs_split / wrs_pack on the build's own partition arrays reproduce its records and
    table."""
    import torch
    W = pkg.wrs
    N, split = 250001, 12
    w = weights_zipf(N, 9)
    b = Serial(pkg, w, _cfg(pkg, "ff", mode, split))
    v = b.views
    rec = torch.zeros(3 * b.K, dtype=torch.int32, device="cuda")
    b.wrs.split(None, v["partition_prefix"], N, rec, b.bufs.internals,
                prefix_lo=v["partition_prefix_lo"])
    assert np.array_equal(rec.cpu().numpy().view(np.uint32), b.records.view(np.uint32))
    table = torch.zeros(2 * N, dtype=torch.int32, device="cuda")
    b.wrs.pack(None, b.bufs.weights, v["partition_indices"], v["partition_elements"], rec, N,
               table, b.bufs.internals)
    torch.cuda.synchronize()
    assert np.array_equal(table.cpu().numpy().view(np.uint64), b.table.view(np.uint64))


@pytest.mark.parametrize("mode", [1, 2])
def test_serial_degenerate_and_sampling(pkg, cuda, oracle, mode):
    """Equal weights (no heavy item) give the identity table; a serial-mode table samples
    like the inline one (chi-square)."""
    W = pkg.wrs
    N = 5000
    b = Serial(pkg, np.full(N, 0.5, np.float32), _cfg(pkg, "comp64", mode, 7))
    assert b.hc == 0
    assert np.all(b.table["a"] == np.arange(N)) and np.all(b.table["p"] == 1.0)
    w = weights_uniform(1 << 16, 3)
    b = Serial(pkg, w, _cfg(pkg, "ff", mode, 9))
    st = oracle.sample_stats(oracle.alias_sample(b.table, 1 << 20, 5, rng=1, nthreads=4), w)
    assert st["p_value"] > 1e-4, st


def test_serial_modes_rejected_where_unsupported(pkg, cuda):
    W = pkg.wrs
    cfg = _cfg(pkg, "ff", W.SPLITPACK_SERIAL, 8)
    with pytest.raises(W.WRSError) as e:
        W.Batch(W.Handle(cfg), 4, 1000, 1000)
    assert e.value.status == 5
    # buffers made for the inline mode hold no records
    inline = W.WRS(_cfg(pkg, "ff", W.SPLITPACK_INLINE, 8))
    serial = W.WRS(cfg)
    bufs = W.WRSBuffers.allocate(1000, 1, inline.config, handle=inline.handle)
    bufs.weights.copy_(h2d(weights_uniform(1000, 1)))
    with pytest.raises(W.WRSError) as e:
        serial.build(None, bufs, 1000)
    assert e.value.status == 1
