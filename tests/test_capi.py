"""CPU tests of the C-ABI library: it loads, exports every symbol include/wrs.h declares,
and validates configurations and arguments on the host (no call here reaches a GPU)."""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared_functions() -> list[str]:
    text = open(os.path.join(ROOT, "include", "wrs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wrs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.wrs.lib()
    declared = _declared_functions()
    assert len(declared) >= 25
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_build_targets_sm103a_only():
    import importlib
    b = importlib.import_module("merian-wrs_gb300.build")
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_config_defaults_and_validation(pkg):
    w = pkg.wrs
    L = w.lib()
    cfg = w._Config()
    assert L.wrs_config_init(C.byref(cfg), w.METHOD_ALIAS_TABLE) == 0
    assert (cfg.split_size, cfg.use_partition_elements, cfg.rng, cfg.coop_size) == (2, 1, 0, 0)
    assert L.wrs_config_init(C.byref(cfg), w.METHOD_ITS) == 0
    assert cfg.guiding_entry_size == 4  # the ITS search's cell size (0 = no cells)
    assert w.Handle(w.ITSConfig(guiding_entry_size=0, scan_precision=w.SCAN_COMPENSATED)).ptr
    # the Cutpoint alternative of WRSConfig (CutpointConfig(..., guidingEntrySize))
    assert L.wrs_config_init(C.byref(cfg), w.METHOD_CUTPOINT) == 0
    assert (cfg.method, cfg.guiding_entry_size, cfg.coop_size) == (w.METHOD_CUTPOINT, 32, 0)
    assert L.wrs_config_init(C.byref(cfg), 9) == 1
    assert L.wrs_config_init(None, 0) == 1
    bad = [
        w.WRSConfig(split_size=0),
        w.WRSConfig(method=w.METHOD_ITS, coop_size=8),  # ITS coop must be 0 or >= 32
        w.WRSConfig(coop_size=128, rng=w.RNG_PHILOX4X32_10),
        w.WRSConfig(rng=7),
        w.WRSConfig(scan_precision=3),
        w.CutpointConfig(guiding_entry_size=0),
        w.CutpointConfig(coop_size=64),  # the Cutpoint method has no cooperative size
        w.AliasTableConfig(split_pack_mode=3),  # unknown split-pack alternative
    ]
    for c in bad:
        with pytest.raises(w.WRSError) as e:
            w.Handle(c)
        assert e.value.status == 1
    assert w.Handle(w.CutpointConfig(128)).ptr
    h = w.Handle(w.AliasTableConfig(split_size=32, coop_size=128))
    assert h.ptr


def test_argument_validation_without_device_work(pkg):
    w = pkg.wrs
    L = w.lib()
    h = w.Handle(w.AliasTableConfig())
    out = C.c_void_p()
    assert L.wrs_buffers_create(h.ptr, 0, C.byref(out)) == 1
    assert L.wrs_buffers_create(h.ptr, 0x80000000, C.byref(out)) == 1
    assert L.wrs_build(h.ptr, None, None, 16, None) == 1
    assert L.wrs_alias_sample(h.ptr, None, None, 16, 16, 1, 0, None) == 1
    assert L.wrs_alias_sample(h.ptr, None, 8, 0, 16, 1, 0, 8) == 1  # n == 0
    assert b"NULL" in L.wrs_last_error() or b"range" in L.wrs_last_error()
    assert L.wrs_status_string(3) == b"a lookback wait gave up"
    cp = w.Handle(w.CutpointConfig())
    assert L.wrs_cutpoint_guide(cp.ptr, None, None, 16, None) == 1
    assert L.wrs_cutpoint_guide(h.ptr, None, 8, 16, 8) == 1  # alias handle
    assert L.wrs_cutpoint_sample(cp.ptr, None, 8, 0, 8, 16, 1, 0, 8) == 1  # n == 0
    assert L.wrs_version() == 100
    # a buffers object needs ~20 B per weight for the alias method, ~4 B for ITS (the CMF);
    # ITS with cells adds 32 B per cell (8 B per weight at the default cell size 4), and FP32
    # ITS above 2^16 weights the stored probe-tree blocks (2^20 weights: tree levels 0 .. 17,
    # 1 + 8 + 64 + 512 + 4096 + 32768 blocks of 32 B)
    n = 1 << 20
    assert 20 * n <= L.wrs_buffers_bytes(h.ptr, n) <= 21 * n + (1 << 20)
    tree = 32 * (585 + 4096 + 32768)
    plain = w.Handle(w.ITSConfig(guiding_entry_size=0))  # FP32, bisection only
    assert 4 * n + tree <= L.wrs_buffers_bytes(plain.ptr, n) <= 5 * n + tree + (1 << 20)
    assert L.wrs_buffers_bytes(plain.ptr, 1 << 16) <= 5 * (1 << 16) + (1 << 20)
    cells = w.Handle(w.ITSConfig())  # FP32, cells of 4 and the tree for marked cells
    assert 12 * n + tree <= L.wrs_buffers_bytes(cells.ptr, n) <= 13 * n + tree + (1 << 20)
    comp = w.Handle(w.ITSConfig(scan_precision=w.SCAN_COMPENSATED))  # cells alone
    assert 12 * n <= L.wrs_buffers_bytes(comp.ptr, n) <= 13 * n + (1 << 20)


def test_cpp_facade_compiles(pkg, tmp_path):
    """include/wrs.hpp (the C++ mirror of device::WRS) compiles against the C ABI."""
    src = tmp_path / "t.cpp"
    src.write_text('#include "wrs.hpp"\nint main() { wrs::WRSConfig c = wrs::AliasTableConfig(2);'
                   ' (void)c; return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_batch_argument_checks_on_host(pkg):
    """wrs_batch_* reject bad arguments before touching a GPU."""
    w = pkg.wrs
    L = w.lib()
    out = C.c_void_p()
    h = w.Handle(w.AliasTableConfig())
    assert L.wrs_batch_create(None, 1, 1, 1, C.byref(out)) == 1
    assert L.wrs_batch_create(h.ptr, 0, 1, 1, C.byref(out)) == 1       # max_dists = 0
    assert L.wrs_batch_create(h.ptr, 1 << 25, 1, 1, C.byref(out)) == 1  # too many
    its = w.Handle(w.ITSConfig())
    assert L.wrs_batch_create(its.ptr, 1, 1, 1, C.byref(out)) == 5     # alias method only
    assert L.wrs_batch_set(None, None, None, 0) == 1
    assert L.wrs_batch_build(h.ptr, None, None) == 1
    assert L.wrs_batch_sample(h.ptr, None, None) == 1
    assert L.wrs_batch_status(None, None, None) == 1
    assert L.wrs_batch_bytes(its.ptr, 1, 1, 1) == 0
    assert L.wrs_batch_bytes(h.ptr, 4096, 1 << 28, 1 << 30) > (1 << 28) * 12


def test_server_argument_checks_on_host(pkg):
    """wrs_server_* validate their configuration before touching a GPU."""
    w = pkg.wrs
    L = w.lib()
    c = w.ServerConfig()
    assert L.wrs_server_config_init(C.byref(c)) == 0
    assert (c.memory_budget, c.slots, c.max_batch_dists) == (16 << 30, 3, 1024)
    assert (c.max_batch_weights, c.max_batch_samples) == (1 << 25, 1 << 24)
    h = w.Handle(w.AliasTableConfig())
    out = C.c_void_p()
    assert L.wrs_server_create(None, C.byref(c), C.byref(out)) == 1
    bad = w.ServerConfig.from_buffer_copy(c)
    bad.slots = 0
    assert L.wrs_server_create(h.ptr, C.byref(bad), C.byref(out)) == 1
    small = w.ServerConfig.from_buffer_copy(c)
    small.memory_budget = 1 << 20  # below one slot's batch scratch
    assert L.wrs_server_create(h.ptr, C.byref(small), C.byref(out)) == 1
    its = w.Handle(w.ITSConfig())
    assert L.wrs_server_create(its.ptr, C.byref(c), C.byref(out)) == 1
    assert L.wrs_server_submit(None, None, None) == 1
    assert L.wrs_server_progress(None, None, 0, None) == 1
    assert L.wrs_server_pending(None) == 0


def test_server_table_arena(pkg):
    """The server's table arena (best fit over free blocks indexed by offset and by size):
    random allocations and releases never overlap, the byte count matches, and everything
    released coalesces back into one block -- host code, no device."""
    L = pkg.wrs.lib()
    for seed in (1, 2, 3):
        assert L.wrs_test_arena(seed, 100000) == 0


def test_served_workload_shape(pkg):
    """The served request stream: Poisson arrivals at the stated rate, N and S in range,
    about 30% of requests reuse an earlier table id, and a reused id keeps its n and its
    weights slice."""
    import importlib
    import numpy as np
    wl = importlib.import_module("merian-wrs_gb300.workloads").served(
        "cpu", 20000, 50000.0, seed=7, n_max=1 << 16, pool_log2=20)
    a = wl["arrivals"]
    assert np.all(np.diff(a) >= 0) and abs(len(a) / a[-1] - 50000.0) < 2500.0
    assert wl["n"].min() >= 256 and wl["n"].max() <= 1 << 16
    assert wl["s"].min() >= 1 and wl["s"].max() <= 65536
    reused = wl["table_id"] != np.arange(len(a))
    assert 0.27 < reused.mean() < 0.33
    for i in np.nonzero(reused)[0][:200]:
        j = wl["table_id"][i]
        assert wl["n"][i] == wl["n"][j] and wl["w_off"][i] == wl["w_off"][j]
    assert np.all(wl["w_off"] % 32 == 0) and wl["w"].numel() == 1 << 20


def test_statistics_and_probe_argument_checks_on_host(pkg):
    w = pkg.wrs
    L = w.lib()
    assert L.wrs_histogram(None, None, 5, 10, None, None) == 1
    assert L.wrs_histogram(None, 8, 5, 0, 8, 8) == 1           # n == 0
    assert L.wrs_statistics_scratch_bytes(1 << 20) >= 128 + 4 * 8 * 256
    assert L.wrs_sample_statistics(None, 8, 8, 10, 5, 8 + 64, 8) == 1  # misaligned scratch
    assert L.wrs_sample_statistics(None, 8, 8, 0, 5, 128, 8) == 1      # n == 0
    assert L.wrs_probe_random_gather(None, 256, 1 << 20, 16, 12, 8) == 1   # width 12
    assert L.wrs_probe_random_gather(None, 8, 1 << 20, 16, 16, 8) == 1    # misaligned buffer


def test_autotune_argument_checks_on_host(pkg):
    w = pkg.wrs
    L = w.lib()
    assert L.wrs_set_l2_fetch_granularity(200) == 1             # above 128 bytes
    assert L.wrs_get_l2_fetch_granularity(None) == 1
    res = w.TuneResult()
    alias = w.AliasTableConfig(split_size=8).c()
    its = w.ITSConfig().c()
    assert L.wrs_autotune_alias(None, None, 8, 16, 0, None, None, C.byref(res), None, 0) == 1
    assert L.wrs_autotune_alias(C.byref(its), None, 8, 16, 0, None, None, C.byref(res), None,
                                0) == 5                          # alias method only
    assert L.wrs_autotune_alias(C.byref(alias), None, None, 16, 0, None, None, C.byref(res),
                                None, 0) == 1                    # no weights
    assert L.wrs_autotune_alias(C.byref(alias), None, 8, 0, 0, None, None, C.byref(res), None,
                                0) == 1                          # n == 0
    assert L.wrs_autotune_alias(C.byref(alias), None, 8, 16, 4, None, None, C.byref(res), None,
                                0) == 1                          # samples without a buffer
    bad_l2, keep = w._tune_space(None, [64, 256], 1, 1)
    assert L.wrs_autotune_alias(C.byref(alias), None, 8, 16, 0, None, C.byref(bad_l2),
                                C.byref(res), None, 0) == 1      # L2 candidate above 128
    bad_split, keep2 = w._tune_space([0, 8], [], 1, 1)
    assert L.wrs_autotune_alias(C.byref(alias), None, 8, 16, 0, None, C.byref(bad_split),
                                C.byref(res), None, 0) == 1      # split size 0
    assert L.wrs_autotune_batch(C.byref(alias), None, None, 0, None, C.byref(res), None,
                                0) == 1                          # no distributions


def test_split_records_count(pkg):
    L = pkg.wrs.lib()
    assert L.wrs_split_records_count(1000, 7) == 143   # ceil(1000 / 7)
    assert L.wrs_split_records_count(1024, 32) == 32
    assert L.wrs_split_records_count(5, 32) == 1
    assert L.wrs_split_records_count(5, 0) == 0
