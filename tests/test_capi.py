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
    # the Cutpoint alternative of WRSConfig is not implemented
    assert L.wrs_config_init(C.byref(cfg), w.METHOD_CUTPOINT) == 5
    assert L.wrs_config_init(C.byref(cfg), 9) == 1
    assert L.wrs_config_init(None, 0) == 1
    bad = [
        w.WRSConfig(split_size=0),
        w.WRSConfig(method=w.METHOD_ITS, coop_size=8),  # ITS coop must be 0 or >= 32
        w.WRSConfig(coop_size=128, rng=w.RNG_PHILOX4X32_10),
        w.WRSConfig(rng=7),
        w.WRSConfig(scan_precision=3),
    ]
    for c in bad:
        with pytest.raises(w.WRSError) as e:
            w.Handle(c)
        assert e.value.status == 1
    with pytest.raises(w.WRSError) as e:
        w.Handle(w.WRSConfig(method=w.METHOD_CUTPOINT))
    assert e.value.status == 5
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
    assert L.wrs_version() == 100
    # a buffers object needs ~20 B per weight for the alias method, ~4 B for ITS
    n = 1 << 20
    assert 20 * n <= L.wrs_buffers_bytes(h.ptr, n) <= 21 * n + (1 << 20)
    hi = w.Handle(w.ITSConfig())
    assert 4 * n <= L.wrs_buffers_bytes(hi.ptr, n) <= 5 * n + (1 << 20)


def test_cpp_facade_compiles(pkg, tmp_path):
    """include/wrs.hpp (the C++ mirror of device::WRS) compiles against the C ABI."""
    src = tmp_path / "t.cpp"
    src.write_text('#include "wrs.hpp"\nint main() { wrs::WRSConfig c = wrs::AliasTableConfig(2);'
                   ' (void)c; return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
