"""The benchmark's CPU legs and configuration naming, on the CPU: the small configuration's CPU
path, the large configuration's CPU scan and ITS sampler, and the config's sizes (the driver's
benchmark run relies on each of them)."""
from __future__ import annotations

import numpy as np

from conftest import weights_uniform


def test_small_cpu_path_statistics():
    """The CPU path's histogram matches the weights, and against the same samples its RMSE to
    the GPU histogram is zero."""
    import bench
    from oracle.oracle import RNG_PHILOX4X32_10, Oracle
    w = weights_uniform(4096, 1)
    orc = Oracle()
    table, _, _ = orc.psa_build(w, 2, nthreads=1)
    s = 1 << 16
    same = orc.alias_sample(table, s, 1, rng=RNG_PHILOX4X32_10)
    r = bench.small_cpu_path(w, same, s)
    assert r["kind"] == "port" and r["cores"] == 1
    assert r["builds_per_s"] > 0 and r["samples_per_s"] > 0
    assert r["df"] == 4095 and 0.0 <= r["p_value"] <= 1.0
    assert r["rmse_gpu_vs_cpu_histogram"] == 0.0


def test_cpu_scan_its():
    import bench
    w = weights_uniform(1 << 16, 2)
    r = bench.cpu_scan_its(w, 2, s=1 << 12)
    assert r["weights_scanned_per_s"] > 0 and r["its_samples_per_s"] > 0
    assert r["scan_cores"] == 1 and r["its_cores"] == 2


def test_headline_config_names_its_sizes():
    import bench
    full = bench.headline_config(1 << bench.LOG2_N, 1 << bench.LOG2_S, 1)
    assert full["workload"] == bench.WORKLOAD
    small = bench.headline_config(1 << 20, 1 << 22, 2)
    assert "N=2^20" in small["workload"] and "S=2^22" in small["workload"]
    assert "2^26" not in small["workload"] and small["parallelism"] == "replicas x2"
    assert np.all([small["N"] == 1 << 20, small["S"] == 1 << 22])
