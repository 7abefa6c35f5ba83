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


def test_multinomial_chi2_variance():
    """The exact variance of Pearson's chi-square matches simulated multinomial draws at
    expected counts far below 5 (about 0.1 per item), where the chi-square distribution's
    2 (k - 1) is about half the true spread."""
    import bench
    rng = np.random.default_rng(3)
    k, s, reps = 200, 20, 20000
    p = rng.uniform(0.2, 1.0, k)
    p /= p.sum()
    e = s * p
    x2 = ((rng.multinomial(s, p, size=reps) - e) ** 2 / e).sum(1)
    var = bench.multinomial_chi2_var(p, s)
    assert var > 1.5 * 2 * (k - 1)
    assert abs(x2.mean() - (k - 1)) < 4 * np.sqrt(var / reps)
    assert abs(x2.var(ddof=1) / var - 1.0) < 0.08
    # zero-probability cells are left out, as the chi-square leaves them out
    assert bench.multinomial_chi2_var(np.concatenate([p, [0.0, 0.0]]), s) == var


def test_chi2_report_multinomial_fields():
    import bench
    r = bench.chi2_report(99.0, 99, 400.0)
    assert r["z_multinomial"] == 0.0 and abs(r["p_value_multinomial"] - 0.5) < 1e-12
    r = bench.chi2_report(99.0 + 2 * 20.0, 99, 400.0)
    assert abs(r["z_multinomial"] - 2.0) < 1e-12
    assert abs(r["p_value_multinomial"] - 0.022750131948179) < 1e-9
    assert "z_multinomial" not in bench.chi2_report(99.0, 99)


def test_binned_chi2_bins_and_variance():
    """Bins of G consecutive items with a mean expectation of at least the target; the bin
    probabilities p_binned gives are those the statistic uses."""
    import torch
    import bench
    n, s = 1000, 4000
    p = torch.full((n,), 1.0 / n, dtype=torch.float64)
    o = torch.bincount(torch.randint(0, n, (s,), generator=torch.Generator().manual_seed(1)),
                       minlength=n).double()
    r = bench.binned_chi2(o, p * s, 64.0)
    assert r["bin_items"] == 16 and r["df"] == (n + 15) // 16 - 1
    pb = bench.p_binned(p * s, 16)
    assert abs(float(pb.sum()) - 1.0) < 1e-12 and pb.numel() == 63
    assert "p_value_multinomial" in r


def test_profiled_traffic_reads_the_committed_capture():
    """The roofline's traffic comes from the committed ncu summary of the sampler with its coin
    filters, at the granularities captured there (64 B), and is absent at the others."""
    import bench
    t = bench.profiled_traffic(64)
    assert t is not None and 1e10 < t < 2e10
    assert bench.profiled_traffic(128) is None


def test_launches_per_step():
    """Six launches per headline step at N = 2^26 (mass, partition, split descent, split-pack,
    coin filter, sampling); no filter above 2^26, no descent for small grids."""
    import bench
    assert bench.launches_per_step(1 << 26) == 6
    assert bench.launches_per_step((1 << 26) + 5) == 5
    assert bench.launches_per_step(65536) == 4
