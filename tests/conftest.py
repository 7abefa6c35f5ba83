"""Shared fixtures: the `gpu` marker, the oracle (CPU checker) and the product package.

CPU tests (-m "not gpu") check the oracle against the golden vectors and the reference's
own CPU code, the host logic and that the C-ABI library loads and exports its symbols.
GPU tests (-m gpu) are the parity tests proper: they drive the CUDA path through the C ABI
and compare with the oracle on the same inputs.
"""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build_oracle
    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("the reference's CPU code (oracle/_ref) is not built on this machine")
    return Reference()


@pytest.fixture(scope="session")
def pkg():
    """The product package, built for sm_103a (fails loudly if it cannot be built)."""
    m = importlib.import_module("merian-wrs_gb300")
    m.build()
    return m


@pytest.fixture(scope="session")
def cuda(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.init()
    return torch


def golden_path(name: str) -> str:
    return os.path.join(ROOT, "tests", "golden", name)


# ---- synthetic weights (the shapes of the benchmark configurations) -----------------

def weights_uniform(n: int, seed: int) -> np.ndarray:
    """uniform(0,1]: ((x >> 40) + 1) * 2^-24 from a seeded 64-bit generator."""
    x = np.random.default_rng(seed).integers(0, 2**64, size=n, dtype=np.uint64)
    return (((x >> np.uint64(40)) + np.uint64(1)).astype(np.float64) * 2.0**-24).astype(np.float32)


def weights_zipf(n: int, seed: int, s: float = 1.1) -> np.ndarray:
    """w_i = (i+1)^-s, randomly permuted."""
    w = np.power(np.arange(1, n + 1, dtype=np.float64), -s).astype(np.float32)
    return np.random.default_rng(seed).permutation(w)


def weights_lognormal(n: int, seed: int, mu: float = 0.0, sigma: float = 2.0) -> np.ndarray:
    z = np.random.default_rng(seed).standard_normal(n)
    return np.exp(mu + sigma * z).astype(np.float32)


def weights_precision(n: int, seed: int) -> np.ndarray:
    """log-normal(0, 3) with 1% forced to 0 and 0.01% scaled by 1e6."""
    rng = np.random.default_rng(seed)
    w = np.exp(3.0 * rng.standard_normal(n)).astype(np.float32)
    w[rng.random(n) < 0.01] = 0.0
    big = rng.random(n) < 1e-4
    w[big] = (w[big].astype(np.float64) * 1e6).astype(np.float32)
    return w
