"""GPU test: the Philox4x32-10 stream against cuRAND as a library oracle.

cuRAND's `curandStatePhilox4_32_10_t` (curand_kernel.h, CUDA toolkit) with
`curand_init(seed, 0, 4 * g, &state)` produces, through `curand4`, the four words of
Random123 Philox4x32-10 at key (seed lo, seed hi) and counter (g lo, g hi, 0, 0) -- the
stream the RNG_PHILOX4X32_10 mode draws sample g from.  The test compiles a small cuRAND
kernel with nvcc, and checks (1) cuRAND's words against the oracle's restatement (itself
pinned to Random123's published known answers) and (2) the alias sampler's indices against
the index that cuRAND's first word selects (umulhi(x, N)) on a table of p = 1 entries."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SRC = r"""
#include <cstdint>
#include <curand_kernel.h>

__global__ void k_words(unsigned long long seed, unsigned long long offset, unsigned n,
                        uint4* out) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed, 0ull, 4ull * (offset + i), &st);
    out[i] = curand4(&st);
}

extern "C" int curand_philox_words(unsigned long long seed, unsigned long long offset,
                                   unsigned n, void* out) {
    k_words<<<(n + 255) / 256, 256>>>(seed, offset, n, static_cast<uint4*>(out));
    if (cudaGetLastError() != cudaSuccess) return 1;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}
"""


@pytest.fixture(scope="module")
def curand_lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    d = tmp_path_factory.mktemp("curand")
    src, lib = d / "curand_words.cu", d / "libcurand_words.so"
    src.write_text(SRC)
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared",
                        "-Xcompiler", "-fPIC", str(src), "-o", str(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(str(lib))
    L.curand_philox_words.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_void_p]
    L.curand_philox_words.restype = C.c_int
    return L


def _words(curand_lib, seed, offset, n):
    import torch
    out = torch.empty(4 * n, dtype=torch.int32, device="cuda")
    assert curand_lib.curand_philox_words(seed, offset, n, out.data_ptr()) == 0
    return out.cpu().numpy().view(np.uint32).reshape(n, 4)


@pytest.mark.parametrize("seed,offset", [(0, 0), (12345, 99), (0xDEADBEEFCAFEF00D, (1 << 32) - 7)])
def test_curand_philox_equals_the_oracle(pkg, cuda, oracle, curand_lib, seed, offset):
    n = 4096
    got = _words(curand_lib, seed, offset, n)
    key = [seed & 0xFFFFFFFF, seed >> 32]
    for i in list(range(0, n, 97)) + [n - 1]:
        g = offset + i
        assert oracle.philox4x32_10([g & 0xFFFFFFFF, g >> 32, 0, 0], key) == \
            [int(v) for v in got[i]], (seed, g)


def test_alias_sampler_draws_curands_indices(pkg, cuda, curand_lib):
    """With every entry at p = 1 (no alias taken) the Philox-mode alias sampler returns
    exactly the index cuRAND's first word selects: floor(x * N / 2^32)."""
    import torch
    W = pkg.wrs
    N, S, seed, offset = 1_000_003, 1 << 16, 777, 5
    table = torch.zeros(2 * N, dtype=torch.int32, device="cuda")
    t = table.view(torch.float32).view(N, 2)
    t[:, 0] = 1.0
    table.view(N, 2)[:, 1] = torch.arange(N, dtype=torch.int32, device="cuda")
    wrs = W.WRS(pkg.AliasTableConfig(rng=W.RNG_PHILOX4X32_10))
    out = torch.empty(S, dtype=torch.int32, device="cuda")
    wrs.alias_sample(None, table, N, S, seed, offset, out)
    torch.cuda.synchronize()
    x = _words(curand_lib, seed, offset, S)[:, 0].astype(np.uint64)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ((x * N) >> 32).astype(np.uint32))
