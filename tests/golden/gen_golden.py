"""Generate the golden vectors in this directory from the reference's own CPU code.

Requires oracle/_ref/libwrs_ref.so (built by `make -C oracle ref` against a checkout of
the reference).  Run from the repository root:

    python tests/golden/gen_golden.py

Each fixture holds inputs and the reference's outputs for them:
  ref_pru_{N}.npz  (N = 1024, 8192; weights = the reference's PSEUDO_RANDOM_UNIFORM
                    generator, src/host/gen/weight_generator.h:75-87)
    weights              float32[N]
    mean                 float32   pivot used below (FP64 total mass / N, rounded once)
    kahan_prefix         reference::prefix_sum(weights)          (prefix_sum.hpp:17-34)
    partition            reference::stable_partition_indicies(weights, mean), with the
                         light run reversed into the device layout (partition.hpp:37-52)
    heavy_count
    heavy_prefix         reference::prefix_sum(heavy weights)
    light_prefix         reference::prefix_sum(light weights)
    psa_p, psa_a         reference::psa_alias_table(weights, K = N/32) (psa_alias_table.hpp:23-67)
    samples              a fixed uint32 sample vector (seeded numpy draw)
    chi_square, js       host::chi_square / host::js_divergence of those samples
                         (chi_square.hpp:17-37, js_divergence.hpp:48-92)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference, build_oracle  # noqa: E402


def main() -> None:
    build_oracle(ref=True)
    ref, orc = Reference(), Oracle()
    for N in (1024, 8192):
        w = ref.generate_weights(1, N)
        mean = np.float32(orc.mean(w))
        ridx, hc = ref.stable_partition_indices(w, mean)
        part = np.concatenate([ridx[:hc], ridx[hc:][::-1]]).astype(np.uint32)
        hp = ref.prefix_sum(w[ridx[:hc]])
        lp = ref.prefix_sum(w[ridx[hc:]])
        table = ref.psa_alias_table(w, N // 32)
        rng = np.random.default_rng(N)
        samples = rng.choice(N, size=4 * N, p=w.astype(np.float64) / w.astype(np.float64).sum())
        samples = samples.astype(np.uint32)
        np.savez_compressed(
            os.path.join(HERE, f"ref_pru_{N}.npz"),
            weights=w, mean=mean, kahan_prefix=ref.prefix_sum(w), partition=part,
            heavy_count=np.uint32(hc), heavy_prefix=hp, light_prefix=lp,
            psa_p=table["p"], psa_a=table["a"], samples=samples,
            chi_square=np.float32(ref.chi_square(samples, w)),
            js=np.float32(ref.js_divergence(samples, w)))
        print("wrote", f"ref_pru_{N}.npz")


if __name__ == "__main__":
    main()
