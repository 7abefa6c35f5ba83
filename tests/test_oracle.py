"""CPU tests of the oracle: pinned against the reference's own CPU code (golden vectors
generated by tests/golden/gen_golden.py, and live through oracle/_ref when it is built
here), against published known answers (Philox4x32-10) and against scipy (chi-square)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import (golden_path, weights_lognormal, weights_precision, weights_uniform,
                      weights_zipf)

GOLDEN = ("ref_pru_1024.npz", "ref_pru_8192.npz")


def _load(name):
    return dict(np.load(golden_path(name)))


# ---------------------------------------------------------------- golden vectors ---

@pytest.mark.parametrize("name", GOLDEN)
def test_golden_kahan_prefix_bit_exact(oracle, name):
    g = _load(name)
    got = oracle.prefix_kahan(g["weights"])
    assert np.array_equal(got.view(np.uint32), g["kahan_prefix"].view(np.uint32))


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_partition_bit_exact(oracle, name):
    g = _load(name)
    idx, elems, hc = oracle.partition(g["weights"], g["mean"])
    assert hc == int(g["heavy_count"])
    assert np.array_equal(idx, g["partition"])
    assert np.array_equal(elems, g["weights"][g["partition"]])


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_mean(oracle, name):
    g = _load(name)
    assert np.float32(oracle.mean(g["weights"])) == g["mean"]


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_split_satisfies_reference_crossing(oracle, name):
    """Every device-semantics split (n = k*s) satisfies the host split's crossing
    condition sigma <= target < sigma2 of src/host/reference/split.hpp:46-48, evaluated on
    the reference's own heavy/light Kahan prefixes."""
    g = _load(name)
    w, mean, hc = g["weights"], g["mean"], int(g["heavy_count"])
    hp, lp = g["heavy_prefix"], g["light_prefix"]
    prefix = np.concatenate([hp, lp[::-1]])
    N = w.size
    for s in (2, 32):
        _, (si, sj, ss) = oracle.split_pack(w, g["partition"], prefix, hc, mean, s,
                                            return_splits=True)
        for k in range(1, N // s):
            i, j = int(si[k]), int(sj[k])
            assert i + j == k * s or i == N - hc - 1
            target = np.float32(mean) * np.float32(k * s)
            heavy = np.float32(0) if j == 0 else hp[j - 1]
            light = np.float32(0) if i == 0 else lp[i - 1]
            assert np.float32(light + heavy) <= target
            assert np.float32(light + hp[j]) > target
            assert ss[k] == np.float32(np.float32(hp[j] + light) - target)


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_psa_table_matches_reference(oracle, name):
    """The oracle's PSA table (device semantics, split size 32, fed the reference's Kahan
    partition prefixes) encodes the same distribution as reference::psa_alias_table."""
    g = _load(name)
    w, mean, hc = g["weights"], g["mean"], int(g["heavy_count"])
    prefix = np.concatenate([g["heavy_prefix"], g["light_prefix"][::-1]])
    table = oracle.split_pack(w, g["partition"], prefix, hc, mean, 32)
    ref = np.zeros(w.size, table.dtype)
    ref["p"], ref["a"] = g["psa_p"], g["psa_a"]
    got_w = oracle.alias_to_weights(table)
    ref_w = oracle.alias_to_weights(ref)
    target = w.astype(np.float64) / w.astype(np.float64).mean()
    assert np.abs(got_w - target).max() < 1e-3
    assert np.abs(ref_w - target).max() < 1e-3
    assert np.abs(got_w - ref_w).max() < 2e-3  # both within 1e-3 of the target
    assert np.all(table["a"] < w.size)


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_statistics(oracle, name):
    g = _load(name)
    w, s = g["weights"], g["samples"]
    hist = oracle.histogram(s, w.size)
    assert oracle.chi_square(hist, w, s.size) == pytest.approx(float(g["chi_square"]), rel=1e-4)
    assert oracle.js_divergence(hist, w, s.size) == pytest.approx(float(g["js"]), rel=1e-3,
                                                                   abs=1e-7)


# ---------------------------------------------------------------- live reference ---

@pytest.mark.parametrize("N", [64, 1000, 4097, 65536])
def test_live_partition_and_prefix(oracle, reference, N):
    w = reference.generate_weights(1, N)
    mean = oracle.mean(w)
    idx, _, hc = oracle.partition(w, mean)
    ridx, rhc = reference.stable_partition_indices(w, mean)
    assert hc == rhc
    assert np.array_equal(idx, np.concatenate([ridx[:rhc], ridx[rhc:][::-1]]))
    kp = oracle.prefix_kahan(w)
    assert np.array_equal(kp.view(np.uint32), reference.prefix_sum(w).view(np.uint32))
    assert reference.assert_is_inclusive_prefix(w, kp) == (0, 0)
    # the FP64 prefix rounded once is an inclusive prefix for the reference's checker
    assert reference.assert_is_inclusive_prefix(w, oracle.prefix_f64(w).astype(np.float32)) == (0, 0)


@pytest.mark.parametrize("N,s", [(1024, 2), (1024, 32), (65536, 2), (65536, 32)])
def test_live_splits_and_tables_pass_reference_checkers(oracle, reference, N, s):
    w = reference.generate_weights(1, N)
    mean = oracle.mean(w)
    idx, _, hc = oracle.partition(w, mean)
    ridx, rhc = reference.stable_partition_indices(w, mean)
    hp = reference.prefix_sum(w[ridx[:rhc]])
    lp = reference.prefix_sum(w[ridx[rhc:]])
    prefix = np.concatenate([hp, lp[::-1]])
    table, (si, sj, ss) = oracle.split_pack(w, idx, prefix, hc, mean, s, return_splits=True)
    # the reference checker expects K splits whose last one is (lightCount, heavyCount-1)
    dsj = sj[1:].copy()
    dsj[-1] = hc - 1
    assert reference.assert_is_split(si[1:], dsj, ss[1:], hp, lp, mean, 1e-2) == (0, 0)
    assert reference.assert_is_alias_table(w, table, oracle.total_mass(w), 1e-2) == (0, 0)


def test_live_reference_sampling_semantics(oracle, reference):
    """host sample_single keeps u1 when u2 <= p (sample_alias_table.hpp:19); the device
    shader keeps ix when u.y < p.  They differ only at u2 == p exactly."""
    w = reference.generate_weights(1, 256)
    table, _, _ = oracle.psa_build(w, 4)
    for ix in (0, 17, 255):
        p = float(table["p"][ix])
        assert reference.sample_single(table, ix, np.float32(min(p, 1.0) * 0.5)) == ix
        if p < 1.0:
            assert reference.sample_single(table, ix, np.float32(np.nextafter(np.float32(p), 2))) \
                == table["a"][ix]


# ---------------------------------------------------------------- generators ---

def test_philox4x32_10_known_answers(oracle):
    """Random123's published known-answer vectors for philox4x32 with 10 rounds."""
    assert oracle.philox4x32_10([0, 0, 0, 0], [0, 0]) == \
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2) == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def _philox2x32_7_py(x0, x1, key):
    k = key
    for _ in range(7):
        m = x0 * 0xD256D193
        hi, lo = (m >> 32) & 0xFFFFFFFF, m & 0xFFFFFFFF
        x0, x1 = x1 ^ hi, (lo + k) & 0xFFFFFFFF
        k = (k + 0x9E3779B9) & 0xFFFFFFFF
    return x0, x1


def test_philox2x32_7_shader_variant(oracle):
    """src/device/wrs/alias/sampling/shader.comp:39-54 restated in pure Python."""
    rng = np.random.default_rng(0)
    for _ in range(200):
        c1, key = (int(v) for v in rng.integers(0, 2**32, 2))
        assert oracle.philox2x32_7(0, c1, key) == _philox2x32_7_py(0, c1, key)


def test_philox_uniform_operator(oracle):
    """The PRNG operator (src/device/prng/philox/shader.comp:47-55) restated in pure Python:
    element i = float(x1) / 2^32 of Philox2x32-7 at counter (i, 0), key = seed, the float
    conversion rounding to nearest (numpy's uint32 -> float32 conversion)."""
    for seed in (0, 12345, 0xFFFFFFFF):
        got = oracle.philox_uniform(seed, 1000)
        x1 = np.array([_philox2x32_7_py(i, 0, seed)[1] for i in range(1000)], np.uint32)
        want = x1.astype(np.float32) * np.float32(2.0 ** -32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        assert got.min() >= 0.0 and got.max() <= 1.0


def test_wang_hash(oracle):
    def py(s):
        s = (s ^ 61) ^ (s >> 16)
        s = (s * 9) & 0xFFFFFFFF
        s = s ^ (s >> 4)
        s = (s * 0x27d4eb2d) & 0xFFFFFFFF
        return s ^ (s >> 15)
    for s in (0, 1, 12345, 0xA9EC5C80, 0xFFFFFFFF):
        assert oracle.wang_hash(s) == py(s)


# ---------------------------------------------------------------- statistics ---

def test_chi2_sf_matches_scipy(oracle):
    scipy_stats = pytest.importorskip("scipy.stats")
    for df in (1, 5, 63, 1000, 65535, 2**20):
        for q in (0.01, 0.3, 0.5, 0.9, 0.999):
            x = float(scipy_stats.chi2.ppf(q, df))
            assert oracle.chi2_sf(x, df) == pytest.approx(1 - q, rel=1e-6, abs=1e-12)


def test_reference_split_tail_defect_and_fix(oracle):
    """With the shader's light cap (lightCount - 1) the last split of this log-normal input
    has i + j < n, the last heavy bucket aliases the last light item and that item gains one
    mean of mass; capping at lightCount (SPLIT_FULL_LIGHT) removes it."""
    from oracle.oracle import SPLIT_FULL_LIGHT
    w = weights_lognormal(4096, 11)
    target = w / w.astype(np.float64).mean()
    ref_table, _, _ = oracle.psa_build(w, 2)
    fix_table, _, _ = oracle.psa_build(w, 2, flags=SPLIT_FULL_LIGHT)
    ref_err = np.abs(oracle.alias_to_weights(ref_table) - target)
    fix_err = np.abs(oracle.alias_to_weights(fix_table) - target)
    # the light item gains the mass the last heavy bucket loses
    assert ref_err.max() > 0.9 and np.count_nonzero(ref_err > 0.1) == 2
    assert fix_err.max() < 1e-3


def _coarse_partition(oracle, w):
    """The stable partition with prefixes summed sequentially in FP32 (each class's running
    sum rounded at every step): prefixes far coarser than the device's, so that PSA's last
    subproblem runs out of heavy items before its light ones."""
    mean = np.float32(oracle.mean(w))
    idx, elems, hc = oracle.partition(w, mean)
    heavy = np.cumsum(elems[:hc], dtype=np.float32)
    light = np.cumsum(elems[hc:][::-1], dtype=np.float32)[::-1]
    return mean, idx, elems, hc, np.concatenate([heavy, light])


def test_table_end_rule_never_aliases_a_light_item(oracle):
    """When a PSA walk runs out of heavy items (the last heavy residual's rounding error),
    the shader's next heavy is the first light item: with the reference's table end the last
    light item -- here of weight zero -- is aliased by the last heavy bucket and by every
    light bucket packed after it.  The table-end rule of the full light cap keeps the last
    heavy item as (1, itself) and the later light buckets alias it: no entry aliases a light
    item and zero weights keep p = 0."""
    from oracle.oracle import SPLIT_FULL_LIGHT
    w = weights_precision(1 << 20, 5)
    w[-1] = 0.0  # the light item past the heavy range (position heavyCount)
    mean, idx, elems, hc, prefix = _coarse_partition(oracle, w)
    heavy = np.zeros(w.size, bool)
    heavy[idx[:hc]] = True
    zero = w == 0
    for flags in (0, SPLIT_FULL_LIGHT):
        table = oracle.split_pack(w, idx, prefix, hc, mean, 4, flags=flags, elems=elems)
        aliased = table["a"][table["p"] < 1]
        if flags:
            assert heavy[aliased].all()
            assert np.all(table["p"][zero] == 0)
            assert table["p"][idx[hc - 1]] == np.float32(1.0)
            assert table["a"][idx[hc - 1]] == idx[hc - 1]
        else:
            # the reference's table end: the item at position heavyCount is aliased
            assert np.count_nonzero(aliased == w.size - 1) >= 1
            assert not heavy[aliased].all()
    # a single subproblem walks the whole table: the same holds with split size >= N
    table = oracle.split_pack(w, idx, prefix, hc, mean, w.size, flags=SPLIT_FULL_LIGHT,
                              elems=elems)
    assert heavy[table["a"][table["p"] < 1]].all()


@pytest.mark.parametrize("gen", [weights_uniform, weights_zipf, weights_lognormal])
def test_oracle_psa_alias_sampling_is_unbiased(oracle, gen):
    """The oracle's own PSA build (light cap fixed) + alias sampling passes a chi-square
    test."""
    from oracle.oracle import SPLIT_FULL_LIGHT
    N, S = 4096, 1 << 20
    w = gen(N, 11)
    table, mean, hc = oracle.psa_build(w, 2, flags=SPLIT_FULL_LIGHT)
    rw = oracle.alias_to_weights(table)
    assert np.abs(rw - w / w.astype(np.float64).mean()).max() < 1e-3
    for rng in (0, 1):
        st = oracle.sample_stats(oracle.alias_sample(table, S, 7, rng=rng, nthreads=4), w)
        assert st["p_value"] > 1e-4, st


def test_oracle_its_sampling_is_unbiased(oracle):
    N, S = 4096, 1 << 20
    w = weights_uniform(N, 3)
    cmf = oracle.prefix_f64(w).astype(np.float32)
    for rng in (0, 1):
        st = oracle.sample_stats(oracle.its_sample(cmf, S, 9, rng=rng, nthreads=4), w)
        assert st["p_value"] > 1e-4, st


def test_oracle_threaded_equals_serial(oracle):
    w = weights_lognormal(20000, 5)
    t1, m1, h1 = oracle.psa_build(w, 2, nthreads=1)
    t4, m4, h4 = oracle.psa_build(w, 2, nthreads=4)
    assert m1 == m4 and h1 == h4
    assert np.abs(oracle.alias_to_weights(t1) - oracle.alias_to_weights(t4)).max() < 1e-3
    a1 = oracle.alias_sample(t1, 10000, 3, nthreads=1)
    a4 = oracle.alias_sample(t1, 10000, 3, nthreads=4)
    assert np.array_equal(a1, a4)


def test_cutpoint_oracle_against_numpy(oracle):
    """The oracle's guiding table is the lower bound of u_k = fl(fl(total / G) * k) in the CMF
    (numpy searchsorted on the same FP32 values), and each sample lies in the cell its group
    of 32 drew: [guide[k], guide[k+1]] (N - 1 for the last cell)."""
    import numpy as np
    from oracle.oracle import RNG_PHILOX4X32_10, RNG_REFERENCE
    rng = np.random.default_rng(3)
    for N, entry in [(1, 32), (7, 1), (1000, 32), (65537, 128)]:
        w = rng.random(N).astype(np.float32)
        w[rng.random(N) < 0.1] = 0.0
        cmf = oracle.prefix_kahan(w)
        G = (N + entry - 1) // entry
        step = np.float32(cmf[-1]) / np.float32(G)
        u = (step * np.arange(G, dtype=np.float32)).astype(np.float32)
        guide = oracle.cutpoint_guide(cmf, entry)
        assert np.array_equal(guide, np.searchsorted(cmf, u, side="left").astype(np.uint32))
        for r in (RNG_REFERENCE, RNG_PHILOX4X32_10):
            S = 3000
            s = oracle.cutpoint_sample(cmf, guide, S, 11, rng=r)
            assert s.max() < N
            again = oracle.cutpoint_sample(cmf, guide, S, 11, rng=r, nthreads=4)
            assert np.array_equal(s, again)
            # all 32 samples of a group come from one cell
            for g0 in range(0, S, 32):
                grp = s[g0:g0 + 32]
                ks = [k for k in range(G)
                      if guide[k] <= grp.min() and grp.max() <= (guide[k + 1] if k + 1 < G else N - 1)]
                assert ks, (N, entry, g0)


def test_cutpoint_reference_stream(oracle):
    """The reference mode draws u1 = wang_hash(seed + g0) for the cell and
    u2 = wang_hash((seed ^ 0x079145147) + g) inside it (cutpoint/sampling/shader.comp)."""
    import numpy as np
    N, entry, seed = 5000, 50, 777
    w = np.full(N, 1.0, np.float32)
    cmf = oracle.prefix_kahan(w)
    guide = oracle.cutpoint_guide(cmf, entry)
    G = guide.size
    s = oracle.cutpoint_sample(cmf, guide, 64, seed)
    for i in range(64):
        g0 = i & ~31
        u1 = np.float32(oracle.wang_hash(seed + g0)) * np.float32(2.0 ** -32)
        k = min(int(np.float32(u1) * np.float32(G)), G - 1)
        lo, hi = int(guide[k]), int(guide[k + 1]) if k + 1 < G else N - 1
        assert lo <= s[i] <= hi


# ------------------------------------------------------------ serial split-pack ---

@pytest.mark.parametrize("N,s", [(1024, 2), (1000, 7), (65536, 32), (65537, 5)])
def test_live_serial_split_records_pass_reference_checkers(oracle, reference, N, s):
    """ScalarSplit's records sit at n_k = ceil(N k / K), the positions the reference's
    assert_is_split checks, and ScalarPack's table from them passes assert_is_alias_table."""
    w = reference.generate_weights(1, N)
    mean = oracle.mean(w)
    idx, _, hc = oracle.partition(w, mean)
    ridx, rhc = reference.stable_partition_indices(w, mean)
    hp = reference.prefix_sum(w[ridx[:rhc]])
    lp = reference.prefix_sum(w[ridx[rhc:]])
    prefix = np.concatenate([hp, lp[::-1]])
    rec = oracle.scalar_split(prefix, hc, mean, s)
    assert rec.size == -(-N // s)
    assert (int(rec[-1]["i"]), int(rec[-1]["j"]), float(rec[-1]["spill"])) == (N - hc, hc, 0.0)
    dsj = rec["j"].copy()
    dsj[-1] = hc - 1  # the checker's last split (it checks records 0 .. K - 2)
    assert reference.assert_is_split(rec["i"].copy(), dsj, rec["spill"].copy(), hp, lp, mean,
                                     1e-2) == (0, 0)
    table = oracle.scalar_pack(w, idx, hc, mean, s, rec)
    assert reference.assert_is_alias_table(w, table, oracle.total_mass(w), 1e-2) == (0, 0)


@pytest.mark.parametrize("gen", [weights_uniform, weights_zipf, weights_lognormal])
@pytest.mark.parametrize("s", [2, 8, 64])
def test_serial_split_pack_equals_inline_when_n_divides(oracle, gen, s):
    """With N a multiple of the split size both split-packs cut at k * s: the records equal
    the inline splits and ScalarPack's table equals the inline table bit for bit; otherwise
    the tables still encode w / mean."""
    from oracle.oracle import SPLIT_FULL_LIGHT
    for N in (64 * s, 64 * s + 3):
        w = gen(N, 5 + s)
        mean = oracle.mean(w)
        idx, _, hc = oracle.partition(w, mean)
        prefix = oracle.partition_prefix_f64(w, mean).astype(np.float32)
        inline, (si, sj, ss) = oracle.split_pack(w, idx, prefix, hc, mean, s,
                                                 flags=SPLIT_FULL_LIGHT, return_splits=True)
        rec = oracle.scalar_split(prefix, hc, mean, s, flags=SPLIT_FULL_LIGHT)
        table = oracle.scalar_pack(w, idx, hc, mean, s, rec, flags=SPLIT_FULL_LIGHT)
        if N % s == 0:
            assert np.array_equal(rec["i"], si[1:]) and np.array_equal(rec["j"], sj[1:])
            assert np.array_equal(rec["spill"].view(np.uint32), ss[1:].view(np.uint32))
            assert np.array_equal(table.view(np.uint64), inline.view(np.uint64))
        implied = oracle.alias_to_weights(table)
        assert np.abs(implied - w / w.astype(np.float64).mean()).max() < 1e-3


def test_coin_filter_bound_never_changes_a_decision():
    """The alias sampler's coin filter stores q = floor(256 p) per bucket (255 for p >= 1, 0 for
    p <= 0 or NaN) and keeps a bucket early when the coin lies below q's bound.  The bound is
    below the keep threshold in both generator modes -- q * 2^24 <= ceil(p * 2^32) for the 32-bit
    Philox coin and q / 256 <= p for the shader's float coin -- so no early decision differs
    from the full one; checked over random FP32 bit patterns in [0, 2) and the edge values."""
    rng = np.random.default_rng(11)
    p = rng.integers(0, 0x40000000, 1 << 21, dtype=np.uint32).view(np.float32)
    edges = np.array([0.0, -0.0, 1.0, np.nextafter(np.float32(1), np.float32(0)), 1.0 / 256,
                      np.nextafter(np.float32(1.0 / 256), np.float32(0)), np.inf, np.nan, -1.0,
                      1e-45], dtype=np.float32)
    p = np.concatenate([p, edges])
    with np.errstate(invalid="ignore"):
        q = np.where(~(p > 0), 0, np.where(p >= 1, 255, np.floor(p.astype(np.float64) * 256)))
    q = q.astype(np.int64)
    assert q.min() >= 0 and q.max() <= 255
    with np.errstate(invalid="ignore"):
        below_one = (p > 0) & (p < 1)
    ceil_p = np.ceil(p[below_one].astype(np.float64) * 2.0 ** 32).astype(np.int64)
    assert np.all((q[below_one] << 24) <= ceil_p)
    assert np.all(q[below_one] / 256.0 <= p[below_one].astype(np.float64))
    # p >= 1 keeps every coin; its code's bound stays below 2^32 and below 1
    assert (255 << 24) < 2 ** 32 and 255 / 256 < 1
