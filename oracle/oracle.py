"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

`Oracle` wraps oracle/libwrs_oracle.so, the plain-C restatement of the
reference's device shaders (see wrs_oracle.c for the file:line of each
function).  `Reference` wraps oracle/_ref/libwrs_ref.so, the reference's own
header-only CPU code compiled from its sources.  Only tests/, the smoke check
and the CPU legs of bench.py import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ENTRY_DTYPE = np.dtype([("p", "<f4"), ("a", "<u4")])
SPLIT_DTYPE = np.dtype([("i", "<u4"), ("j", "<u4"), ("spill", "<f4")])  # wrs_split_record

RNG_REFERENCE = 0
RNG_PHILOX4X32_10 = 1
SPLIT_F64 = 1          # split-point residual (spill) in FP64
SPLIT_FULL_LIGHT = 2   # light count capped at lightCount (not the shader's lightCount - 1)
SPLIT_FLOAT_FLOAT = 4  # psa_build: float-float partition prefix for the split search


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the oracle must be contiguous"
    return a.ctypes.data_as(C.c_void_p)


def build_oracle(ref: bool = False) -> None:
    """Compile libwrs_oracle.so (and, when asked and the reference is present, _ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _load(path: str) -> C.CDLL:
    return C.CDLL(path)


class Oracle:
    """CPU restatement of the reference's device arithmetic."""

    _lib: C.CDLL | None = None

    def __init__(self) -> None:
        if Oracle._lib is None:
            path = os.path.join(HERE, "libwrs_oracle.so")
            if not os.path.exists(path):
                build_oracle()
            lib = _load(path)
            vp, u32, u64, f32, f64, i32 = (C.c_void_p, C.c_uint32, C.c_uint64, C.c_float,
                                           C.c_double, C.c_int)
            sig = {
                "wrso_philox2x32_7": (None, [u32, u32, u32, vp]),
                "wrso_philox4x32_10": (None, [vp, vp, vp]),
                "wrso_wang_hash": (u32, [u32]),
                "wrso_philox_uniform": (None, [u32, u32, vp]),
                "wrso_unit_ref": (f32, [u32]),
                "wrso_total_mass": (f64, [vp, u64]),
                "wrso_mean": (f32, [vp, u64]),
                "wrso_partition": (None, [vp, u32, f32, vp, vp, vp]),
                "wrso_partition_prefix_f64": (None, [vp, u32, f32, vp]),
                "wrso_prefix_f64": (None, [vp, u64, vp]),
                "wrso_prefix_kahan": (None, [vp, u64, vp]),
                "wrso_prefix_seq_f32": (None, [vp, u64, vp]),
                "wrso_split": (None, [vp, vp, u32, u32, f32, f64, u32, i32, vp, vp, vp]),
                "wrso_split_pack": (None, [vp, vp, vp, vp, vp, u32, f32, f64, u32, u32, i32, vp,
                                           vp]),
                "wrso_split_pack_mt": (None, [vp, vp, vp, vp, vp, u32, f32, f64, u32, u32, i32,
                                              i32, vp, vp]),
                "wrso_psa_build": (None, [vp, u32, u32, i32, i32, vp, vp, vp]),
                "wrso_scalar_split": (None, [vp, vp, u32, u32, f32, f64, u32, i32, vp]),
                "wrso_scalar_pack": (None, [vp, vp, vp, u32, f32, u32, u32, i32, vp, vp]),
                "wrso_alias_sample": (None, [vp, u32, u64, u64, u64, u32, u32, i32, vp]),
                "wrso_its_sample": (None, [vp, u32, u64, u64, u64, u32, u32, i32, i32, vp]),
                "wrso_cutpoint_guide": (None, [vp, u32, u32, vp]),
                "wrso_cutpoint_sample": (None, [vp, u32, vp, u32, u64, u64, u64, u32, i32, vp]),
                "wrso_histogram": (None, [vp, u64, u32, vp]),
                "wrso_chi_square": (f64, [vp, vp, u32, u64]),
                "wrso_chi_square_binned": (f64, [vp, vp, u32, u64, f64, vp]),
                "wrso_chi2_sf": (f64, [f64, f64]),
                "wrso_rmse": (f64, [vp, vp, u32, u64]),
                "wrso_js_divergence": (f64, [vp, vp, u32, u64]),
                "wrso_alias_to_weights": (None, [vp, u32, vp]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            Oracle._lib = lib
        self.lib = Oracle._lib

    # -- generators -------------------------------------------------------------
    def philox2x32_7(self, c0: int, c1: int, key: int) -> tuple[int, int]:
        out = np.zeros(2, np.uint32)
        self.lib.wrso_philox2x32_7(c0, c1, key, _ptr(out))
        return int(out[0]), int(out[1])

    def philox4x32_10(self, ctr, key) -> list[int]:
        c = np.asarray(ctr, np.uint32)
        k = np.asarray(key, np.uint32)
        out = np.zeros(4, np.uint32)
        self.lib.wrso_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
        return [int(x) for x in out]

    def philox_uniform(self, seed: int, n: int) -> np.ndarray:
        """The PRNG operator's n floats (prng/philox/shader.comp:47-55)."""
        out = np.empty(n, np.float32)
        self.lib.wrso_philox_uniform(seed & 0xFFFFFFFF, n, _ptr(out))
        return out

    def wang_hash(self, x: int) -> int:
        return int(self.lib.wrso_wang_hash(x & 0xFFFFFFFF))

    # -- build ------------------------------------------------------------------
    def total_mass(self, w: np.ndarray) -> float:
        w = np.ascontiguousarray(w, np.float32)
        return float(self.lib.wrso_total_mass(_ptr(w), w.size))

    def mean(self, w: np.ndarray) -> float:
        w = np.ascontiguousarray(w, np.float32)
        return float(np.float32(self.lib.wrso_mean(_ptr(w), w.size)))

    def partition(self, w: np.ndarray, pivot: float):
        w = np.ascontiguousarray(w, np.float32)
        idx = np.empty(w.size, np.uint32)
        elems = np.empty(w.size, np.float32)
        hc = np.zeros(1, np.uint32)
        self.lib.wrso_partition(_ptr(w), w.size, np.float32(pivot), _ptr(idx), _ptr(elems),
                                _ptr(hc))
        return idx, elems, int(hc[0])

    def partition_prefix_f64(self, w: np.ndarray, pivot: float) -> np.ndarray:
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.float64)
        self.lib.wrso_partition_prefix_f64(_ptr(w), w.size, np.float32(pivot), _ptr(out))
        return out

    def prefix_f64(self, w: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.float64)
        self.lib.wrso_prefix_f64(_ptr(w), w.size, _ptr(out))
        return out

    def prefix_kahan(self, w: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.float32)
        self.lib.wrso_prefix_kahan(_ptr(w), w.size, _ptr(out))
        return out

    def prefix_seq_f32(self, w: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.float32)
        self.lib.wrso_prefix_seq_f32(_ptr(w), w.size, _ptr(out))
        return out

    def split(self, prefix: np.ndarray, heavy_count: int, mean: float, n: int, flags: int = 0,
              prefix_lo: np.ndarray | None = None, mean64: float = 0.0):
        prefix = np.ascontiguousarray(prefix, np.float32)
        lo = None if prefix_lo is None else np.ascontiguousarray(prefix_lo, np.float32)
        i = np.zeros(1, np.uint32)
        j = np.zeros(1, np.uint32)
        s = np.zeros(1, np.float32)
        self.lib.wrso_split(_ptr(prefix), _ptr(lo), prefix.size, heavy_count, np.float32(mean),
                            float(mean64), n, flags, _ptr(i), _ptr(j), _ptr(s))
        return int(i[0]), int(j[0]), np.float32(s[0])

    def split_pack(self, w, idx, prefix, heavy_count, mean, split_size, flags=0, elems=None,
                   return_splits=False, prefix_lo=None, mean64=0.0, nthreads=1):
        """prefix_lo / mean64: the float-float mode's low words and FP64 mean; nthreads
        spreads the split searches (the table does not depend on it)."""
        w = np.ascontiguousarray(w, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        prefix = np.ascontiguousarray(prefix, np.float32)
        lo = None if prefix_lo is None else np.ascontiguousarray(prefix_lo, np.float32)
        N = w.size
        table = np.zeros(N, ENTRY_DTYPE)
        K = max(N // split_size, 1)
        splits = np.zeros(3 * (K + 1), np.uint32) if return_splits else None
        self.lib.wrso_split_pack_mt(_ptr(w), _ptr(idx),
                                    _ptr(np.ascontiguousarray(elems, np.float32))
                                    if elems is not None else None,
                                    _ptr(prefix), _ptr(lo), heavy_count, np.float32(mean),
                                    float(mean64), N, split_size, flags, int(nthreads),
                                    _ptr(table), _ptr(splits))
        if return_splits:
            sp = splits.reshape(K + 1, 3)
            return table, (sp[:, 0].copy(), sp[:, 1].copy(), sp[:, 2].view(np.float32).copy())
        return table

    def scalar_split(self, prefix, heavy_count, mean, split_size, flags=0, prefix_lo=None,
                     mean64=0.0):
        """ScalarSplit's ceil(N / split_size) records as a SPLIT_DTYPE array."""
        prefix = np.ascontiguousarray(prefix, np.float32)
        lo = None if prefix_lo is None else np.ascontiguousarray(prefix_lo, np.float32)
        N = prefix.size
        K = max((N + split_size - 1) // split_size, 1)
        rec = np.zeros(K, SPLIT_DTYPE)
        self.lib.wrso_scalar_split(_ptr(prefix), _ptr(lo), N, heavy_count, np.float32(mean),
                                   float(mean64), split_size, flags, _ptr(rec))
        return rec

    def scalar_pack(self, w, idx, heavy_count, mean, split_size, records, elems=None, flags=0):
        """ScalarPack from split records (SPLIT_DTYPE); flags & SPLIT_FULL_LIGHT applies the
        table-end rule of the full light cap."""
        w = np.ascontiguousarray(w, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        rec = np.ascontiguousarray(records, SPLIT_DTYPE)
        table = np.zeros(w.size, ENTRY_DTYPE)
        self.lib.wrso_scalar_pack(_ptr(w), _ptr(idx),
                                  _ptr(np.ascontiguousarray(elems, np.float32))
                                  if elems is not None else None,
                                  heavy_count, np.float32(mean), w.size, split_size, int(flags),
                                  _ptr(rec), _ptr(table))
        return table

    def psa_build(self, w, split_size=2, nthreads=1, flags=0):
        w = np.ascontiguousarray(w, np.float32)
        table = np.zeros(w.size, ENTRY_DTYPE)
        mean = np.zeros(1, np.float32)
        hc = np.zeros(1, np.uint32)
        self.lib.wrso_psa_build(_ptr(w), w.size, split_size, flags, nthreads, _ptr(table), _ptr(mean),
                                _ptr(hc))
        return table, float(mean[0]), int(hc[0])

    # -- sampling ---------------------------------------------------------------
    def alias_sample(self, table, S, seed, rng=RNG_REFERENCE, coop=0, offset=0, nthreads=1):
        table = np.ascontiguousarray(table, ENTRY_DTYPE)
        out = np.empty(S, np.uint32)
        self.lib.wrso_alias_sample(_ptr(table), table.size, S, seed, offset, rng, coop,
                                   nthreads, _ptr(out))
        return out

    def its_sample(self, cmf, S, seed, rng=RNG_REFERENCE, coop=0, parray=False, offset=0,
                   nthreads=1):
        cmf = np.ascontiguousarray(cmf, np.float32)
        out = np.empty(S, np.uint32)
        self.lib.wrso_its_sample(_ptr(cmf), cmf.size, S, seed, offset, rng, coop, int(parray),
                                 nthreads, _ptr(out))
        return out

    def cutpoint_guide(self, cmf, entry_size: int):
        cmf = np.ascontiguousarray(cmf, np.float32)
        G = (cmf.size + entry_size - 1) // entry_size
        guide = np.empty(G, np.uint32)
        self.lib.wrso_cutpoint_guide(_ptr(cmf), cmf.size, G, _ptr(guide))
        return guide

    def cutpoint_sample(self, cmf, guide, S, seed, rng=RNG_REFERENCE, offset=0, nthreads=1):
        cmf = np.ascontiguousarray(cmf, np.float32)
        guide = np.ascontiguousarray(guide, np.uint32)
        out = np.empty(S, np.uint32)
        self.lib.wrso_cutpoint_sample(_ptr(cmf), cmf.size, _ptr(guide), guide.size, S, seed,
                                      offset, rng, nthreads, _ptr(out))
        return out

    # -- statistics -------------------------------------------------------------
    def histogram(self, samples, N):
        samples = np.ascontiguousarray(samples, np.uint32)
        hist = np.zeros(N, np.uint64)
        self.lib.wrso_histogram(_ptr(samples), samples.size, N, _ptr(hist))
        return hist

    def chi_square(self, hist, w, S):
        w = np.ascontiguousarray(w, np.float32)
        hist = np.ascontiguousarray(hist, np.uint64)
        return float(self.lib.wrso_chi_square(_ptr(hist), _ptr(w), w.size, S))

    def chi_square_binned(self, hist, w, S, min_expected=5.0):
        w = np.ascontiguousarray(w, np.float32)
        hist = np.ascontiguousarray(hist, np.uint64)
        bins = np.zeros(1, np.uint64)
        chi2 = float(self.lib.wrso_chi_square_binned(_ptr(hist), _ptr(w), w.size, S,
                                                     min_expected, _ptr(bins)))
        return chi2, int(bins[0])

    def chi2_sf(self, x, df):
        return float(self.lib.wrso_chi2_sf(float(x), float(df)))

    def rmse(self, hist, w, S):
        w = np.ascontiguousarray(w, np.float32)
        hist = np.ascontiguousarray(hist, np.uint64)
        return float(self.lib.wrso_rmse(_ptr(hist), _ptr(w), w.size, S))

    def js_divergence(self, hist, w, S):
        w = np.ascontiguousarray(w, np.float32)
        hist = np.ascontiguousarray(hist, np.uint64)
        return float(self.lib.wrso_js_divergence(_ptr(hist), _ptr(w), w.size, S))

    def alias_to_weights(self, table):
        table = np.ascontiguousarray(table, ENTRY_DTYPE)
        out = np.empty(table.size, np.float64)
        self.lib.wrso_alias_to_weights(_ptr(table), table.size, _ptr(out))
        return out

    def sample_stats(self, samples, w, min_expected=5.0):
        """chi-square (binned), its p-value, RMSE and JS divergence of a sample set."""
        w = np.ascontiguousarray(w, np.float32)
        S = int(samples.size)
        hist = self.histogram(samples, w.size)
        chi2, bins = self.chi_square_binned(hist, w, S, min_expected)
        df = max(bins - 1, 1)
        return {
            "chi2": chi2,
            "df": df,
            "p_value": self.chi2_sf(chi2, df),
            "rmse": self.rmse(hist, w, S),
            "js": self.js_divergence(hist, w, S),
        }


class Reference:
    """The reference's own CPU code (oracle/_ref), when it was compiled here."""

    _lib: C.CDLL | None = None

    @staticmethod
    def path() -> str:
        return os.path.join(HERE, "_ref", "libwrs_ref.so")

    @staticmethod
    def available() -> bool:
        p = Reference.path()
        if not os.path.exists(p):
            return False
        try:
            _load(p)
            return True
        except OSError:
            return False

    def __init__(self) -> None:
        if Reference._lib is None:
            lib = _load(Reference.path())
            vp, u32, u64, f32, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
            sig = {
                "ref_generate_weights": (i32, [i32, u32, vp]),
                "ref_psa_alias_table": (None, [vp, u32, u32, vp, vp]),
                "ref_prefix_sum": (None, [vp, u64, vp]),
                "ref_kahan_reduction": (f32, [vp, u64]),
                "ref_stable_partition_indices": (None, [vp, u32, f32, vp, vp]),
                "ref_split": (None, [vp, u32, vp, u32, f32, u32, vp, vp, vp]),
                "ref_splitK": (None, [vp, u32, vp, u32, f32, u32, u32, vp, vp, vp]),
                "ref_pack_splits": (None, [vp, u32, vp, u32, vp, u32, f32, vp, vp, vp, u32, vp,
                                           vp]),
                "ref_alias_to_normalized_weights": (None, [vp, vp, u32, vp]),
                "ref_assert_is_alias_table": (i32, [vp, u32, vp, vp, f32, f32, vp]),
                "ref_assert_is_inclusive_prefix": (i32, [vp, vp, u64, vp]),
                "ref_assert_is_split": (i32, [vp, vp, vp, u32, vp, u32, vp, u32, f32, f32, vp]),
                "ref_chi_square": (f32, [vp, u64, vp, u32]),
                "ref_js_divergence": (f32, [vp, u64, vp, u32]),
                "ref_sample_single": (u32, [vp, vp, u32, u32, f32]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            Reference._lib = lib
        self.lib = Reference._lib

    def generate_weights(self, dist: int, count: int) -> np.ndarray:
        out = np.empty(count, np.float32)
        assert self.lib.ref_generate_weights(dist, count, _ptr(out)) == 0
        return out

    def psa_alias_table(self, w, K):
        w = np.ascontiguousarray(w, np.float32)
        p = np.empty(w.size, np.float32)
        a = np.empty(w.size, np.uint32)
        self.lib.ref_psa_alias_table(_ptr(w), w.size, K, _ptr(p), _ptr(a))
        t = np.zeros(w.size, ENTRY_DTYPE)
        t["p"], t["a"] = p, a
        return t

    def prefix_sum(self, w):
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.float32)
        self.lib.ref_prefix_sum(_ptr(w), w.size, _ptr(out))
        return out

    def kahan_reduction(self, w):
        w = np.ascontiguousarray(w, np.float32)
        return np.float32(self.lib.ref_kahan_reduction(_ptr(w), w.size))

    def stable_partition_indices(self, w, pivot):
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(w.size, np.uint32)
        hc = np.zeros(1, np.uint32)
        self.lib.ref_stable_partition_indices(_ptr(w), w.size, np.float32(pivot), _ptr(out),
                                              _ptr(hc))
        return out, int(hc[0])

    def split(self, heavy_prefix, light_prefix, mean, n):
        hp = np.ascontiguousarray(heavy_prefix, np.float32)
        lp = np.ascontiguousarray(light_prefix, np.float32)
        i = np.zeros(1, np.uint32)
        j = np.zeros(1, np.uint32)
        s = np.zeros(1, np.float32)
        self.lib.ref_split(_ptr(hp), hp.size, _ptr(lp), lp.size, np.float32(mean), n, _ptr(i),
                           _ptr(j), _ptr(s))
        return int(i[0]), int(j[0]), np.float32(s[0])

    def splitK(self, heavy_prefix, light_prefix, mean, N, K):
        hp = np.ascontiguousarray(heavy_prefix, np.float32)
        lp = np.ascontiguousarray(light_prefix, np.float32)
        i = np.zeros(K, np.uint32)
        j = np.zeros(K, np.uint32)
        s = np.zeros(K, np.float32)
        self.lib.ref_splitK(_ptr(hp), hp.size, _ptr(lp), lp.size, np.float32(mean), N, K,
                            _ptr(i), _ptr(j), _ptr(s))
        return i, j, s

    def pack_splits(self, heavy_idx, light_idx, w, mean, si, sj, sspill):
        hi = np.ascontiguousarray(heavy_idx, np.uint32)
        li = np.ascontiguousarray(light_idx, np.uint32)
        w = np.ascontiguousarray(w, np.float32)
        si = np.ascontiguousarray(si, np.uint32)
        sj = np.ascontiguousarray(sj, np.uint32)
        ss = np.ascontiguousarray(sspill, np.float32)
        p = np.empty(w.size, np.float32)
        a = np.empty(w.size, np.uint32)
        self.lib.ref_pack_splits(_ptr(hi), hi.size, _ptr(li), li.size, _ptr(w), w.size,
                                 np.float32(mean), _ptr(si), _ptr(sj), _ptr(ss), si.size,
                                 _ptr(p), _ptr(a))
        t = np.zeros(w.size, ENTRY_DTYPE)
        t["p"], t["a"] = p, a
        return t

    def alias_to_normalized_weights(self, table):
        table = np.ascontiguousarray(table, ENTRY_DTYPE)
        p = np.ascontiguousarray(table["p"])
        a = np.ascontiguousarray(table["a"])
        out = np.empty(table.size, np.float32)
        self.lib.ref_alias_to_normalized_weights(_ptr(p), _ptr(a), table.size, _ptr(out))
        return out

    def assert_is_alias_table(self, w, table, total_weight, margin):
        w = np.ascontiguousarray(w, np.float32)
        table = np.ascontiguousarray(table, ENTRY_DTYPE)
        p = np.ascontiguousarray(table["p"])
        a = np.ascontiguousarray(table["a"])
        cnt = np.zeros(1, np.uint64)
        t = self.lib.ref_assert_is_alias_table(_ptr(w), w.size, _ptr(p), _ptr(a),
                                               np.float32(total_weight), np.float32(margin),
                                               _ptr(cnt))
        return t, int(cnt[0])

    def assert_is_inclusive_prefix(self, elements, prefix):
        e = np.ascontiguousarray(elements, np.float32)
        p = np.ascontiguousarray(prefix, np.float32)
        cnt = np.zeros(1, np.uint64)
        t = self.lib.ref_assert_is_inclusive_prefix(_ptr(e), _ptr(p), e.size, _ptr(cnt))
        return t, int(cnt[0])

    def assert_is_split(self, si, sj, sspill, heavy_prefix, light_prefix, mean, margin):
        si = np.ascontiguousarray(si, np.uint32)
        sj = np.ascontiguousarray(sj, np.uint32)
        ss = np.ascontiguousarray(sspill, np.float32)
        hp = np.ascontiguousarray(heavy_prefix, np.float32)
        lp = np.ascontiguousarray(light_prefix, np.float32)
        cnt = np.zeros(1, np.uint64)
        t = self.lib.ref_assert_is_split(_ptr(si), _ptr(sj), _ptr(ss), si.size, _ptr(hp),
                                         hp.size, _ptr(lp), lp.size, np.float32(mean),
                                         np.float32(margin), _ptr(cnt))
        return t, int(cnt[0])

    def chi_square(self, samples, w):
        s = np.ascontiguousarray(samples, np.uint32)
        w = np.ascontiguousarray(w, np.float32)
        return float(self.lib.ref_chi_square(_ptr(s), s.size, _ptr(w), w.size))

    def js_divergence(self, samples, w):
        s = np.ascontiguousarray(samples, np.uint32)
        w = np.ascontiguousarray(w, np.float32)
        return float(self.lib.ref_js_divergence(_ptr(s), s.size, _ptr(w), w.size))

    def sample_single(self, table, u1, u2):
        table = np.ascontiguousarray(table, ENTRY_DTYPE)
        p = np.ascontiguousarray(table["p"])
        a = np.ascontiguousarray(table["a"])
        return int(self.lib.ref_sample_single(_ptr(p), _ptr(a), table.size, u1, np.float32(u2)))
