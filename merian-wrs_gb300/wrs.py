"""Host-side mirror of merian-wrs's operator facade over the C ABI (include/wrs.h).

Mirrors (paths relative to the reference project):
  WRSConfig / AliasTableConfig / ITSConfig   src/device/wrs/WRS.hpp:14,
                                             src/device/wrs/alias/AliasTable.hpp:10-22,
                                             src/device/wrs/its/ITS.hpp:68-77
  WRSBuffers.allocate(N, S, config)          src/device/wrs/WRS.hpp:60-88
  WRS(config).build(stream, buffers, N)      src/device/wrs/WRS.hpp:121-143
  WRS.sample(stream, buffers, N, S, seed)    src/device/wrs/WRS.hpp:145-168 (seed = 12345)

Device memory and streams come from PyTorch (plumbing only); all compute runs in
libwrs_gb300.so.  There is no fallback: if the library cannot be loaded, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libwrs_gb300.so")

METHOD_ALIAS_TABLE = 0
METHOD_ITS = 1
METHOD_CUTPOINT = 2
RNG_REFERENCE = 0
RNG_PHILOX4X32_10 = 1
SCAN_FP32 = 0
SCAN_COMPENSATED = 1
SCAN_FLOAT_FLOAT = 2
SPLITPACK_INLINE = 0
SPLITPACK_SERIAL = 1
SPLITPACK_SERIAL_SUBGROUP = 2

DEVICE_TIMEOUT = 1
DEVICE_NONMONOTONE_SPLIT = 2


class WRSError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"wrs status {status}: {message}")
        self.status = status


class _Config(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "method", "split_size", "use_partition_elements", "coop_size", "its_parray", "rng",
        "scan_precision", "split_residual_f64", "split_full_light", "guiding_entry_size",
        "split_pack_mode")]


class SplitRecord(C.Structure):
    """wrs_split_record: {i, j, spill} (the shaders' Split, 12 bytes)."""
    _fields_ = [("i", C.c_uint32), ("j", C.c_uint32), ("spill", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget", C.c_uint64), ("slots", C.c_uint32),
                ("max_batch_dists", C.c_uint32), ("max_batch_weights", C.c_uint64),
                ("max_batch_samples", C.c_uint64)]


class Request(C.Structure):
    """wrs_request: one build+sample request (device pointers)."""
    _fields_ = [("table_id", C.c_uint64), ("weights", C.c_void_p), ("samples", C.c_void_p),
                ("s", C.c_uint64), ("seed", C.c_uint64), ("n", C.c_uint32),
                ("reserved", C.c_uint32)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("submit_s", C.c_double), ("done_s", C.c_double),
                ("built", C.c_uint32), ("status", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "submitted", "completed", "batches", "builds", "reuses", "evictions",
        "table_arena_bytes", "table_bytes_peak", "scratch_bytes", "device_status")]


class TuneSpace(C.Structure):
    _fields_ = [("split_sizes", C.POINTER(C.c_uint32)), ("split_count", C.c_uint32),
                ("l2_fetch", C.POINTER(C.c_uint32)), ("l2_count", C.c_uint32),
                ("warmup", C.c_uint32), ("reps", C.c_uint32)]


class TuneTrial(C.Structure):
    _fields_ = [("split_size", C.c_uint32), ("l2_fetch", C.c_uint32), ("build_ms", C.c_float),
                ("sample_ms", C.c_float)]


class TuneResult(C.Structure):
    _fields_ = [("split_size", C.c_uint32), ("l2_fetch", C.c_uint32), ("build_ms", C.c_float),
                ("sample_ms", C.c_float), ("trials", C.c_uint32)]


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Load libwrs_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with merian-wrs_gb300/build.py "
                               "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp, u32, u64, f32, i32, sz = (C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int,
                                      C.c_size_t)
        cfgp = C.POINTER(_Config)
        sig = {
            "wrs_version": (i32, []),
            "wrs_status_string": (C.c_char_p, [i32]),
            "wrs_last_error": (C.c_char_p, []),
            "wrs_config_init": (i32, [cfgp, u32]),
            "wrs_create": (i32, [cfgp, C.POINTER(vp)]),
            "wrs_destroy": (None, [vp]),
            "wrs_buffers_bytes": (sz, [vp, u32]),
            "wrs_buffers_create": (i32, [vp, u32, C.POINTER(vp)]),
            "wrs_buffers_destroy": (None, [vp]),
            "wrs_build": (i32, [vp, vp, vp, u32, vp]),
            "wrs_sample": (i32, [vp, vp, vp, u32, u64, u64, vp]),
            "wrs_sample_at": (i32, [vp, vp, vp, u32, u64, u64, u64, vp]),
            "wrs_buffers_status": (i32, [vp, vp, C.POINTER(u32)]),
            "wrs_buffers_alias_table": (vp, [vp]),
            "wrs_buffers_cmf": (vp, [vp]),
            "wrs_buffers_guide_table": (vp, [vp]),
            "wrs_cutpoint_guide": (i32, [vp, vp, vp, u32, vp]),
            "wrs_cutpoint_sample": (i32, [vp, vp, vp, u32, vp, u64, u64, u64, vp]),
            "wrs_buffers_partition_indices": (vp, [vp]),
            "wrs_buffers_partition_prefix": (vp, [vp]),
            "wrs_buffers_partition_elements": (vp, [vp]),
            "wrs_buffers_partition_prefix_lo": (vp, [vp]),
            "wrs_buffers_mean": (vp, [vp]),
            "wrs_buffers_total": (vp, [vp]),
            "wrs_buffers_heavy_count": (vp, [vp]),
            "wrs_total_mass": (i32, [vp, vp, vp, u32, vp]),
            "wrs_prefix_sum": (i32, [vp, vp, vp, u32, vp, vp]),
            "wrs_prefix_partition": (i32, [vp, vp, vp, u32, vp, vp, vp, vp, vp]),
            "wrs_split_pack": (i32, [vp, vp, vp, vp, vp, vp, vp, u32, vp, vp]),
            "wrs_alias_sample": (i32, [vp, vp, vp, u32, u64, u64, u64, vp]),
            "wrs_its_sample": (i32, [vp, vp, vp, u32, u64, u64, u64, vp]),
            "wrs_buffers_set_partition_info": (i32, [vp, vp, f32, C.c_double, u32]),
            "wrs_buffers_mean64": (vp, [vp]),
            "wrs_test_prefix_sum_stalled": (i32, [vp, vp, vp, u32, vp, vp, u32]),
            "wrs_test_arena": (i32, [u64, u32]),
            "wrs_prefix_sum_noalloc": (i32, [vp, vp, u32, vp, u32, vp]),
            "wrs_philox": (i32, [vp, u32, u32, vp]),
            "wrs_batch_bytes": (sz, [vp, u32, u64, u64]),
            "wrs_batch_create": (i32, [vp, u32, u64, u64, C.POINTER(vp)]),
            "wrs_batch_destroy": (None, [vp]),
            "wrs_batch_set": (i32, [vp, vp, vp, u32]),
            "wrs_batch_count": (u32, [vp]),
            "wrs_batch_build": (i32, [vp, vp, vp]),
            "wrs_batch_sample": (i32, [vp, vp, vp]),
            "wrs_batch_status": (i32, [vp, vp, C.POINTER(u32)]),
            "wrs_probe_random_gather": (i32, [vp, vp, u64, u64, u32, vp]),
            "wrs_histogram": (i32, [vp, vp, u64, u32, vp, vp]),
            "wrs_statistics_scratch_bytes": (sz, [u32]),
            "wrs_sample_statistics": (i32, [vp, vp, vp, u32, u64, vp, vp]),
            "wrs_server_config_init": (i32, [C.POINTER(ServerConfig)]),
            "wrs_server_create": (i32, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
            "wrs_server_destroy": (None, [vp]),
            "wrs_server_submit": (i32, [vp, C.POINTER(Request), C.POINTER(u64)]),
            "wrs_server_progress": (i32, [vp, C.POINTER(Completion), u32, C.POINTER(u32)]),
            "wrs_server_pending": (u64, [vp]),
            "wrs_server_get_stats": (i32, [vp, C.POINTER(ServerStats)]),
            "wrs_server_run_trace": (i32, [vp, C.POINTER(Request), C.POINTER(C.c_double), u32,
                                           C.POINTER(Completion)]),
            "wrs_prefix_sum_blockwise": (i32, [vp, vp, vp, u32, vp, vp]),
            "wrs_prefix_partition_blockwise": (i32, [vp, vp, vp, u32, vp, vp, vp, vp]),
            "wrs_split_records_count": (u32, [u32, u32]),
            "wrs_split": (i32, [vp, vp, vp, vp, u32, vp, vp]),
            "wrs_pack": (i32, [vp, vp, vp, vp, vp, vp, u32, vp, vp]),
            "wrs_buffers_split_records": (vp, [vp]),
            "wrs_set_l2_fetch_granularity": (i32, [u32]),
            "wrs_get_l2_fetch_granularity": (i32, [C.POINTER(u32)]),
            "wrs_autotune_alias": (i32, [cfgp, vp, vp, u32, u64, vp, C.POINTER(TuneSpace),
                                         C.POINTER(TuneResult), C.POINTER(TuneTrial), u32]),
            "wrs_autotune_batch": (i32, [cfgp, vp, vp, u32, C.POINTER(TuneSpace),
                                         C.POINTER(TuneResult), C.POINTER(TuneTrial), u32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise WRSError(status, lib().wrs_last_error().decode())


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def _dev_ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("device tensors must be contiguous CUDA tensors")
    return t.data_ptr()


@dataclass
class WRSConfig:
    """The WRSConfig variant: method plus the knobs of its sub-configs."""
    method: int = METHOD_ALIAS_TABLE
    split_size: int = 2
    use_partition_elements: bool = True
    coop_size: int = 0
    its_parray: bool = False
    rng: int = RNG_REFERENCE
    scan_precision: int = SCAN_FP32
    split_residual_f64: bool = False
    split_full_light: bool = False
    guiding_entry_size: int = 32
    split_pack_mode: int = SPLITPACK_INLINE

    def c(self) -> _Config:
        return _Config(self.method, self.split_size, int(self.use_partition_elements),
                       self.coop_size, int(self.its_parray), self.rng, self.scan_precision,
                       int(self.split_residual_f64), int(self.split_full_light),
                       self.guiding_entry_size, self.split_pack_mode)

    def split_flags(self) -> int:
        """The oracle's split flags for this configuration."""
        return (1 if self.split_residual_f64 else 0) | (2 if self.split_full_light else 0)

    def name(self) -> str:
        if self.method == METHOD_ITS:
            coop = f"-COOP-{self.coop_size}-{'PARRAY' if self.its_parray else 'BINARY'}" \
                if self.coop_size else ""
            return f"ITS{coop}"
        if self.method == METHOD_CUTPOINT:
            return f"Cutpoint-{self.guiding_entry_size}"
        return f"AliasTable-PSA-split{self.split_size}-coop{self.coop_size}"


def AliasTableConfig(split_size: int = 2, use_partition_elements: bool = True,
                     coop_size: int = 0, **kw) -> WRSConfig:
    """AliasTableConfig(PSAConfig(..., InlineSplitPackConfig(split_size), usePartitionElements),
    SampleAliasTableConfig(coop_size))."""
    return WRSConfig(METHOD_ALIAS_TABLE, split_size, use_partition_elements, coop_size, **kw)


def ITSConfig(coop_size: int = 0, parray: bool = False, guiding_entry_size: int = 4,
              **kw) -> WRSConfig:
    """ITSConfig(DecoupledPrefixSumConfig(), InverseTransformSamplingConfig(512, coop, parray)).
    guiding_entry_size: weights per cell of the cell blocks that steer the searches (both
    precisions; on an FP32 CMF the cells its decreases can reach bisect); 0 = none (the
    bisection through the stored probe tree).  Indices do not depend on it."""
    return WRSConfig(METHOD_ITS, coop_size=coop_size, its_parray=parray,
                     guiding_entry_size=guiding_entry_size, **kw)


def CutpointConfig(guiding_entry_size: int = 32, **kw) -> WRSConfig:
    """CutpointConfig(DecoupledPrefixSumConfig(), guidingEntrySize)."""
    return WRSConfig(METHOD_CUTPOINT, guiding_entry_size=guiding_entry_size, **kw)


class Handle:
    """Owns a wrs_handle."""

    def __init__(self, config: WRSConfig):
        self.config = config
        self._cfg = config.c()
        h = C.c_void_p()
        check(lib().wrs_create(C.byref(self._cfg), C.byref(h)))
        self.ptr = h.value

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.wrs_destroy(self.ptr)
            self.ptr = None


class Internals:
    """Owns a wrs_buffers (the method's internal device buffers)."""

    def __init__(self, handle: Handle, max_n: int):
        b = C.c_void_p()
        check(lib().wrs_buffers_create(handle.ptr, max_n, C.byref(b)))
        self.ptr = b.value
        self.max_n = max_n
        self.handle = handle

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.wrs_buffers_destroy(self.ptr)
            self.ptr = None

    def status(self, stream=None) -> int:
        v = C.c_uint32(0)
        st = lib().wrs_buffers_status(self.ptr, _stream_ptr(stream), C.byref(v))
        if st not in (0, 3):
            check(st)
        return int(v.value)

    def views(self) -> dict:
        L = lib()
        return {
            "alias_table": L.wrs_buffers_alias_table(self.ptr),
            "cmf": L.wrs_buffers_cmf(self.ptr),
            "guide_table": L.wrs_buffers_guide_table(self.ptr),
            "split_records": L.wrs_buffers_split_records(self.ptr),
            "partition_indices": L.wrs_buffers_partition_indices(self.ptr),
            "partition_prefix": L.wrs_buffers_partition_prefix(self.ptr),
            "partition_elements": L.wrs_buffers_partition_elements(self.ptr),
            "partition_prefix_lo": L.wrs_buffers_partition_prefix_lo(self.ptr),
            "mean": L.wrs_buffers_mean(self.ptr),
            "mean64": L.wrs_buffers_mean64(self.ptr),
            "total": L.wrs_buffers_total(self.ptr),
            "heavy_count": L.wrs_buffers_heavy_count(self.ptr),
        }


@dataclass
class WRSBuffers:
    """weights [N] float32 and samples [S] (uint32 stored as int32) are caller-owned device
    tensors; `internals` holds the method's buffers."""
    weights: object
    samples: object
    internals: Internals = field(repr=False)

    @classmethod
    def allocate(cls, N: int, S: int, config: WRSConfig, device="cuda", handle=None):
        import torch
        handle = handle or Handle(config)
        w = torch.empty(N, dtype=torch.float32, device=device)
        s = torch.empty(S, dtype=torch.int32, device=device)
        return cls(w, s, Internals(handle, N))


class WRS:
    """device::WRS: build() records the construction of the sampler of buffers.weights[:N],
    sample() draws S samples into buffers.samples.  Both are asynchronous on `stream`."""

    def __init__(self, config: WRSConfig):
        self.config = config
        self.handle = Handle(config)

    def build(self, stream, buffers: WRSBuffers, N: int) -> None:
        check(lib().wrs_build(self.handle.ptr, _stream_ptr(stream), _dev_ptr(buffers.weights),
                              N, buffers.internals.ptr))

    def sample(self, stream, buffers: WRSBuffers, N: int, S: int, seed: int = 12345,
               offset: int = 0) -> None:
        check(lib().wrs_sample_at(self.handle.ptr, _stream_ptr(stream), buffers.internals.ptr,
                                  N, S, seed, offset, _dev_ptr(buffers.samples)))

    # primitives -----------------------------------------------------------------
    def total_mass(self, stream, weights, N, internals: Internals) -> None:
        check(lib().wrs_total_mass(self.handle.ptr, _stream_ptr(stream), _dev_ptr(weights), N,
                                   internals.ptr))

    def prefix_sum(self, stream, inp, N, out, internals: Internals) -> None:
        check(lib().wrs_prefix_sum(self.handle.ptr, _stream_ptr(stream), _dev_ptr(inp), N,
                                   _dev_ptr(out), internals.ptr))

    def prefix_partition(self, stream, weights, N, idx, prefix, elems, internals,
                         prefix_lo=None) -> None:
        check(lib().wrs_prefix_partition(self.handle.ptr, _stream_ptr(stream), _dev_ptr(weights),
                                         N, _dev_ptr(idx), _dev_ptr(prefix), _dev_ptr(elems),
                                         _dev_ptr(prefix_lo), internals.ptr))

    def split_pack(self, stream, weights, idx, prefix, elems, N, table, internals,
                   prefix_lo=None) -> None:
        check(lib().wrs_split_pack(self.handle.ptr, _stream_ptr(stream), _dev_ptr(weights),
                                   _dev_ptr(idx), _dev_ptr(prefix), _dev_ptr(elems),
                                   _dev_ptr(prefix_lo), N, _dev_ptr(table), internals.ptr))

    def prefix_sum_blockwise(self, stream, inp, N, out, internals) -> None:
        """wrs_prefix_sum_blockwise: the reduce-then-scan baseline (FP32 carries)."""
        check(lib().wrs_prefix_sum_blockwise(self.handle.ptr, _stream_ptr(stream), _dev_ptr(inp),
                                             N, _dev_ptr(out), internals.ptr))

    def prefix_partition_blockwise(self, stream, weights, N, idx, prefix, elems,
                                   internals) -> None:
        """wrs_prefix_partition_blockwise: the reduce-then-scan baseline (FP32 carries)."""
        check(lib().wrs_prefix_partition_blockwise(self.handle.ptr, _stream_ptr(stream),
                                                   _dev_ptr(weights), N, _dev_ptr(idx),
                                                   _dev_ptr(prefix), _dev_ptr(elems),
                                                   internals.ptr))

    def split(self, stream, prefix, N, records, internals, prefix_lo=None) -> None:
        """wrs_split: the serial split-pack's ceil(N / split_size) split records."""
        check(lib().wrs_split(self.handle.ptr, _stream_ptr(stream), _dev_ptr(prefix),
                              _dev_ptr(prefix_lo), N, _dev_ptr(records), internals.ptr))

    def pack(self, stream, weights, idx, elems, records, N, table, internals) -> None:
        """wrs_pack: the alias table from split records (scalar or warp strategy)."""
        check(lib().wrs_pack(self.handle.ptr, _stream_ptr(stream), _dev_ptr(weights),
                             _dev_ptr(idx), _dev_ptr(elems), _dev_ptr(records), N,
                             _dev_ptr(table), internals.ptr))

    def alias_sample(self, stream, table, N, S, seed, offset, out) -> None:
        check(lib().wrs_alias_sample(self.handle.ptr, _stream_ptr(stream), _dev_ptr(table), N, S,
                                     seed, offset, _dev_ptr(out)))

    def its_sample(self, stream, cmf, N, S, seed, offset, out) -> None:
        check(lib().wrs_its_sample(self.handle.ptr, _stream_ptr(stream), _dev_ptr(cmf), N, S,
                                   seed, offset, _dev_ptr(out)))

    def cutpoint_guide(self, stream, cmf, N, guide) -> None:
        check(lib().wrs_cutpoint_guide(self.handle.ptr, _stream_ptr(stream), _dev_ptr(cmf), N,
                                       _dev_ptr(guide)))

    def cutpoint_sample(self, stream, cmf, N, guide, S, seed, offset, out) -> None:
        check(lib().wrs_cutpoint_sample(self.handle.ptr, _stream_ptr(stream), _dev_ptr(cmf), N,
                                        _dev_ptr(guide), S, seed, offset, _dev_ptr(out)))


class PRNG:
    """The reference's PRNG operator with its one alternative, PhiloxConfig
    (src/device/prng/PRNG.hpp:15-56): run(cmd, buffers, S, seed = 12345) fills buffers.samples
    with S uniform floats, element i = float(x1) / 2^32 of the shaders' Philox2x32-7 at counter
    (i, 0), key = seed (src/device/prng/philox/shader.comp:47-55).  `samples` is a float32
    device tensor (or a raw device address)."""

    def run(self, stream, samples, S: int, seed: int = 12345) -> None:
        check(lib().wrs_philox(_stream_ptr(stream), seed & 0xFFFFFFFF, S, _dev_ptr(samples)))


class DistDesc(C.Structure):
    """wrs_dist_desc: one distribution of a batch (device pointers)."""
    _fields_ = [("weights", C.c_void_p), ("table", C.c_void_p), ("samples", C.c_void_p),
                ("s", C.c_uint64), ("seed", C.c_uint64), ("n", C.c_uint32),
                ("reserved", C.c_uint32)]


class Batch:
    """Many distributions built and sampled with one launch per stage (wrs_batch_*): the
    batched form of WRS.build / WRS.sample.  No counterpart in the reference."""

    def __init__(self, handle: Handle, max_dists: int, max_weights: int, max_samples: int):
        self.handle = handle
        p = C.c_void_p()
        check(lib().wrs_batch_create(handle.ptr, max_dists, max_weights, max_samples,
                                     C.byref(p)))
        self.ptr = p.value
        self._descs = None

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().wrs_batch_destroy(self.ptr)
            self.ptr = None

    @staticmethod
    def bytes(handle: Handle, max_dists: int, max_weights: int, max_samples: int) -> int:
        return lib().wrs_batch_bytes(handle.ptr, max_dists, max_weights, max_samples)

    def set(self, stream, dists) -> None:
        """dists: iterable of (weights, table, samples, n, s, seed); weights / samples may be
        None (sample only / build only); tensors or raw device addresses."""
        dists = list(dists)
        arr = (DistDesc * max(1, len(dists)))()
        for i, (w, t, out, n, s, seed) in enumerate(dists):
            arr[i] = DistDesc(_dev_ptr(w), _dev_ptr(t), _dev_ptr(out), s, seed, n, 0)
        self._descs = arr
        check(lib().wrs_batch_set(self.ptr, _stream_ptr(stream), arr, len(dists)))

    def build(self, stream) -> None:
        check(lib().wrs_batch_build(self.handle.ptr, _stream_ptr(stream), self.ptr))

    def sample(self, stream) -> None:
        check(lib().wrs_batch_sample(self.handle.ptr, _stream_ptr(stream), self.ptr))

    def count(self) -> int:
        return lib().wrs_batch_count(self.ptr)

    def status(self, stream=None) -> int:
        v = C.c_uint32()
        check(lib().wrs_batch_status(self.ptr, _stream_ptr(stream), C.byref(v)))
        return v.value


class Server:
    """The served request loop (wrs_server_*): continuous batching of build+sample requests
    with resident alias tables under a device memory budget.  No counterpart in the
    reference."""

    def __init__(self, handle: Handle, memory_budget: int = 16 << 30, slots: int = 3,
                 max_batch_dists: int = 1024, max_batch_weights: int = 1 << 25,
                 max_batch_samples: int = 1 << 24):
        self.handle = handle
        c = ServerConfig()
        check(lib().wrs_server_config_init(C.byref(c)))
        c.memory_budget, c.slots, c.max_batch_dists = memory_budget, slots, max_batch_dists
        c.max_batch_weights, c.max_batch_samples = max_batch_weights, max_batch_samples
        p = C.c_void_p()
        check(lib().wrs_server_create(handle.ptr, C.byref(c), C.byref(p)))
        self.ptr = p.value

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().wrs_server_destroy(self.ptr)
            self.ptr = None

    @staticmethod
    def requests(rows) -> "C.Array":
        """rows: iterable of (table_id, weights_ptr, samples_ptr, n, s, seed)."""
        rows = list(rows)
        arr = (Request * max(1, len(rows)))()
        for i, (tid, w, out, n, s, seed) in enumerate(rows):
            arr[i] = Request(tid, _dev_ptr(w), _dev_ptr(out), s, seed, n, 0)
        return arr

    def submit(self, req: Request) -> int:
        t = C.c_uint64()
        check(lib().wrs_server_submit(self.ptr, C.byref(req), C.byref(t)))
        return t.value

    def progress(self, max_out: int = 1024) -> list:
        buf = (Completion * max_out)()
        c = C.c_uint32()
        check(lib().wrs_server_progress(self.ptr, buf, max_out, C.byref(c)))
        return [buf[i] for i in range(c.value)]

    def pending(self) -> int:
        return lib().wrs_server_pending(self.ptr)

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().wrs_server_get_stats(self.ptr, C.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def run_trace(self, reqs, arrivals) -> "C.Array":
        """Replays requests at their arrival times (seconds from the call); returns the
        completions in request order."""
        n = len(arrivals)
        arr = (C.c_double * max(1, n))(*arrivals)
        out = (Completion * max(1, n))()
        check(lib().wrs_server_run_trace(self.ptr, reqs, arr, n, out))
        return out


class Statistics:
    """Histogram, chi-square and RMSE of a sample set on the device (wrs_histogram /
    wrs_sample_statistics; the reference's device::ChiSquare and RMSE passes)."""

    def __init__(self, n: int, device="cuda"):
        import torch
        self.n = n
        nbytes = lib().wrs_statistics_scratch_bytes(n)
        self._scratch = torch.zeros((nbytes + 127) // 8 + 16, dtype=torch.float64, device=device)
        off = (-self._scratch.data_ptr()) % 128
        self.scratch = self._scratch.data_ptr() + off
        self.hist = torch.zeros(n, dtype=torch.int64, device=device)
        self.out = torch.zeros(4, dtype=torch.float64, device=device)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)

    def __call__(self, stream, samples, s: int, weights) -> dict:
        """samples: device tensor or address of s uint32 indices; returns chi2, rmse,
        zero-weight draws and total weight (synchronises)."""
        import torch
        self.hist.zero_()
        check(lib().wrs_histogram(_stream_ptr(stream), _dev_ptr(samples), s, self.n,
                                  self.hist.data_ptr(), self.status.data_ptr()))
        check(lib().wrs_sample_statistics(_stream_ptr(stream), self.hist.data_ptr(),
                                          _dev_ptr(weights), self.n, s, self.scratch,
                                          self.out.data_ptr()))
        torch.cuda.synchronize()
        o = self.out.cpu().tolist()
        return {"chi2": o[0], "rmse": o[1], "zero_weight_draws": int(o[2]), "total": o[3],
                "out_of_range": bool(int(self.status.item()) & 4)}


def set_l2_fetch_granularity(nbytes: int) -> None:
    """The CUDA context's L2 fetch-granularity hint (bytes, <= 128); context-wide."""
    check(lib().wrs_set_l2_fetch_granularity(nbytes))


def get_l2_fetch_granularity() -> int:
    v = C.c_uint32()
    check(lib().wrs_get_l2_fetch_granularity(C.byref(v)))
    return v.value


def _tune_space(split_sizes, l2_fetch, warmup, reps):
    sp = TuneSpace()
    keep = []
    if split_sizes is not None:
        arr = (C.c_uint32 * max(1, len(split_sizes)))(*split_sizes)
        keep.append(arr)
        sp.split_sizes = C.cast(arr, C.POINTER(C.c_uint32)) if len(split_sizes) else None
        sp.split_count = len(split_sizes)
    else:
        sp.split_count = 1  # NULL with a nonzero count: the default candidates
    if l2_fetch is not None:
        arr = (C.c_uint32 * max(1, len(l2_fetch)))(*l2_fetch)
        keep.append(arr)
        sp.l2_fetch = C.cast(arr, C.POINTER(C.c_uint32)) if len(l2_fetch) else None
        sp.l2_count = len(l2_fetch)
    else:
        sp.l2_count = 1
    sp.warmup, sp.reps = warmup, reps
    return sp, keep


def _tune_out(res: TuneResult, trials) -> dict:
    return {"split_size": res.split_size, "l2_fetch": res.l2_fetch,
            "build_ms": res.build_ms, "sample_ms": res.sample_ms,
            "trials": [{"split_size": t.split_size, "l2_fetch": t.l2_fetch,
                        "build_ms": t.build_ms, "sample_ms": t.sample_ms}
                       for t in trials[:min(res.trials, len(trials))]]}


def autotune_alias(config: WRSConfig, stream, weights, n: int, s: int = 0, samples=None,
                   split_sizes=None, l2_fetch=None, warmup: int = 1, reps: int = 3) -> dict:
    """wrs_autotune_alias: fastest split size and L2 fetch granularity for building n weights
    and drawing s samples (the context's L2 limit is left at the chosen value).
    split_sizes / l2_fetch None = the library's candidates, [] = not tuned."""
    sp, keep = _tune_space(split_sizes, l2_fetch, warmup, reps)
    res = TuneResult()
    trials = (TuneTrial * 32)()
    cfg = config.c()
    check(lib().wrs_autotune_alias(C.byref(cfg), _stream_ptr(stream), _dev_ptr(weights), n, s,
                                   _dev_ptr(samples), C.byref(sp), C.byref(res), trials, 32))
    del keep
    return _tune_out(res, trials)


def autotune_batch(config: WRSConfig, stream, dists, split_sizes=None, l2_fetch=None,
                   warmup: int = 1, reps: int = 3) -> dict:
    """wrs_autotune_batch over dists as Batch.set takes them."""
    dists = list(dists)
    arr = (DistDesc * max(1, len(dists)))()
    for i, (w, t, out, n, s, seed) in enumerate(dists):
        arr[i] = DistDesc(_dev_ptr(w), _dev_ptr(t), _dev_ptr(out), s, seed, n, 0)
    sp, keep = _tune_space(split_sizes, l2_fetch, warmup, reps)
    res = TuneResult()
    trials = (TuneTrial * 32)()
    cfg = config.c()
    check(lib().wrs_autotune_batch(C.byref(cfg), _stream_ptr(stream), arr, len(dists),
                                   C.byref(sp), C.byref(res), trials, 32))
    del keep
    return _tune_out(res, trials)
