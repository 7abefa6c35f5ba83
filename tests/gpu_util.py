"""Device I/O for the GPU tests: numpy <-> CUDA through PyTorch tensors, and reads of raw
device pointers (the internals' views) through the CUDA runtime."""
from __future__ import annotations

import ctypes as C

import numpy as np

_cudart = None


def cudart():
    global _cudart
    if _cudart is None:
        import torch  # noqa: F401  (initialises the runtime)
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                _cudart = C.CDLL(name)
                break
            except OSError:
                continue
        if _cudart is None:
            raise RuntimeError("libcudart not found")
        _cudart.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _cudart.cudaMemcpy.restype = C.c_int
        _cudart.cudaDeviceSynchronize.restype = C.c_int
    return _cudart


def d2h(ptr: int, count: int, dtype) -> np.ndarray:
    out = np.empty(count, dtype)
    assert cudart().cudaDeviceSynchronize() == 0
    rc = cudart().cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2)
    assert rc == 0, f"cudaMemcpy failed ({rc})"
    return out


def h2d(a: np.ndarray):
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    elif a.dtype.fields is not None:  # alias entries -> raw 32-bit words
        a = a.view(np.int32)
    return torch.from_numpy(a.copy()).cuda()


def empty(n: int, dtype="f32"):
    import torch
    return torch.empty(n, dtype=torch.float32 if dtype == "f32" else torch.int32, device="cuda")


def t2h(t, dtype) -> np.ndarray:
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy().view(dtype)
