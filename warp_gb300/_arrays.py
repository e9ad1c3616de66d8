"""Array plumbing: device memory, streams and ``__cuda_array_interface__`` interop.

The host API takes any object that exposes ``__cuda_array_interface__`` (``wp.array``, torch
tensors, CuPy arrays, ...) and returns torch tensors, which expose the same interface.  PyTorch
is used only for allocation and the current stream; all compute of the path runs in
``libwarp_gb300.so``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as N

_TORCH_TO_GB = {torch.float32: N.GB_F32, torch.float64: N.GB_F64, torch.bfloat16: N.GB_BF16, torch.float16: N.GB_F16}


def gb_dtype(t: torch.dtype) -> int:
    try:
        return _TORCH_TO_GB[t]
    except KeyError:
        raise TypeError(f"unsupported scalar type {t}") from None


def as_tensor(a, dtype: torch.dtype | None = None) -> torch.Tensor:
    """Zero-copy view of a device array as a torch tensor (no host round trip)."""
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        t = a
    elif hasattr(a, "__cuda_array_interface__"):
        t = torch.as_tensor(a, device="cuda")
    else:
        raise TypeError(
            f"expected a device array exposing __cuda_array_interface__, got {type(a).__name__}; "
            "host arrays must be copied to the device explicitly"
        )
    if not t.is_cuda:
        raise ValueError("array must reside on a CUDA device")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"expected dtype {dtype}, got {t.dtype}")
    return t


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def device() -> torch.device:
    return torch.device("cuda", torch.cuda.current_device())


def empty(shape, dtype=torch.float32) -> torch.Tensor:
    return torch.empty(shape, dtype=dtype, device=device())


def zeros(shape, dtype=torch.float32) -> torch.Tensor:
    return torch.zeros(shape, dtype=dtype, device=device())


def workspace(nbytes: int) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device())


def from_numpy(a: np.ndarray, dtype=None) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(device())


def to_numpy(t) -> np.ndarray:
    return as_tensor(t).detach().cpu().numpy()
