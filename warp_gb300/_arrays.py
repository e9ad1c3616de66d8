"""Array plumbing: device memory, streams and ``__cuda_array_interface__`` interop.

The host API takes any object that exposes ``__cuda_array_interface__`` (``wp.array``, torch
tensors, CuPy arrays, ...).  New output vectors come back in the caller's array type: ``wp.array``
when the caller passed ``wp.array`` inputs (``warp.from_torch`` of the result), torch tensors
otherwise (they expose the same interface).  PyTorch is used only for allocation; all compute of
the path runs in ``libwarp_gb300.so``.

Streams: the reference runs every call on Warp's current stream (``wp.get_stream(device)``,
``warp/_src/context.py``).  Each public entry point here runs on the caller's stream, in this
order: the stream of an enclosing ``ScopedStream`` block, else Warp's current stream when the
``warp`` module is loaded in the process, else torch's current stream.  The library's own torch
operations (allocation, fills, copies) are ordered on that same stream.
"""

from __future__ import annotations

import functools
import sys
import threading

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
    """The stream handle the current call runs on (see the module docstring)."""
    return torch.cuda.current_stream().cuda_stream


_SCOPE = threading.local()
_EXTERNAL: dict[int, torch.cuda.Stream] = {}


class ScopedStream:
    """Run the library's calls inside the block on ``stream`` (a ``cudaStream_t`` handle as int, a
    ``torch.cuda.Stream`` or an object with a ``cuda_stream`` attribute such as ``wp.Stream``);
    the counterpart of ``wp.ScopedStream``."""

    def __init__(self, stream_):
        h = getattr(stream_, "cuda_stream", stream_)
        self.handle = int(h) if h is not None else None

    def __enter__(self):
        if not hasattr(_SCOPE, "stack"):
            _SCOPE.stack = []
        _SCOPE.stack.append(self.handle)
        return self

    def __exit__(self, *exc):
        _SCOPE.stack.pop()


def caller_stream() -> int | None:
    """Handle of the stream a call should run on, or None for torch's current stream."""
    stack = getattr(_SCOPE, "stack", None)
    if stack:
        return stack[-1]
    wp = sys.modules.get("warp")
    if wp is not None and hasattr(wp, "get_stream"):
        try:
            return int(wp.get_stream(f"cuda:{torch.cuda.current_device()}").cuda_stream)
        except Exception:
            return None
    return None


def _external(handle: int) -> torch.cuda.Stream:
    s = _EXTERNAL.get(handle)
    if s is None:
        s = torch.cuda.ExternalStream(handle)
        _EXTERNAL[handle] = s
    return s


def on_caller_stream(fn):
    """Decorator of the public entry points: run the call (kernels and the library's own torch
    operations) on the caller's stream."""

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        h = caller_stream()
        if h is None or not torch.cuda.is_available() or h == torch.cuda.current_stream().cuda_stream:
            return fn(*args, **kwargs)
        with torch.cuda.stream(_external(h)):
            return fn(*args, **kwargs)

    return wrapper


def is_warp_array(a) -> bool:
    return a is not None and type(a).__module__.split(".")[0] == "warp"


def like(template, t: torch.Tensor):
    """Return the new output ``t`` in the array type of the caller's input ``template``."""
    if is_warp_array(template):
        wp = sys.modules.get("warp")
        if wp is not None and hasattr(wp, "from_torch"):
            return wp.from_torch(t)
    return t


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
