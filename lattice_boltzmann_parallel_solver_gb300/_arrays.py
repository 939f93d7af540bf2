"""Array plumbing between the caller's arrays and CUDA device tensors.

The drop-in functions accept what the reference's functions accept (NumPy
arrays) and also torch tensors.  NumPy / CPU inputs are copied to the
device once and results are returned in the caller's kind, so a NumPy
caller gets NumPy back.
"""
from __future__ import annotations

import numpy as np
import torch

NUMPY, TORCH_CPU, TORCH_CUDA = 0, 1, 2


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("lattice_boltzmann_parallel_solver_gb300 needs a CUDA device (there is no CPU path)")


def kind_of(a) -> int:
    if isinstance(a, torch.Tensor):
        return TORCH_CUDA if a.is_cuda else TORCH_CPU
    return NUMPY


def to_device(a, dtype=torch.float64) -> torch.Tensor:
    """Contiguous device tensor of ``dtype`` holding ``a`` (no copy when it already is one)."""
    require_cuda()
    if isinstance(a, torch.Tensor):
        t = a
    else:
        arr = np.asarray(a)
        if arr.dtype == np.bool_:
            arr = arr.astype(np.uint8)
        t = torch.from_numpy(np.ascontiguousarray(arr))
    if not t.is_cuda:
        t = t.pin_memory() if t.numel() * t.element_size() > (1 << 20) else t
        t = t.to("cuda", non_blocking=True)
    if t.dtype != dtype:
        t = t.to(dtype)
    return t.contiguous()


def to_kind(t: torch.Tensor, kind: int):
    """Device result back in the caller's kind; host results land in pinned
    memory (the caching host allocator reuses it across calls)."""
    if kind == TORCH_CUDA:
        return t
    out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    out.copy_(t, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return out if kind == TORCH_CPU else out.numpy()


def write_back(dst, src: torch.Tensor):
    """In-place update of the caller's array (the reference closures mutate and return their argument)."""
    if isinstance(dst, torch.Tensor):
        if dst.data_ptr() != src.data_ptr():
            dst.copy_(src)
        return dst
    dst[...] = src.cpu().numpy()
    return dst


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()
