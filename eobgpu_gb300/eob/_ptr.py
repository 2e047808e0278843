"""Pointer plumbing of the drop-in shims: the reference's Cython layer takes
raw device addresses as Python ints (via bbhx's pointer_adjust,
src/eob.pyx:4); these shims accept torch CUDA tensors or ints."""
from __future__ import annotations

import ctypes

import torch


def addr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise ValueError("device arrays only: the EOB entry points take CUDA tensors")
        return ctypes.c_void_p(x.data_ptr())
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    if hasattr(x, "__cuda_array_interface__"):
        return ctypes.c_void_p(x.__cuda_array_interface__["data"][0])
    raise TypeError(f"cannot take a device address of {type(x)}")


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
