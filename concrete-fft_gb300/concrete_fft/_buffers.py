"""Buffer plumbing: torch CUDA tensors go to the device entry points on the
current stream, numpy arrays and CPU tensors to the *_host entry points."""
import ctypes

import numpy as np

try:
    import torch
except ImportError:  # numpy-only use of the host entry points
    torch = None


def is_device(buf):
    return torch is not None and isinstance(buf, torch.Tensor) and buf.is_cuda


def stream_of(buf):
    return ctypes.c_void_p(torch.cuda.current_stream(buf.device).cuda_stream)


def points(buf, elem_bytes):
    """Total element count of a contiguous buffer measured in `elem_bytes` units."""
    if torch is not None and isinstance(buf, torch.Tensor):
        if not buf.is_contiguous():
            raise ValueError("buffer must be contiguous")
        nbytes = buf.numel() * buf.element_size()
    else:
        if not buf.flags["C_CONTIGUOUS"]:
            raise ValueError("buffer must be C-contiguous")
        nbytes = buf.nbytes
    if nbytes % elem_bytes:
        raise ValueError("buffer size is not a multiple of %d bytes" % elem_bytes)
    return nbytes // elem_bytes


def ptr(buf):
    if torch is not None and isinstance(buf, torch.Tensor):
        return ctypes.c_void_p(buf.data_ptr())
    return ctypes.c_void_p(buf.ctypes.data)


def check_dtype(buf, allowed):
    dt = str(buf.dtype).replace("torch.", "")
    if dt not in allowed:
        raise TypeError("buffer dtype %s not in %s" % (dt, allowed))


def batch_of(buf, n, elem_bytes):
    total = points(buf, elem_bytes)
    if total % n:
        raise ValueError("buffer length %d is not a multiple of the plan size %d" % (total, n))
    return total // n


C64_DTYPES = ("complex128", "float64")
