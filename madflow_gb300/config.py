"""Types and device selection (madflow config.py:16-79).

``MADFLOW_FLOAT`` (64 by default) selects the arithmetic of the matrix-element
kernels: 64 runs everything in FP64, 32 runs the mixed path (FP32
wavefunctions, vertices and colour sum; FP64 momenta, propagator denominators
and accumulation).  Host-facing tensors are always float64 / complex128, like
the reference's default.
"""
import os

import torch

DTYPE = torch.float64
DTYPEINT = torch.int32
DTYPECOMPLEX = torch.complex128
MADFLOW_FLOAT = int(os.environ.get("MADFLOW_FLOAT", "64"))


def default_precision():
    from ._lib import MF_PREC_FP64, MF_PREC_MIXED

    return MF_PREC_MIXED if MADFLOW_FLOAT == 32 else MF_PREC_FP64


def device():
    """The CUDA device the library runs on (the current torch device)."""
    if not torch.cuda.is_available():
        raise RuntimeError("madflow_gb300 needs a CUDA device: there is no CPU fallback")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def float_me(x):
    return torch.as_tensor(x, dtype=DTYPE, device=device())


def int_me(x):
    return torch.as_tensor(x, dtype=DTYPEINT, device=device())


def complex_me(x):
    return torch.as_tensor(x, dtype=DTYPECOMPLEX, device=device())


def to_device(x, dtype=DTYPE):
    """Move an array-like to the library's device as a contiguous tensor."""
    if isinstance(x, torch.Tensor):
        return x.to(device=device(), dtype=dtype).contiguous()
    return torch.as_tensor(x, dtype=dtype, device=device()).contiguous()
