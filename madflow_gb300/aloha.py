"""The ALOHA vertex/propagator routines madflow's generated modules call
(tests/mockup_debug_me.py: FFV1_0 :43, FFV1_1 :67, FFV1_2 :207, VVV1P0_1 :341),
batched on the GPU.  Wavefunctions are (6, N) complex tensors."""
import torch

from . import _lib
from .config import DTYPE, device, stream_ptr
from .wavefunctions import to_slots


def _coup(c):
    c = complex(c)
    return _lib.dbl_array([c.real, c.imag])


def FFV1_0(F1, F2, V3, COUP):
    a, b, c = to_slots(F1), to_slots(F2), to_slots(V3)
    N = a.shape[-1]
    out = torch.empty((2, N), dtype=DTYPE, device=device())
    _lib.call("mf_FFV1_0", a.data_ptr(), b.data_ptr(), c.data_ptr(), _coup(COUP), N, out.data_ptr(), stream_ptr())
    return torch.complex(out[0], out[1])


def _current(name, A, B, COUP, M, W):
    a, b = to_slots(A), to_slots(B)
    N = a.shape[-1]
    out = torch.empty((6, 2, N), dtype=DTYPE, device=device())
    _lib.call(name, a.data_ptr(), b.data_ptr(), _coup(COUP), float(M), float(W), N, out.data_ptr(), stream_ptr())
    return torch.view_as_complex(out.permute(0, 2, 1).contiguous())


def FFV1_1(F2, V3, COUP, M1, W1):
    return _current("mf_FFV1_1", F2, V3, COUP, M1, W1)


def FFV1_2(F1, V3, COUP, M2, W2):
    return _current("mf_FFV1_2", F1, V3, COUP, M2, W2)


def VVV1P0_1(V2, V3, COUP, M1, W1):
    return _current("mf_VVV1P0_1", V2, V3, COUP, M1, W1)
