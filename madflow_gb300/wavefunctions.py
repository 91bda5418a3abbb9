"""External wavefunctions (madflow wavefunctions_flow.py) evaluated on the
GPU for a batch of momenta.  Each returns the reference's (6, N) complex128
tensor (3 slots for sxxxxx): slots 0-1 carry the momentum flow, 2-5 the
spinor or polarisation vector."""
import torch

from . import _lib
from .config import DTYPE, device, stream_ptr, to_device


def _run(name, p, *args, nslots=6):
    q = to_device(p)
    N = q.shape[0]
    pt = q.T.contiguous()
    out = torch.empty((nslots, 2, N), dtype=DTYPE, device=device())
    _lib.call(name, pt.data_ptr(), N, *[float(a) for a in args], out.data_ptr(), stream_ptr())
    return torch.view_as_complex(out.permute(0, 2, 1).contiguous())


def ixxxxx(p, fmass, nhel, nsf):
    """Incoming fermion (wavefunctions_flow.py:56-85)."""
    return _run("mf_ixxxxx", p, fmass, nhel, nsf)


def oxxxxx(p, fmass, nhel, nsf):
    """Outgoing fermion (wavefunctions_flow.py:89-116)."""
    return _run("mf_oxxxxx", p, fmass, nhel, nsf)


def vxxxxx(p, vmass, nhel, nsv):
    """Vector boson; nhel = 4 is the BRST check (wavefunctions_flow.py:120-154)."""
    return _run("mf_vxxxxx", p, vmass, nhel, nsv)


def sxxxxx(p, nss):
    """Scalar (wavefunctions_flow.py:34-51): [p0, p3] nss, [p1, p2] nss, 1."""
    return _run("mf_sxxxxx", p, nss, nslots=3)


def to_slots(w):
    """(6, N) complex -> [6][2][N] float64 device layout of the C ABI."""
    w = to_device(w, dtype=torch.complex128)
    return torch.view_as_real(w).permute(0, 2, 1).contiguous()
