"""Quick-start integration helpers (madflow utilities.py)."""
import math

import torch

from . import _lib
from .phasespace import ramboflow
from .vegas import vegas_wrapper


def generate_initial_states(matrices):
    """List of ([flavours hadron 1], [flavours hadron 2]) per matrix
    (utilities.py:25-39)."""
    initial_flavours = []
    for matrix in matrices:
        initials = matrix.initial_states
        flavs_1, flavs_2 = zip(*initials)
        if matrix.mirror_initial_states:
            m2, m1 = zip(*initials)
            flavs_1 += m1
            flavs_2 += m2
        initial_flavours.append((flavs_1, flavs_2))
    return initial_flavours


def one_matrix_integration(matrix, model_params, sqrts=7e3, n_events=int(1e5), n_iter=5, q=91.46, pdf=None,
                           flavours=None, out_masses=None, seed=4):
    """Integrate one matrix element (utilities.py:56-90).

    ``pdf`` is a callable xfx(x, q2) -> x f(x) (None: luminosity 1); the
    integrand is f = smatrix(ramboflow(x)) * lum(x1, x2) * weight."""
    nparticles = int(matrix.nexternal)
    q2 = float(q) ** 2

    def cross_section(xrand, **kwargs):
        all_ps, wts, x1, x2 = ramboflow(xrand, nparticles, sqrts, masses=out_masses)
        sm = matrix.smatrix(all_ps, *model_params)
        if pdf is None:
            lum = torch.ones_like(x1)
        else:
            lum = pdf(x1, q2) * pdf(x2, q2) / x1 / x2
        return sm * lum * wts

    ndim = (nparticles - 2) * 4 + 2
    return vegas_wrapper(cross_section, ndim, n_iter, n_events, seed=seed)


def synthetic_pdf(x, q2, pdg=21):
    """x f(x) of the synthetic density of flavour pdg (GPU table lookup): the
    gluon x g(x) = A x^-0.2 (1-x)^5 (pdg 21) or a light quark or antiquark
    (pdg +-1..+-4, see mf_pdf_xfx_flavour)."""
    from .config import stream_ptr, to_device

    xv = to_device(x).reshape(-1)
    out = torch.empty_like(xv)
    if pdg == 21:
        _lib.call("mf_pdf_xfx", xv.data_ptr(), xv.numel(), float(q2), out.data_ptr(), stream_ptr())
    else:
        _lib.call("mf_pdf_xfx_flavour", int(pdg), xv.data_ptr(), xv.numel(), float(q2), out.data_ptr(),
                  stream_ptr())
    return out.reshape(torch.as_tensor(x).shape) if not isinstance(x, torch.Tensor) else out.reshape(x.shape)


def alphas_to_couplings(alpha_s):
    """(GC_10, GC_11, GC_12) of the SM QCD vertices for a given alpha_s."""
    g = 2.0 * math.sqrt(math.pi * alpha_s)
    return -g, 1j * g, 1j * g * g
