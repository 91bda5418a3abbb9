"""The generated per-process matrix-element modules of madflow, as classes
backed by the CUDA kernels.

madflow's PyOut exporter writes a ``Matrix_<proc>`` class per process
(madgraph_plugin/template_files/matrix_method_python.inc:56-138) whose
``smatrix(all_ps, <masses/widths>, <couplings>)`` returns |M|^2 summed over
helicities and colours and averaged, and ``matrix(all_ps, hel, ...)`` one
helicity.  The classes here keep that call for g g > t t~ + n gluons; the
parameters follow the reference order, sorted masses/widths then sorted
couplings (PyOut_exporter.py:244, 378-407): mdl_MT, mdl_WT, GC_10, GC_11,
GC_12.  Couplings may be scalars or per-event complex tensors (running
alpha_s).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .config import DTYPE, DTYPECOMPLEX, default_precision, device, stream_ptr, to_device


class _Process:
    """Owner of one mf_process handle."""

    def __init__(self, n_gluons, precision):
        h = ctypes.c_void_p()
        _lib.call("mf_process_create", n_gluons, precision, ctypes.byref(h))
        self.h = h
        vals = [ctypes.c_int() for _ in range(4)]
        den = ctypes.c_double()
        _lib.call("mf_process_info", self.h, *[ctypes.byref(v) for v in vals], ctypes.byref(den))
        self.nexternal, self.ncomb, self.ncolor, self.ndiags = (v.value for v in vals)
        self.denominator = den.value
        hel = (ctypes.c_double * (self.ncomb * self.nexternal))()
        _lib.call("mf_process_helicities", self.h, hel)
        self.helicities = np.array(hel[:], dtype=np.float64).reshape(self.ncomb, self.nexternal)
        col = (ctypes.c_double * (self.ncolor * self.ncolor))()
        _lib.call("mf_process_colour_matrix", self.h, col)
        self.colour_matrix = np.array(col[:], dtype=np.float64).reshape(self.ncolor, self.ncolor)

    def __del__(self):
        try:
            if self.h:
                _lib.load().mf_process_destroy(self.h)
        except Exception:
            pass


class MatrixTTNG:
    """g g > t t~ + (n_gluons - 2) g."""

    n_gluons = 2
    process_string = "gg_ttx"
    initial_states = [(21, 21)]
    mirror_initial_states = False

    def __init__(self, precision=None):
        self.precision = default_precision() if precision is None else precision
        self._proc = _Process(self.n_gluons, self.precision)
        p = self._proc
        self.nexternal = float(p.nexternal)
        self.ndiags = float(p.ndiags)
        self.ncomb = float(p.ncomb)
        self.helicities = torch.tensor(p.helicities, dtype=DTYPE)
        self.denominator = float(p.denominator)
        self.colour_matrix = p.colour_matrix

    def __str__(self):
        return self.process_string

    @property
    def handle(self):
        return self._proc.h

    def _couplings(self, N, GC_10, GC_11, GC_12):
        cs = []
        per_event = False
        for c in (GC_10, GC_11, GC_12):
            if c is None:
                c = 0j
            if isinstance(c, torch.Tensor) and c.numel() > 1:
                per_event = True
            cs.append(c)
        if per_event:
            cols = []
            for c in cs:
                t = torch.as_tensor(c, dtype=DTYPECOMPLEX, device=device()).reshape(-1)
                cols.append(t.expand(N) if t.numel() == 1 else t)
            arr = torch.view_as_real(torch.stack(cols, dim=1)).reshape(N, 6).contiguous()
            return arr, 1
        flat = []
        for c in cs:
            c = complex(c.item() if isinstance(c, torch.Tensor) else c)
            flat += [c.real, c.imag]
        return torch.tensor(flat, dtype=DTYPE, device=device()), 0

    def _run(self, all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12, with_hel):
        ps = to_device(all_ps)
        if ps.dim() != 3 or ps.shape[1] != self._proc.nexternal or ps.shape[2] != 4:
            raise ValueError(f"all_ps must have shape (N, {self._proc.nexternal}, 4), got {tuple(ps.shape)}")
        N = ps.shape[0]
        soa = ps.permute(1, 2, 0).contiguous()
        coup, stride = self._couplings(N, GC_10, GC_11, GC_12)
        out = torch.empty(N, dtype=DTYPE, device=device())
        hel = torch.empty((self._proc.ncomb, N), dtype=DTYPE, device=device()) if with_hel else None
        _lib.call("mf_smatrix", self.handle, soa.data_ptr(), N, float(mdl_MT), float(mdl_WT), coup.data_ptr(), stride,
                  out.data_ptr(), hel.data_ptr() if with_hel else None, stream_ptr())
        return out, hel

    def tuning(self):
        """Launch configuration of the matrix-element kernel (see
        mf_process_tuning): dict(colour, waves, tuned, variant_ms)."""
        c, w, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_float * _lib.MF_TUNE_VARIANTS)()
        _lib.call("mf_process_tuning", self.handle, ctypes.byref(c), ctypes.byref(w), ctypes.byref(t), ms)
        return dict(colour=c.value, waves=w.value, tuned=bool(t.value), variant_ms=[float(v) for v in ms])

    def set_tuning(self, colour, waves):
        """Fix the launch configuration (colour 0 SIMT / 1 tensor cores; waves 1, 2, 4, 8)."""
        _lib.call("mf_process_set_tuning", self.handle, int(colour), int(waves))

    def smatrix(self, all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12=None):
        """|M|^2 averaged over initial and summed over final helicities and colours."""
        return self._run(all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12, False)[0]

    def cusmatrix(self, *args):
        """madflow's custom-operator variant of smatrix (the method its
        custom_op/generation.py:259-283 adds to the module, called by
        scripts/madflow_exec.py:404, 446 with --custom_op): here the same
        CUDA evaluation as smatrix."""
        return self.smatrix(*args)

    def smatrix_per_helicity(self, all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12=None):
        """(smatrix, per-helicity matrix values (ncomb, N))."""
        return self._run(all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12, True)

    def matrix(self, all_ps, hel, mdl_MT, mdl_WT, GC_10, GC_11, GC_12=None):
        """|M|^2 of one helicity combination, summed over colours."""
        h = np.asarray(torch.as_tensor(hel).cpu(), dtype=np.float64).reshape(-1)
        idx = np.where((self._proc.helicities == h).all(axis=1))[0]
        if len(idx) != 1:
            raise ValueError(f"helicity {h.tolist()} is not one of the process combinations")
        _, per = self._run(all_ps, mdl_MT, mdl_WT, GC_10, GC_11, GC_12, True)
        return per[int(idx[0])]


class Matrix_1_gg_ttx(MatrixTTNG):
    """g g > t t~ (3 diagrams, 2 colour flows, 16 helicities); the process of
    madflow's frozen test module tests/mockup_debug_me.py:419-543."""

    n_gluons = 2
    process_string = "1_gg_ttx"


class Matrix_1_gg_ttxg(MatrixTTNG):
    """g g > t t~ g (16 diagrams, 6 colour flows, 32 helicities)."""

    n_gluons = 3
    process_string = "1_gg_ttxg"


class Matrix_1_gg_ttxgg(MatrixTTNG):
    """g g > t t~ g g (123 diagrams, 24 colour flows, 64 helicities)."""

    n_gluons = 4
    process_string = "1_gg_ttxgg"


class Matrix_1_gg_ttxggg(MatrixTTNG):
    """g g > t t~ g g g (1240 diagrams, 120 colour flows, 128 helicities)."""

    n_gluons = 5
    process_string = "1_gg_ttxggg"


PROCESSES = {2: Matrix_1_gg_ttx, 3: Matrix_1_gg_ttxg, 4: Matrix_1_gg_ttxgg, 5: Matrix_1_gg_ttxggg}


class Matrix_1_uux_ttx:
    """q q~ > t t~ (1 diagram, 2 colour flows, 16 helicities): the
    light-quark processes of madflow's p p > t t~ run, one module for the
    flavours d u s c as MadGraph groups them (initial states and their mirror
    images).  smatrix(all_ps, mdl_MT, mdl_WT, GC_11) with all_ps (N, 4, 4)
    ordered q, q~, t, t~ (C ABI mf_smatrix_qq_ttx)."""

    process_string = "1_uux_ttx"
    initial_states = [(2, -2), (4, -4), (1, -1), (3, -3)]
    mirror_initial_states = True
    nexternal = 4.0
    ndiags = 1.0
    ncomb = 16.0
    denominator = 36.0

    def __init__(self, precision=None):
        self.precision = default_precision() if precision is None else precision
        h = [[a, b, c, d] for a in (-1, 1) for b in (-1, 1) for c in (-1, 1) for d in (-1, 1)]
        self.helicities = torch.tensor(h, dtype=DTYPE)

    def __str__(self):
        return self.process_string

    def cusmatrix(self, *args):
        """madflow's custom-operator variant of smatrix: the same evaluation."""
        return self.smatrix(*args)

    def smatrix(self, all_ps, mdl_MT, mdl_WT, GC_11):
        """|M|^2 averaged over the initial spins (4) and colours (9)."""
        ps = to_device(all_ps)
        if ps.dim() != 3 or ps.shape[1] != 4 or ps.shape[2] != 4:
            raise ValueError(f"all_ps must have shape (N, 4, 4), got {tuple(ps.shape)}")
        N = ps.shape[0]
        soa = ps.permute(1, 2, 0).contiguous()
        coup, stride = MatrixTTNG._couplings(self, N, None, GC_11, None)
        out = torch.empty(N, dtype=DTYPE, device=device())
        _lib.call("mf_smatrix_qq_ttx", int(self.precision), soa.data_ptr(), N, float(mdl_MT), float(mdl_WT),
                  coup.data_ptr(), stride, out.data_ptr(), stream_ptr())
        return out


class _MatrixQQ3:
    """A light-quark process of p p > t t~ j (5 diagrams, 32 helicities; one
    module for the flavours d u s c as MadGraph groups them, initial states
    and their mirror images).  smatrix(all_ps, mdl_MT, mdl_WT, GC_10, GC_11)
    with all_ps (N, 5, 4) in MadGraph's particle order (C ABI
    mf_smatrix_qq_ttxj)."""

    channel = None
    mirror_initial_states = True
    nexternal = 5.0
    ndiags = 5.0
    ncomb = 32.0

    def __init__(self, precision=None):
        self.precision = default_precision() if precision is None else precision
        h = [[a, b, c, d, e] for a in (-1, 1) for b in (-1, 1) for c in (-1, 1) for d in (-1, 1) for e in (-1, 1)]
        self.helicities = torch.tensor(h, dtype=DTYPE)

    def __str__(self):
        return self.process_string

    def cusmatrix(self, *args):
        """madflow's custom-operator variant of smatrix: the same evaluation."""
        return self.smatrix(*args)

    def smatrix(self, all_ps, mdl_MT, mdl_WT, GC_10, GC_11):
        """|M|^2 averaged over the initial spins and colours."""
        ps = to_device(all_ps)
        if ps.dim() != 3 or ps.shape[1] != 5 or ps.shape[2] != 4:
            raise ValueError(f"all_ps must have shape (N, 5, 4), got {tuple(ps.shape)}")
        N = ps.shape[0]
        soa = ps.permute(1, 2, 0).contiguous()
        coup, stride = MatrixTTNG._couplings(self, N, GC_10, GC_11, None)
        out = torch.empty(N, dtype=DTYPE, device=device())
        _lib.call("mf_smatrix_qq_ttxj", int(self.precision), int(self.channel), soa.data_ptr(), N, float(mdl_MT),
                  float(mdl_WT), coup.data_ptr(), stride, out.data_ptr(), stream_ptr())
        return out


class Matrix_1_uux_ttxg(_MatrixQQ3):
    """q q~ > t t~ g, particles q, q~, t, t~, g; averaged over 4 spins and 9
    colours."""

    process_string = "1_uux_ttxg"
    channel = 0
    initial_states = [(2, -2), (4, -4), (1, -1), (3, -3)]
    denominator = 36.0


class Matrix_1_ug_ttxu(_MatrixQQ3):
    """q g > t t~ q, particles q, g, t, t~, q; averaged over 4 spins and 24
    colours."""

    process_string = "1_ug_ttxu"
    channel = 1
    initial_states = [(2, 21), (4, 21), (1, 21), (3, 21)]
    denominator = 96.0


class Matrix_1_uxg_ttxux(_MatrixQQ3):
    """q~ g > t t~ q~, particles q~, g, t, t~, q~; averaged over 4 spins and
    24 colours."""

    process_string = "1_uxg_ttxux"
    channel = 2
    initial_states = [(-2, 21), (-4, 21), (-1, 21), (-3, 21)]
    denominator = 96.0


def smatrix_multi(batches, mdl_MT, mdl_WT, GC_10, GC_11, GC_12=None):
    """|M|^2 of several processes in one persistent launch (C ABI
    ``mf_smatrix_multi``): batches is a list of (matrix, all_ps) with distinct
    matrix objects of one precision; scalar couplings shared by all.  Returns
    the list of results, one per batch."""
    if not batches or len(batches) > 4:
        raise ValueError("one to four batches")
    handles, ptrs, ns, outs, keep = [], [], [], [], []
    coup = None
    for m, all_ps in batches:
        ps = to_device(all_ps)
        if ps.dim() != 3 or ps.shape[1] != m._proc.nexternal or ps.shape[2] != 4:
            raise ValueError(f"all_ps must have shape (N, {m._proc.nexternal}, 4), got {tuple(ps.shape)}")
        n = ps.shape[0]
        soa = ps.permute(1, 2, 0).contiguous()
        out = torch.empty(n, dtype=DTYPE, device=device())
        c, stride = m._couplings(n, GC_10, GC_11, GC_12)
        if stride != 0:
            raise ValueError("smatrix_multi takes scalar couplings")
        coup = c
        keep += [soa, out]
        handles.append(m.handle)
        ptrs.append(soa.data_ptr())
        ns.append(n)
        outs.append(out)
    k = len(batches)
    _lib.call("mf_smatrix_multi", (ctypes.c_void_p * k)(*handles), k, (ctypes.c_void_p * k)(*ptrs),
              (ctypes.c_int64 * k)(*ns), float(mdl_MT), float(mdl_WT), coup.data_ptr(),
              (ctypes.c_void_p * k)(*[o.data_ptr() for o in outs]), stream_ptr())
    return outs
