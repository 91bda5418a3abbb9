"""ctypes front end of the CPU oracle (``mf_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by ``__graft_entry__.smoke``
to compare against, and by the CPU-baseline leg of ``bench.py``.  The product
package never imports it.

Each wrapper mirrors the madflow function it restates (same argument meaning,
numpy arrays in the reference's AoS layouts).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmf_oracle.so")
# the same source at -O3 with fused multiply-adds: the timed CPU baseline
FAST_LIB_PATH = os.path.join(HERE, "_build", "libmf_oracle_fast.so")
FAST_FLAGS = "-O3 -ffp-contract=fast -fno-math-errno -fopenmp"

_libs = {}
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)


def build(force=False):
    """Compile the oracle (parity build and timing build) with the committed
    Makefile (a few seconds)."""
    if force or any(not os.path.exists(p) or _stale(p) for p in (LIB_PATH, FAST_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _stale(path):
    so = os.path.getmtime(path)
    return any(os.path.getmtime(os.path.join(HERE, f)) > so for f in ("mf_oracle.cpp", "mf_oracle.hpp", "Makefile"))


def lib(fast=False):
    """The parity build, or with fast=True the timing build (-O3, fused
    multiply-adds; results agree with the parity build to rounding)."""
    if fast not in _libs:
        build()
        _lib = ctypes.CDLL(FAST_LIB_PATH if fast else LIB_PATH)
        _lib.orc_ttng_create.restype = ctypes.c_void_p
        _lib.orc_ttng_create.argtypes = [ctypes.c_int, _dp]
        for name in ("orc_ttng_destroy",):
            getattr(_lib, name).argtypes = [ctypes.c_void_p]
        _lib.orc_ttng_denominator.restype = ctypes.c_double
        _lib.orc_ttng_denominator.argtypes = [ctypes.c_void_p]
        _lib.orc_ttng_flops.restype = ctypes.c_double
        _lib.orc_ttng_flops.argtypes = [ctypes.c_void_p, _dp, _dp]
        _lib.orc_ggttx_flops.restype = ctypes.c_double
        _lib.orc_rambo.restype = ctypes.c_int
        _lib.orc_ramboflow.restype = ctypes.c_int
        _lib.orc_pass_cuts.restype = ctypes.c_int
        _lib.orc_num_threads.restype = ctypes.c_int
        _libs[fast] = _lib
    return _libs[fast]


def _p(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# --- constants the reference carries (float32-rounded Python literals)
PI_F32 = float(np.float32(np.pi))
SQH_F32 = float(np.float32(np.sqrt(np.float32(0.5))))
GEV2PB_F32 = float(np.float32(389379365.6))
NEWTON_BATCH, NEWTON_PER_EVENT = 0, 1


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def uniforms(seed, stream, iteration, event0, n, ndim):
    u = np.empty((n, ndim))
    lib().orc_uniforms(ctypes.c_uint64(seed), ctypes.c_uint32(stream), ctypes.c_uint32(iteration),
                       ctypes.c_uint64(event0), ctypes.c_int64(n), ctypes.c_int(ndim), _p(u))
    return u


def rambo(xrand, n_particles, sqrts, masses=None, f32q=True, rule=NEWTON_BATCH):
    x = _c64(xrand)
    N = x.shape[0]
    sq = _c64(np.broadcast_to(np.asarray(sqrts, dtype=np.float64), (N,)))
    m = None if masses is None else _c64(masses)
    p = np.empty((N, n_particles, 4))
    w = np.empty(N)
    it = lib().orc_rambo(_p(x), ctypes.c_int64(N), ctypes.c_int(n_particles), _p(sq), _p(m), ctypes.c_int(int(f32q)),
                         ctypes.c_int(rule), _p(p), _p(w))
    return p, w, it


def ramboflow(xrand, nparticles, com_sqrts, masses=None, f32q=True, rule=NEWTON_BATCH):
    x = _c64(xrand)
    N = x.shape[0]
    m = None if masses is None else _c64(masses)
    p = np.empty((N, nparticles, 4))
    w, x1, x2 = np.empty(N), np.empty(N), np.empty(N)
    lib().orc_ramboflow(_p(x), ctypes.c_int64(N), ctypes.c_int(nparticles), ctypes.c_double(com_sqrts), _p(m),
                        ctypes.c_int(int(f32q)), ctypes.c_int(rule), _p(p), _p(w), _p(x1), _p(x2))
    return p, w, x1, x2


def boost_to_lab(p, x1, x2):
    q = _c64(p).copy()
    lib().orc_boost_to_lab(_p(q), ctypes.c_int64(q.shape[0]), ctypes.c_int(q.shape[1]), _p(_c64(x1)), _p(_c64(x2)))
    return q


def _wf_call(fn, p, *args):
    p = _c64(p)
    out = np.empty((p.shape[0], 6, 2))
    fn(_p(p), ctypes.c_int64(p.shape[0]), *[ctypes.c_double(a) for a in args[:3]], *args[3:], _p(out))
    return (out[..., 0] + 1j * out[..., 1]).T  # (6, N) as the reference returns


def ixxxxx(p, fmass, nhel, nsf):
    return _wf_call(lib().orc_ixxxxx, p, fmass, nhel, nsf)


def oxxxxx(p, fmass, nhel, nsf):
    return _wf_call(lib().orc_oxxxxx, p, fmass, nhel, nsf)


def vxxxxx(p, vmass, nhel, nsv, f32q=True):
    return _wf_call(lib().orc_vxxxxx, p, vmass, nhel, nsv, ctypes.c_int(int(f32q)))


def _to_c(w):
    w = np.asarray(w).T  # (N, 6)
    return _c64(np.stack([w.real, w.imag], axis=-1))


def _coup(c):
    return _c64([complex(c).real, complex(c).imag])


def FFV1_0(F1, F2, V3, coup):
    a, b, c = _to_c(F1), _to_c(F2), _to_c(V3)
    out = np.empty((a.shape[0], 2))
    lib().orc_FFV1_0(_p(a), _p(b), _p(c), _p(_coup(coup)), ctypes.c_int64(a.shape[0]), _p(out))
    return out[:, 0] + 1j * out[:, 1]


def _cur(fn, A, B, coup, M, W):
    a, b = _to_c(A), _to_c(B)
    out = np.empty((a.shape[0], 6, 2))
    fn(_p(a), _p(b), _p(_coup(coup)), ctypes.c_double(M), ctypes.c_double(W), ctypes.c_int64(a.shape[0]), _p(out))
    return (out[..., 0] + 1j * out[..., 1]).T


def FFV1_1(F2, V3, coup, M1, W1):
    return _cur(lib().orc_FFV1_1, F2, V3, coup, M1, W1)


def FFV1_2(F1, V3, coup, M2, W2):
    return _cur(lib().orc_FFV1_2, F1, V3, coup, M2, W2)


def VVV1P0_1(V2, V3, coup, M1, W1):
    return _cur(lib().orc_VVV1P0_1, V2, V3, coup, M1, W1)


def smatrix_ggttx(all_ps, mdl_MT, mdl_WT, GC_10, GC_11, per_helicity=False, f32q=True):
    p = _c64(all_ps)
    N = p.shape[0]
    prm = _c64([mdl_MT, mdl_WT, complex(GC_10).real, complex(GC_10).imag, complex(GC_11).real, complex(GC_11).imag])
    out = np.empty(N)
    hel = np.empty((16, N)) if per_helicity else None
    lib().orc_smatrix_ggttx(_p(p), ctypes.c_int64(N), _p(prm), ctypes.c_int(int(f32q)), _p(out), _p(hel))
    return (out, hel) if per_helicity else out


# Colour-ordered vertex factors of the tt~ + n g recursion (see mf_oracle.cpp):
# c3 multiplies GC_10 in the ordered three-gluon current, c4 multiplies GC_12
# in the ordered four-gluon current.  c3 = -i reproduces the frozen gg -> tt~
# module; c4 = -1 makes every colour-ordered amplitude gauge invariant and
# matches the colour-dressed full Feynman rules (tests/test_physics_checks.py).
C3 = -1j
C4 = -1.0


class TTNG:
    """tt~ + k gluons (k = total number of gluons, 2..5) in the oracle."""

    def __init__(self, k, colour=None, fast=False):
        self.k, self.fast = k, fast
        L = lib(fast)
        c = None if colour is None else _c64(colour)
        self.h = L.orc_ttng_create(ctypes.c_int(k), _p(c))
        info = (ctypes.c_int * 6)()
        L.orc_ttng_info(ctypes.c_void_p(self.h), info)
        self.nperm, self.njnode, self.nonode, self.ncomb, self.npart = info[1], info[2], info[3], info[4], info[5]
        self.denominator = L.orc_ttng_denominator(ctypes.c_void_p(self.h))

    def __del__(self):
        try:
            lib(self.fast).orc_ttng_destroy(ctypes.c_void_p(self.h))
        except Exception:
            pass

    @property
    def colour(self):
        out = np.empty((self.nperm, self.nperm))
        lib().orc_ttng_colour(ctypes.c_void_p(self.h), _p(out))
        return out

    @property
    def helicities(self):
        out = np.empty((self.ncomb, self.npart))
        lib().orc_ttng_helicities(ctypes.c_void_p(self.h), _p(out))
        return out

    @staticmethod
    def params(mt, wt, gc10, gc11, gc12, c3=None, c4=None):
        c3 = C3 if c3 is None else c3
        c4 = C4 if c4 is None else c4
        v = [mt, wt, gc10, gc11, gc12, c3, c4]
        out = [v[0], v[1]]
        for z in v[2:]:
            out += [complex(z).real, complex(z).imag]
        return _c64(out)

    def partials(self, p, hel, prm, f32q=True):
        out = np.empty((self.nperm, 2))
        lib().orc_ttng_partials(ctypes.c_void_p(self.h), _p(_c64(p)), _p(_c64(hel)), _p(prm), ctypes.c_int(int(f32q)),
                                _p(out))
        return out[:, 0] + 1j * out[:, 1]

    def smatrix(self, all_ps, prm, per_helicity=False, f32q=True):
        p = _c64(all_ps)
        N = p.shape[0]
        out = np.empty(N)
        hel = np.empty((self.ncomb, N)) if per_helicity else None
        lib().orc_ttng_smatrix(ctypes.c_void_p(self.h), _p(p), ctypes.c_int64(N), _p(prm), ctypes.c_int(int(f32q)),
                               _p(out), _p(hel))
        return (out, hel) if per_helicity else out

    def flops(self, p, prm):
        return lib().orc_ttng_flops(ctypes.c_void_p(self.h), _p(_c64(p)), _p(prm))


def ttng_dressed(k, p, hel, colours, prm, s3=1.0, kappa=0j, f32q=True):
    out = np.empty(2)
    col = (ctypes.c_int * len(colours))(*colours)
    lib().orc_ttng_dressed(ctypes.c_int(k), _p(_c64(p)), _p(_c64(hel)), col, _p(prm), ctypes.c_double(s3),
                           ctypes.c_double(complex(kappa).real), ctypes.c_double(complex(kappa).imag),
                           ctypes.c_int(int(f32q)), _p(out))
    return out[0] + 1j * out[1]


def colour_string(labels, i, j):
    out = np.empty(2)
    arr = (ctypes.c_int * len(labels))(*labels)
    lib().orc_colour_string(ctypes.c_int(len(labels)), arr, ctypes.c_int(i), ctypes.c_int(j), _p(out))
    return out[0] + 1j * out[1]


def colour_matrix(k):
    import math

    n = math.factorial(k)
    out = np.empty((n, n))
    lib().orc_colour_matrix(ctypes.c_int(k), _p(out))
    return out


def ggttx_flops(p, prm6):
    return lib().orc_ggttx_flops(_p(_c64(p)), _p(_c64(prm6)))


def smatrix_uux_ttx(all_ps, mdl_MT, mdl_WT, GC_11):
    """q q~ > t t~ |M|^2 (averaged) for momenta (N, 4, 4) ordered q, q~, t, t~."""
    p = _c64(all_ps)
    out = np.empty(p.shape[0])
    prm = _c64([mdl_MT, mdl_WT, complex(GC_11).real, complex(GC_11).imag])
    lib().orc_smatrix_uux_ttx(_p(p), ctypes.c_int64(p.shape[0]), _p(prm), _p(out))
    return out


QQ3_CHANNELS = {"uux_ttxg": 0, "ug_ttxu": 1, "uxg_ttxux": 2}


def smatrix_qq3(channel, all_ps, mdl_MT, mdl_WT, GC_10, GC_11, f32q=True):
    """|M|^2 (averaged) of the light-quark channels of p p > t t~ j for
    momenta (N, 5, 4): "uux_ttxg" (q q~ > t t~ g), "ug_ttxu" (q g > t t~ q),
    "uxg_ttxux" (q~ g > t t~ q~), MadGraph's particle order.  f32q: madflow's
    float32 sqrt(1/2) in the gluon polarisations."""
    p = _c64(all_ps)
    out = np.empty(p.shape[0])
    prm = _c64([mdl_MT, mdl_WT, complex(GC_10).real, complex(GC_10).imag, complex(GC_11).real, complex(GC_11).imag])
    if lib().orc_smatrix_qq3(ctypes.c_int(QQ3_CHANNELS[channel]), _p(p), ctypes.c_int64(p.shape[0]), _p(prm),
                             ctypes.c_int(int(bool(f32q))), _p(out)):
        raise ValueError(channel)
    return out


def pdf_xfx(x, q2):
    x = _c64(x)
    out = np.empty_like(x)
    lib().orc_pdf_xfx(_p(x), ctypes.c_int64(x.size), ctypes.c_double(q2), _p(out))
    return out


def pdf_xfx_flavour(pdg, x, q2):
    """x f(x, Q^2) of the synthetic density of flavour pdg (21 gluon, 1..4 d u s
    c, negative: antiquarks)."""
    x = _c64(x)
    out = np.empty_like(x)
    if lib().orc_pdf_xfx_flavour(ctypes.c_int(pdg), _p(x), ctypes.c_int64(x.size), ctypes.c_double(q2), _p(out)):
        raise ValueError(f"no synthetic density for flavour {pdg}")
    return out


def pdf_table():
    tab = np.empty((50, 100))
    vals = [ctypes.c_double() for _ in range(4)]
    lib().orc_pdf_table(_p(tab), *[ctypes.byref(v) for v in vals])
    return tab, [v.value for v in vals]


def vegas_sample(div, u):
    div = _c64(div)
    u = _c64(u)
    N, ndim = u.shape
    nb = div.shape[1] - 1
    x = np.empty((N, ndim))
    jac = np.empty(N)
    bins = np.empty((N, ndim), dtype=np.int32)
    lib().orc_vegas_sample(_p(div), ctypes.c_int(ndim), ctypes.c_int(nb), _p(u), ctypes.c_int64(N), _p(x), _p(jac),
                           bins.ctypes.data_as(_ip))
    return x, jac, bins


def vegas_accumulate(fw, bins, nb):
    fw = _c64(fw)
    bins = np.ascontiguousarray(bins, dtype=np.int32)
    N, ndim = bins.shape
    sums = np.zeros(2)
    hist = np.zeros((ndim, nb))
    lib().orc_vegas_accumulate(_p(fw), bins.ctypes.data_as(_ip), ctypes.c_int64(N), ctypes.c_int(ndim),
                               ctypes.c_int(nb), _p(sums), _p(hist))
    return sums, hist


def vegas_refine(div, hist, alpha=1.5):
    d = _c64(div).copy()
    h = _c64(hist)
    lib().orc_vegas_refine(_p(d), _p(h), ctypes.c_int(d.shape[0]), ctypes.c_int(d.shape[1] - 1), ctypes.c_double(alpha))
    return d


def pass_cuts(plab, ptmin, etamax, drmin):
    plab = _c64(plab)
    return bool(lib().orc_pass_cuts(_p(plab), ctypes.c_int(plab.shape[0]), ctypes.c_double(ptmin),
                                    ctypes.c_double(etamax), ctypes.c_double(drmin)))


def integrand(cfg, x, plan=None, fast=False):
    """cfg: [kind, k, sqrts, mt, wt, alphas, ptmin, etamax, drmin, newton_rule
    (, initial_states: 0 g g, 1 p p (, dynamic scale: 0 fixed Q = mt, 1
    madflow's sum of m_T / 2 with alphas = alpha_s(M_Z^2) (, pt_all: > 0
    madflow's --pt_cut on every outgoing particle (, the registered cuts as
    cut_vector gives them))))].  fast: the timing build (plan, if given,
    must come from the same build)."""
    if plan is not None:
        fast = plan.fast
    cfg = list(cfg) + [0] * (14 - len(cfg))
    x = _c64(x)
    f = np.empty(x.shape[0])
    lib(fast).orc_integrand(_p(_c64(cfg)), ctypes.c_void_p(plan.h if plan is not None else None), _p(x),
                            ctypes.c_int64(x.shape[0]), _p(f))
    return f


CUT_VARIABLES = {"pt": 0, "mt": 1, "mt2": 2, "eta": 3}


def cut_vector(cuts):
    """The integrand configuration's tail for registered cuts:
    (variable, particle, min_val, max_val) tuples (None: no bound)."""
    out = [len(cuts)]
    for variable, particle, lo, hi in cuts:
        out += [CUT_VARIABLES[variable], particle, int(lo is not None), int(hi is not None),
                0.0 if lo is None else float(lo), 0.0 if hi is None else float(hi)]
    return out


def num_threads(fast=False):
    return lib(fast).orc_num_threads()
