"""Vectorised NumPy FP64 restatement of the colour-ordered tt~ + k gluon
|M|^2, in the array style of madflow's CPU path: every wavefunction is a
[6, N] complex128 array over the event axis (the layout of
``wavefunctions_flow.py`` and of the generated ALOHA routines), every
helicity combination is evaluated separately (``matrix_method_python.inc:
80-104`` loops over them), and the colour sum is a dense quadratic form.

TEST INFRASTRUCTURE ONLY: used by ``tests/`` (against the C++ oracle) and by
the optional NumPy CPU-baseline leg of ``bench.py``.  The product package
never imports it.

The arithmetic follows the oracle's C++ restatement (``mf_oracle.hpp``) of
``wavefunctions_flow.py:56-747`` (ixxxxx, oxxxxx, vxxxxx), of the ALOHA
routines of ``tests/mockup_debug_me.py:43-397`` (FFV1_0, FFV1_1, VVV1P0_1)
and of the colour-ordered four-gluon current, organised as a Berends-Giele
recursion over the ordered gluon sequences.
"""
import itertools
import math

import numpy as np

SQH = 0.7071067690849304  # madflow's float32-rounded sqrt(1/2) (wavefunctions_flow.py:10)
C3 = -1j  # colour-ordered vertex factors of the oracle (three- and four-gluon)
C4 = -1.0


def _gluon_particle(j):
    return j if j < 2 else j + 2


def _plan(k):
    """Ordered gluon sequences (by length), their splits and contact triples,
    the top-line prefixes and the amplitude terms of every ordering."""
    seqs = [s for L in range(1, k + 1) for s in itertools.permutations(range(k), L)]
    jid = {s: i for i, s in enumerate(seqs)}
    j2 = [[(jid[s[:i]], jid[s[i:]]) for i in range(1, len(s))] for s in seqs]
    j3 = [[(jid[s[:i]], jid[s[i:j]], jid[s[j:]]) for i in range(1, len(s)) for j in range(i + 1, len(s))]
          for s in seqs]
    prefixes = [()] + [s for s in seqs if len(s) < k]
    oid = {s: i for i, s in enumerate(prefixes)}
    oterms = [[(oid[a[:i]], jid[a[i:]]) for i in range(len(a))] for a in prefixes]
    perms = list(itertools.permutations(range(k)))
    aterms = [[(oid[s[:i]], jid[s[i:]]) for i in range(k)] for s in perms]
    return seqs, j2, j3, prefixes, oterms, aterms


def _helicities(k):
    """MadGraph order: particle i's bit from the top; the t~ (particle 3)
    runs +1 then -1."""
    n = k + 2
    out = []
    for c in range(1 << n):
        h = [1.0 if (c >> (n - 1 - i)) & 1 else -1.0 for i in range(n)]
        h[3] = -h[3]
        out.append(h)
    return np.array(out)


# ---- external wavefunctions ([6, N] complex) --------------------------------

def vxxxxx_massless(p, nhel, nsv):
    """Massless vector polarisation (wavefunctions_flow.py:683-747); p [N, 4]."""
    N = p.shape[0]
    v = np.zeros((6, N), dtype=np.complex128)
    v[0] = p[:, 0] * nsv + 1j * p[:, 3] * nsv
    v[1] = p[:, 1] * nsv + 1j * p[:, 2] * nsv
    ppl = p[:, 0]
    ptl = np.sqrt(p[:, 1] ** 2 + p[:, 2] ** 2)
    v[5] = nhel * ptl / ppl * SQH
    nz = ptl != 0
    safe = np.where(nz, ptl, 1.0)
    pzpt = p[:, 3] / (ppl * safe) * SQH * nhel
    v[3] = np.where(nz, -p[:, 1] * pzpt - 1j * nsv * p[:, 2] / safe * SQH, -nhel * SQH)
    v[4] = np.where(nz, -p[:, 2] * pzpt + 1j * nsv * p[:, 1] / safe * SQH,
                    1j * nsv * SQH * np.sign(p[:, 3]) + 0 * p[:, 3])
    return v


def _massive_spinor(p, fmass, nh, nsf, conj_sign, outgoing):
    """The fmass != 0 branch shared by ixxxxx and oxxxxx; returns the four
    spinor components [4, N]."""
    pp = np.minimum(p[:, 0], np.sqrt(p[:, 1] ** 2 + p[:, 2] ** 2 + p[:, 3] ** 2))
    ip, im = int(math.floor((1 + nh) / 2)), int(math.floor((1 - nh) / 2))
    sf0 = (1 + nsf + (1 - nsf) * nh) * 0.5
    sf1 = (1 + nsf - (1 - nsf) * nh) * 0.5
    ppe = np.where(pp == 0, 1.0, pp)
    om = [np.sqrt(p[:, 0] + pp), fmass / np.sqrt(p[:, 0] + pp)]
    sfo0, sfo1 = sf0 * om[ip], sf1 * om[im]
    pp3 = np.maximum(pp + p[:, 3], 0.0)
    den = np.sqrt(2.0 * ppe * np.where(pp3 == 0, 1.0, pp3))
    chi1 = np.where(pp3 == 0, -nh + 0j, nh * p[:, 1] / den + 1j * conj_sign * p[:, 2] / den)
    chi = [np.sqrt(pp3 * 0.5 / ppe) + 0j, chi1]
    if outgoing:
        w = [sfo1 * chi[im], sfo1 * chi[ip], sfo0 * chi[im], sfo0 * chi[ip]]
    else:
        w = [sfo0 * chi[im], sfo0 * chi[ip], sfo1 * chi[im], sfo1 * chi[ip]]
    w = np.array(w)
    if np.any(pp == 0):  # at rest: wavefunctions_flow.py:370-392
        s0 = math.sqrt(abs(fmass))
        sqm = [s0, s0 * math.copysign(1.0, fmass)]
        if outgoing:
            nhel = nh * nsf
            ipp, imp = int(-math.floor((1 - nh) / 2) * nhel), int(math.floor((1 + nh) / 2) * nhel)
        else:
            ipp, imp = im, ip
        rest = np.array([imp * sqm[abs(imp)], ipp * nsf * sqm[abs(imp)], imp * nsf * sqm[abs(ipp)],
                         ipp * sqm[abs(ipp)]], dtype=np.complex128)
        w[:, pp == 0] = rest[:, None]
    return w


def ixxxxx_massive(p, fmass, nhel, nsf):
    """Incoming fermion spinor, massive (wavefunctions_flow.py:159-330)."""
    N = p.shape[0]
    f = np.zeros((6, N), dtype=np.complex128)
    f[0] = -p[:, 0] * nsf - 1j * p[:, 3] * nsf
    f[1] = -p[:, 1] * nsf - 1j * p[:, 2] * nsf
    f[2:] = _massive_spinor(p, fmass, nhel * nsf, nsf, 1.0, False)
    return f


def oxxxxx_massive(p, fmass, nhel, nsf):
    """Outgoing fermion spinor, massive (wavefunctions_flow.py:336-462)."""
    N = p.shape[0]
    f = np.zeros((6, N), dtype=np.complex128)
    f[0] = p[:, 0] * nsf + 1j * p[:, 3] * nsf
    f[1] = p[:, 1] * nsf + 1j * p[:, 2] * nsf
    f[2:] = _massive_spinor(p, fmass, nhel * nsf, nsf, -1.0, True)
    return f


# ---- vertices ---------------------------------------------------------------

def _mom(w):
    """(E, px, py, pz) [4, N] of a wavefunction's momentum slots."""
    return np.array([w[0].real, w[1].real, w[1].imag, w[0].imag])


def _mdot(a, b):
    return a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3]


def _s_apply(a, x):
    """y = S(a) x in the HELAS chiral basis; a, x [4, N]."""
    a12p, a12m = a[1] + 1j * a[2], a[1] - 1j * a[2]
    return np.array([(a[0] + a[3]) * x[2] + a12p * x[3],
                     a12m * x[2] + (a[0] - a[3]) * x[3],
                     (a[0] - a[3]) * x[0] - a12p * x[1],
                     -a12m * x[0] + (a[0] + a[3]) * x[1]])


def _denom(coup, P, M, W):
    return coup / ((P[0] ** 2 - P[1] ** 2 - P[2] ** 2 - P[3] ** 2) - M * M + 1j * M * W)


def FFV1_0(F1, F2, V3, coup):
    y = _s_apply(V3[2:], F2[2:])
    return coup * (-1j) * (F1[2] * y[0] + F1[3] * y[1] + F1[4] * y[2] + F1[5] * y[3])


def FFV1_1(F2, V3, coup, M1, W1):
    F1 = np.empty_like(F2)
    F1[0] = F2[0] + V3[0]
    F1[1] = F2[1] + V3[1]
    P = -_mom(F1)
    c = 1j * _denom(coup, P, M1, W1)
    y = _s_apply(V3[2:], F2[2:])
    z = _s_apply(-P + 0j, y)
    F1[2:] = c * (z + M1 * y)
    return F1


def VVV1P0_1(V2, V3, coup):
    """Massless off-shell gluon of the three-gluon vertex."""
    V1 = np.empty_like(V2)
    V1[0] = V2[0] + V3[0]
    V1[1] = V2[1] + V3[1]
    P2, P3, P1 = _mom(V2), _mom(V3), -_mom(V1)
    a, b = V2[2:], V3[2:]
    v23 = _mdot(b, a)
    c2 = _mdot(b, P2) - _mdot(b, P1)
    c3 = _mdot(a, P1) - _mdot(a, P3)
    c = 1j * _denom(coup, P1, 0.0, 0.0)
    V1[2:] = c * (v23 * (P3 - P2) + a * c2 + b * c3)
    return V1


def VVVV_ord_1(V2, V3, V4, coup):
    """Colour-ordered four-gluon contact current, leg 1 off shell."""
    V1 = np.empty_like(V2)
    V1[0] = V2[0] + V3[0] + V4[0]
    V1[1] = V2[1] + V3[1] + V4[1]
    P1 = -_mom(V1)
    a, b, d = V2[2:], V3[2:], V4[2:]
    c = 1j * _denom(coup, P1, 0.0, 0.0)
    V1[2:] = c * (2.0 * b * _mdot(a, d) - a * _mdot(b, d) - d * _mdot(a, b))
    return V1


# ---- |M|^2 ------------------------------------------------------------------

class TTNG:
    """g g > t t~ + (k - 2) g: colour-ordered partial amplitudes per
    helicity combination, vectorised over events."""

    def __init__(self, k, colour):
        self.k = k
        self.colour = np.asarray(colour, dtype=np.float64)
        self.seqs, self.j2, self.j3, self.prefixes, self.oterms, self.aterms = _plan(k)
        self.hels = _helicities(k)
        self.denominator = 256.0 * math.factorial(k - 2)

    def partials(self, p, hel, mt, wt, gc10, gc11, gc12):
        """A [nperm, N] for momenta p [N, k+2, 4] and one helicity vector."""
        k = self.k
        c3g, c4g = C3 * gc10, C4 * gc12
        wtop = oxxxxx_massive(p[:, 2], mt, hel[2], 1.0)
        wtb = ixxxxx_massive(p[:, 3], mt, hel[3], -1.0)
        J = []
        for i, s in enumerate(self.seqs):
            if len(s) == 1:
                part = _gluon_particle(s[0])
                J.append(vxxxxx_massless(p[:, part], hel[part], -1.0 if part < 2 else 1.0))
                continue
            acc = None
            for a, b in self.j2[i]:
                t = VVV1P0_1(J[a], J[b], c3g)
                acc = t if acc is None else np.concatenate([acc[:2], acc[2:] + t[2:]])
            for a, b, d in self.j3[i]:
                t = VVVV_ord_1(J[a], J[b], J[d], c4g)
                acc[2:] += t[2:]
            J.append(acc)
        O = [wtop]
        for terms in self.oterms[1:]:
            acc = None
            for o, j in terms:
                t = FFV1_1(O[o], J[j], gc11, mt, wt)
                acc = t if acc is None else np.concatenate([acc[:2], acc[2:] + t[2:]])
            O.append(acc)
        A = np.zeros((len(self.aterms), p.shape[0]), dtype=np.complex128)
        for s, terms in enumerate(self.aterms):
            for o, j in terms:
                A[s] += FFV1_0(wtb, O[o], J[j], gc11)
        return A

    def smatrix(self, p, mt, wt, gc10, gc11, gc12):
        """|M|^2 summed over helicities and colours, averaged over the
        initial ones: p [N, k+2, 4] -> [N]."""
        p = np.asarray(p, dtype=np.float64)
        tot = np.zeros(p.shape[0])
        for h in self.hels:
            A = self.partials(p, h, mt, wt, gc10, gc11, gc12)
            tot += np.einsum("ij,in,jn->n", self.colour, A.conj(), A).real
        return tot / self.denominator
