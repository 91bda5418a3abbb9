"""Tree-level |M|^2 of the top-pair processes with one light-quark line,
evaluated from the textbook QCD Feynman rules, independently of the HELAS /
ALOHA routines the oracle and the CUDA library use.  TEST INFRASTRUCTURE: an
independent check of the quark channels of p p > t t~ (+ jet), which have no
reference output.

Conventions (Peskin & Schroeder): metric (+,-,-,-); Dirac representation of
the gamma matrices; spinors u(p,s) = (sqrt(E+m) xi, sigma.p xi / sqrt(E+m)),
v(p,s) = (sigma.p eta / sqrt(E+m), sqrt(E+m) eta) with xi, eta the two unit
two-spinors (a complete spin basis); gluons summed over two real transverse
polarisation vectors (physical polarisations, so no ghosts); Feynman gauge.
Vertices i g gamma^mu T^a and g f^abc [g^{mu nu}(k-p)^rho + g^{nu rho}(p-q)^mu
+ g^{rho mu}(q-k)^nu] (all momenta incoming), propagators
i (qslash + m) / (q^2 - m^2 + i m Gamma) and -i g_{mu nu} / q^2.  Colour:
T^a = lambda^a / 2 (Gell-Mann), f^abc = -2 i Tr([T^a, T^b] T^c), every colour
of every external leg summed explicitly through the diagrams' colour tensors.

Momenta: (N, n, 4) arrays (E, px, py, pz), MadGraph's particle order of each
process (see each function).  Returns |M|^2 averaged over the initial spins
and colours."""
import itertools

import numpy as np

_SIG = [np.array([[0, 1], [1, 0]], complex), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]], complex)]
_I2, _Z2 = np.eye(2, dtype=complex), np.zeros((2, 2), complex)
GAM = np.array([np.block([[_I2, _Z2], [_Z2, -_I2]])] + [np.block([[_Z2, s], [-s, _Z2]]) for s in _SIG])
_METRIC = np.array([1.0, -1.0, -1.0, -1.0])


def _gell_mann():
    lam = np.zeros((8, 3, 3), complex)
    lam[0][0, 1] = lam[0][1, 0] = 1
    lam[1][0, 1], lam[1][1, 0] = -1j, 1j
    lam[2][0, 0], lam[2][1, 1] = 1, -1
    lam[3][0, 2] = lam[3][2, 0] = 1
    lam[4][0, 2], lam[4][2, 0] = -1j, 1j
    lam[5][1, 2] = lam[5][2, 1] = 1
    lam[6][1, 2], lam[6][2, 1] = -1j, 1j
    lam[7] = np.diag([1, 1, -2]) / np.sqrt(3)
    return lam / 2


T = _gell_mann()
F = np.real(-2j * (np.einsum("aij,bjk,cki->abc", T, T, T) - np.einsum("bij,ajk,cki->abc", T, T, T)))


def mdot(a, b):
    return a[..., 0] * b[..., 0] - a[..., 1] * b[..., 1] - a[..., 2] * b[..., 2] - a[..., 3] * b[..., 3]


def slash(p):
    """p_mu gamma^mu for p (..., 4) with upper indices."""
    return np.einsum("...m,mab->...ab", (p * _METRIC).astype(complex), GAM)


def _sigma_p(p):
    return np.einsum("...i,iab->...ab", p[..., 1:].astype(complex), np.array(_SIG))


def u_spinor(p, m, s):
    E = p[..., 0]
    xi = np.zeros(p.shape[:-1] + (2,), complex)
    xi[..., s] = 1.0
    r = np.sqrt(E + m)[..., None]
    return np.concatenate([r * xi, np.einsum("...ab,...b->...a", _sigma_p(p), xi) / r], axis=-1)


def v_spinor(p, m, s):
    E = p[..., 0]
    eta = np.zeros(p.shape[:-1] + (2,), complex)
    eta[..., s] = 1.0
    r = np.sqrt(E + m)[..., None]
    return np.concatenate([np.einsum("...ab,...b->...a", _sigma_p(p), eta) / r, r * eta], axis=-1)


def bar(psi):
    return np.einsum("...a,ab->...b", psi.conj(), GAM[0])


def polarisations(k):
    """Two real transverse polarisation vectors (0, e1), (0, e2) of a
    massless momentum k (..., 4)."""
    n = k[..., 1:] / np.linalg.norm(k[..., 1:], axis=-1, keepdims=True)
    a = np.zeros_like(n)
    a[..., 2] = 1.0
    near_z = np.abs(n[..., 2]) > 0.9
    a[near_z] = [1.0, 0.0, 0.0]
    e1 = np.cross(a, n)
    e1 /= np.linalg.norm(e1, axis=-1, keepdims=True)
    e2 = np.cross(n, e1)
    z = np.zeros(k.shape[:-1] + (1,))
    return [np.concatenate([z, e1], -1), np.concatenate([z, e2], -1)]


def _prop(q, m, w):
    """i (qslash + m) / (q^2 - m^2 + i m w), (..., 4, 4)."""
    d = mdot(q, q) - m * m + 1j * m * w
    return 1j * (slash(q) + m * np.eye(4)) / d[..., None, None]


def _chain(row, mats, col):
    """row . M1 . M2 ... . col over the event axis."""
    x = row
    for M in mats:
        x = np.einsum("...a,...ab->...b", x, M)
    return np.einsum("...a,...a->...", x, col)


def _current(row, pre, post, col, g):
    """Vector X^nu = row . pre . (i g gamma^nu) . post . col (pre, post:
    lists of matrices)."""
    out = []
    for nu in range(4):
        gn = np.broadcast_to(1j * g * GAM[nu], row.shape[:-1] + (4, 4))
        out.append(_chain(row, pre + [gn] + post, col))
    return np.stack(out, -1)


def _vvv(e1, e2, e3, k1, k2, k3):
    """V^{mu nu rho}(k1, k2, k3) e1_mu e2_nu e3_rho of the triple-gluon vertex."""
    return (mdot(e1, e2) * mdot(k1 - k2, e3) + mdot(e2, e3) * mdot(k2 - k3, e1)
            + mdot(e3, e1) * mdot(k3 - k1, e2))


def _colour_matrix(tensors):
    flat = [t.reshape(-1) for t in tensors]
    return np.array([[np.vdot(b, a) for b in flat] for a in flat])  # CM[d, d'] = sum C_d conj(C_d')


def _sum_squared(amps, cm):
    """sum over helicities of A^T CM A*; amps: list over helicity
    configurations of (ndiag, N) complex."""
    tot = 0.0
    for A in amps:
        tot = tot + np.real(np.einsum("dn,de,en->n", A, cm, A.conj()))
    return tot


# ---- colour tensors ---------------------------------------------------------
# qq-type processes: indices (light-line row, light-line column, i_t, j_tbar, a)
def _colour_light_line():
    TT = np.einsum("bij,ajk->baik", T, T)  # (T^b T^a)_ik as [b, a, i, k]
    c1 = np.einsum("baij,bkl->ijkla", TT, T)                      # (T^b T^a)_row,col T^b_t,tb
    c2 = np.einsum("abij,bkl->ijkla", TT, T)                      # (T^a T^b)_row,col T^b
    c3 = np.einsum("bij,abkl->ijkla", T, TT)                      # T^b (T^a T^b)_t,tb
    c4 = np.einsum("bij,bakl->ijkla", T, TT)                      # T^b (T^b T^a)_t,tb
    c5 = np.einsum("bac,bij,ckl->ijkla", F, T, T)                 # f^bac T^b T^c
    return [c1, c2, c3, c4, c5]


# ---- processes -------------------------------------------------------------
def me2_gg_ttx(p, mt, g):
    """g(p0) g(p1) > t(p2) t~(p3), averaged over 4 spins and 64 colours."""
    p1, p2, p3, p4 = (p[:, i] for i in range(4))
    TT = np.einsum("aij,bjk->abik", T, T)
    cm = _colour_matrix([TT, np.transpose(TT, (1, 0, 2, 3)), np.einsum("abc,cij->abij", F, T)])
    s = mdot(p3 + p4, p3 + p4)
    amps = []
    for h3, h4 in itertools.product(range(2), range(2)):
        ub3, v4 = bar(u_spinor(p3, mt, h3)), v_spinor(p4, mt, h4)
        K = _current(ub3, [], [], v4, g)
        for e1, e2 in itertools.product(polarisations(p1), polarisations(p2)):
            s1, s2 = 1j * g * slash(e1), 1j * g * slash(e2)
            a_t = _chain(ub3, [s1, _prop(p3 - p1, mt, 0.0), s2], v4)
            a_u = _chain(ub3, [s2, _prop(p3 - p2, mt, 0.0), s1], v4)
            a_s = g * _vvv(e1, e2, -1j * K / s[:, None], p1, p2, -(p3 + p4))
            amps.append(np.stack([a_t, a_u, a_s]))
    return _sum_squared(amps, cm) / 256.0


def me2_uux_ttx(p, mt, wt, g):
    """q(p0) q~(p1) > t(p2) t~(p3), averaged over 4 spins and 9 colours."""
    p1, p2, p3, p4 = (p[:, i] for i in range(4))
    cm = _colour_matrix([np.einsum("bij,bkl->ijkl", T, T)])
    s = mdot(p1 + p2, p1 + p2)
    amps = []
    for h in itertools.product(range(2), repeat=4):
        J = _current(bar(v_spinor(p2, 0.0, h[1])), [], [], u_spinor(p1, 0.0, h[0]), g)
        K = _current(bar(u_spinor(p3, mt, h[2])), [], [], v_spinor(p4, mt, h[3]), g)
        amps.append(np.stack([-1j * mdot(J, K) / s]))
    return _sum_squared(amps, cm) / 36.0


def me2_uux_ttxg(p, mt, wt, g):
    """q(p0) q~(p1) > t(p2) t~(p3) g(p4): 5 diagrams; averaged over 4 spins
    and 9 colours.  Colour indices of the light line: (q~ row, q column)."""
    p1, p2, p3, p4, p5 = (p[:, i] for i in range(5))
    cm = _colour_matrix(_colour_light_line())
    s12, s34 = mdot(p1 + p2, p1 + p2), mdot(p3 + p4, p3 + p4)
    amps = []
    for h in itertools.product(range(2), repeat=4):
        vb2, u1 = bar(v_spinor(p2, 0.0, h[1])), u_spinor(p1, 0.0, h[0])
        ub3, v4 = bar(u_spinor(p3, mt, h[2])), v_spinor(p4, mt, h[3])
        J = _current(vb2, [], [], u1, g)
        K = _current(ub3, [], [], v4, g)
        for e5 in polarisations(p5):
            se = 1j * g * slash(e5)
            X1 = _current(vb2, [], [_prop(p1 - p5, 0.0, 0.0), se], u1, g)
            X2 = _current(vb2, [se, _prop(p1 - p3 - p4, 0.0, 0.0)], [], u1, g)
            Y3 = _current(ub3, [se, _prop(p3 + p5, mt, wt)], [], v4, g)
            Y4 = _current(ub3, [], [_prop(-p4 - p5, mt, wt), se], v4, g)
            a1 = -1j * mdot(X1, K) / s34
            a2 = -1j * mdot(X2, K) / s34
            a3 = -1j * mdot(J, Y3) / s12
            a4 = -1j * mdot(J, Y4) / s12
            a5 = g * _vvv(-1j * J / s12[:, None], e5, -1j * K / s34[:, None], p1 + p2, -p5, -(p3 + p4))
            amps.append(np.stack([a1, a2, a3, a4, a5]))
    return _sum_squared(amps, cm) / 36.0


def me2_ug_ttxu(p, mt, wt, g):
    """q(p0) g(p1) > t(p2) t~(p3) q(p4): 5 diagrams; averaged over 4 spins
    and 24 colours.  Light line (outgoing q row, incoming q column)."""
    p1, p2, p3, p4, p5 = (p[:, i] for i in range(5))
    cm = _colour_matrix(_colour_light_line())
    s34, t15 = mdot(p3 + p4, p3 + p4), mdot(p1 - p5, p1 - p5)
    amps = []
    for h in itertools.product(range(2), repeat=4):
        ub5, u1 = bar(u_spinor(p5, 0.0, h[3])), u_spinor(p1, 0.0, h[0])
        ub3, v4 = bar(u_spinor(p3, mt, h[1])), v_spinor(p4, mt, h[2])
        J = _current(ub5, [], [], u1, g)
        K = _current(ub3, [], [], v4, g)
        for e2 in polarisations(p2):
            se = 1j * g * slash(e2)
            X1 = _current(ub5, [], [_prop(p1 + p2, 0.0, 0.0), se], u1, g)
            X2 = _current(ub5, [se, _prop(p1 - p3 - p4, 0.0, 0.0)], [], u1, g)
            Y3 = _current(ub3, [se, _prop(p3 - p2, mt, wt)], [], v4, g)
            Y4 = _current(ub3, [], [_prop(p2 - p4, mt, wt), se], v4, g)
            a1 = -1j * mdot(X1, K) / s34
            a2 = -1j * mdot(X2, K) / s34
            a3 = -1j * mdot(J, Y3) / t15
            a4 = -1j * mdot(J, Y4) / t15
            a5 = g * _vvv(-1j * J / t15[:, None], e2, -1j * K / s34[:, None], p1 - p5, p2, -(p3 + p4))
            amps.append(np.stack([a1, a2, a3, a4, a5]))
    return _sum_squared(amps, cm) / 96.0


def me2_uxg_ttxux(p, mt, wt, g):
    """q~(p0) g(p1) > t(p2) t~(p3) q~(p4): 5 diagrams; averaged over 4 spins
    and 24 colours.  Light line (incoming q~ row, outgoing q~ column)."""
    p1, p2, p3, p4, p5 = (p[:, i] for i in range(5))
    c1, c2, c3, c4, c5 = _colour_light_line()
    # the gluon sits next to the incoming q~ (row) in the first diagram here
    cm = _colour_matrix([c2, c1, c3, c4, c5])
    s34, t15 = mdot(p3 + p4, p3 + p4), mdot(p1 - p5, p1 - p5)
    amps = []
    for h in itertools.product(range(2), repeat=4):
        vb1, v5 = bar(v_spinor(p1, 0.0, h[0])), v_spinor(p5, 0.0, h[3])
        ub3, v4 = bar(u_spinor(p3, mt, h[1])), v_spinor(p4, mt, h[2])
        J = _current(vb1, [], [], v5, g)
        K = _current(ub3, [], [], v4, g)
        for e2 in polarisations(p2):
            se = 1j * g * slash(e2)
            X1 = _current(vb1, [se, _prop(-p5 - p3 - p4, 0.0, 0.0)], [], v5, g)
            X2 = _current(vb1, [], [_prop(p2 - p5, 0.0, 0.0), se], v5, g)
            Y3 = _current(ub3, [se, _prop(p3 - p2, mt, wt)], [], v4, g)
            Y4 = _current(ub3, [], [_prop(p2 - p4, mt, wt), se], v4, g)
            a1 = -1j * mdot(X1, K) / s34
            a2 = -1j * mdot(X2, K) / s34
            a3 = -1j * mdot(J, Y3) / t15
            a4 = -1j * mdot(J, Y4) / t15
            a5 = g * _vvv(-1j * J / t15[:, None], e2, -1j * K / s34[:, None], p1 - p5, p2, -(p3 + p4))
            amps.append(np.stack([a1, a2, a3, a4, a5]))
    return _sum_squared(amps, cm) / 96.0
