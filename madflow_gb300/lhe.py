"""Event output: device-side unweighting and a Les Houches Event File writer
fed from device buffers.

madflow writes every weighted event of every iteration from inside the
integrand through ``tf.py_function`` (``lhe_writer.py:139-196``, called from
``madflow_exec.py:460-464``) and unweights the file afterwards with MG5's
``lhe_parser`` (``lhe_writer.py:316-358``).  Here events are produced on the
device for a frozen grid (``mf_vegas_events``: weights and lab-frame
momenta), unweighted on the device (``mf_unweight``, hit or miss against a
maximum weight), and only the kept events are copied to the host and
written, in LHEF 3.0 (Alwall et al., Comput. Phys. Commun. 176 (2007) 300).

Differences from madflow's writer, on purpose: incoming partons carry their
PDG code (madflow writes 2212 for them and has no code beyond four
particles, ``lhe_writer.py:162-173``), outgoing particles name the two
incoming ones as mothers, and each event carries its scale and alpha_s;
like madflow, colour lines are left at 0.
"""
import ctypes
import gzip
import math

import numpy as np
import torch

from . import _lib
from .config import device, stream_ptr


def truncated_wmax(w, trunc=0.0):
    """Maximum weight for unweighting: max |w|, or with trunc > 0 the
    smallest threshold t such that the weight above it, sum max(|w| - t, 0),
    is at most trunc * sum |w| (overweight events then carry that excess)."""
    a = w.abs().double()
    if a.numel() == 0:
        return 0.0
    if trunc <= 0.0:
        return float(a.max())
    s, _ = torch.sort(a, descending=True)
    total = float(s.sum())
    csum = torch.cumsum(s, 0)
    k = torch.arange(1, s.numel() + 1, device=s.device, dtype=s.dtype)
    # excess if the threshold is s[i]: sum_{j<=i} s[j] - (i+1) s[i]
    excess = csum - k * s
    ok = torch.nonzero(excess <= trunc * total).flatten()
    return float(s[int(ok.max())])


def unweight(w, w_max, seed=11, stream_id=0):
    """Hit-or-miss unweighting of device weights w against w_max (kernel
    ``mf_unweight``).  Returns (indices of kept events, their relative
    weights max(1, |w|/w_max))."""
    w = w.contiguous().double()
    n = w.numel()
    keep = torch.empty(n, dtype=torch.uint8, device=w.device)
    _lib.call("mf_unweight", w.data_ptr(), n, float(w_max), int(seed), int(stream_id), keep.data_ptr(), stream_ptr())
    idx = torch.nonzero(keep).flatten()
    rel = torch.clamp(w[idx].abs() / w_max, min=1.0)
    return idx, rel


class LheWriter:
    """LHEF 3.0 writer (gzip when the path ends in .gz)."""

    def __init__(self, path, beams=(2212, 2212), ebeam=(6500.0, 6500.0), process_id=1, comment=""):
        self.path = str(path)
        self.beams, self.ebeam, self.process_id = beams, ebeam, process_id
        opener = gzip.open if self.path.endswith(".gz") else open
        self._f = opener(self.path, "wt")
        self.n_events = 0
        self._f.write('<LesHouchesEvents version="3.0">\n<header>\n')
        if comment:
            self._f.write(f"<!-- {comment} -->\n")
        self._f.write("</header>\n")

    def write_init(self, xsec, xerr, xmax):
        b1, b2 = self.beams
        e1, e2 = self.ebeam
        # IDWTUP = 3: unweighted events, weights sigma / N (signed)
        self._f.write("<init>\n")
        self._f.write(f" {b1} {b2} {e1:.8e} {e2:.8e} 0 0 0 0 3 1\n")
        self._f.write(f" {xsec:.8e} {xerr:.8e} {xmax:.8e} {self.process_id}\n")
        self._f.write("</init>\n")

    def write_events(self, momenta, weights, pids, scale, aqcd, aqed=-1.0):
        """momenta (M, n, 4) as (E, px, py, pz); weights (M,); pids (n,),
        the first two incoming; scale and aqcd one value or one per event."""
        p = np.asarray(momenta, dtype=np.float64)
        w = np.asarray(weights, dtype=np.float64)
        m, n, _ = p.shape
        scales = np.broadcast_to(np.asarray(scale, dtype=np.float64), (m,))
        aqcds = np.broadcast_to(np.asarray(aqcd, dtype=np.float64), (m,))
        m2 = p[..., 0] ** 2 - (p[..., 1] ** 2 + p[..., 2] ** 2 + p[..., 3] ** 2)
        mass = np.sqrt(np.maximum(m2, 0.0))
        lines = []
        for e in range(m):
            lines.append("<event>\n")
            lines.append(f" {n} {self.process_id} {w[e]:+.10e} {scales[e]:.10e} {aqed:.10e} {aqcds[e]:.10e}\n")
            for i in range(n):
                st, m1, m2_ = (-1, 0, 0) if i < 2 else (1, 1, 2)
                pe = p[e, i]
                lines.append(f" {int(pids[i]):8d} {st:2d} {m1:4d} {m2_:4d} {0:4d} {0:4d} "
                             f"{pe[1]:+.10e} {pe[2]:+.10e} {pe[3]:+.10e} {pe[0]:.10e} {mass[e, i]:.10e} "
                             f"0.0000e+00 9.0000e+00\n")
            lines.append("</event>\n")
        self._f.write("".join(lines))
        self.n_events += m

    def close(self):
        if self._f is not None:
            self._f.write("</LesHouchesEvents>\n")
            self._f.close()
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def dynamic_scale(momenta, alpha_mz, mz=91.1876):
    """(mu, alpha_s(mu^2)) per event of the dynamical scale for momenta
    (M, n, 4): mu = sum over the outgoing particles of m_T / 2, m_T^2 = p.p +
    p_T^2 (scripts/madflow_exec.py:428-431), alpha_s at one loop with five
    flavours from alpha_s(M_Z^2) = alpha_mz."""
    q = np.asarray(momenta, dtype=np.float64)[:, 2:, :]
    m2 = q[..., 0] ** 2 - q[..., 1] ** 2 - q[..., 2] ** 2 - q[..., 3] ** 2
    pt = np.sqrt(q[..., 1] ** 2 + q[..., 2] ** 2)
    mu = np.sqrt(m2 + pt**2).sum(-1) / 2.0
    b0 = 23.0 / (12.0 * math.pi)
    return mu, alpha_mz / (1.0 + alpha_mz * b0 * np.log(mu * mu / (mz * mz)))


def generate_events(integrand, vegas, n_events, path, batch=1_000_000, trunc=1e-3, seed=11, max_batches=1000):
    """Unweighted events of a FusedIntegrand on the (frozen) grid of a
    VegasFlow into an LHE file.  The first batch fixes the maximum weight
    (truncated at ``trunc`` of the cross section); every batch is unweighted
    on the device against it; the cross section and its error in the
    <init> block are the mean and error of all generated weights.

    Returns a dict of statistics."""
    ndim, nb = vegas.n_dim, vegas.nbins
    npart = int(integrand.matrix.nexternal)
    f = torch.empty(batch, dtype=torch.float64, device=device())
    ps = torch.empty((batch, npart, 4), dtype=torch.float64, device=device())
    kept_p, kept_w = [], []
    s1 = s2 = 0.0
    n_gen = 0
    w_max = None
    b = 0
    for b in range(int(max_batches)):
        _lib.call("mf_vegas_events", integrand.matrix.handle, ctypes.byref(integrand._cs), vegas.grid.data_ptr(), nb,
                  int(vegas.seed) + 7919, int(vegas.stream_id), b, batch, f.data_ptr(), ps.data_ptr(), stream_ptr())
        w = f / batch  # weights of this batch's estimate; the mean over batches is the cross section
        s1 += float(w.sum())
        s2 += float((f * f).sum())
        n_gen += batch
        if w_max is None:
            w_max = truncated_wmax(w, trunc)
        idx, rel = unweight(w, w_max, seed=seed, stream_id=b)
        kept_p.append(ps[idx].cpu().numpy())
        kept_w.append(rel.cpu().numpy())
        if sum(len(k) for k in kept_w) >= n_events:
            break
    nb_batches = b + 1
    xsec = s1 / nb_batches
    var = (s2 / n_gen - xsec * xsec) / (n_gen - 1)
    xerr = math.sqrt(max(var, 0.0))
    p = np.concatenate(kept_p)[:n_events]
    rel = np.concatenate(kept_w)[:n_events]
    n_keep = len(rel)
    weights = rel * xsec / rel.sum() if n_keep else rel
    cfg = integrand.cfg
    pids = [21, 21, 6, -6] + [21] * (npart - 4)
    half = cfg["sqrts"] / 2.0
    if cfg["q2"] < 0:
        # the dynamical scale of the integrand: mu = sum of the outgoing m_T / 2,
        # alpha_s(mu^2) at one loop from alpha_s(M_Z^2) (mf_integrand_config)
        scale, aqcd = dynamic_scale(p, cfg["alpha_s"])
    else:
        scale, aqcd = math.sqrt(cfg["q2"]), cfg["alpha_s"]
    with LheWriter(path, ebeam=(half, half), comment=f"madflow_gb300 {integrand.matrix}") as lhe:
        lhe.write_init(xsec, xerr, float(weights.max()) if n_keep else 0.0)
        lhe.write_events(p, weights, pids, scale, aqcd)
    return {"xsec_pb": xsec, "xerr_pb": xerr, "kept": n_keep, "generated": n_gen,
            "efficiency": n_keep / n_gen if n_gen else 0.0, "w_max": w_max, "batches": nb_batches}
