"""Phase-space generation on the GPU, with madflow's interface
(python_package/madflow/phasespace.py).

Momenta are (E, px, py, pz); a full set of momenta has shape
(n_events, n_particles, 4).  The kernels work on structure-of-arrays copies
made once at this boundary.
"""
import torch

from . import _lib
from .config import DTYPE, device, stream_ptr, to_device

NEWTON_BATCH = _lib.MF_NEWTON_BATCH
NEWTON_PER_EVENT = _lib.MF_NEWTON_PER_EVENT


def _masses_arg(masses, n):
    if masses is None:
        return None
    m = [float(v) for v in masses]
    if len(m) != n:
        raise ValueError(f"{len(m)} masses given for {n} particles")
    if sum(m) == 0.0:
        return None
    return _lib.dbl_array(m)


def rambo(xrand, n_particles, sqrts, masses=None, check_physical=False, newton_rule=NEWTON_BATCH):
    """RAMBO (phasespace.py:145-212): xrand (N, 4n) -> (momenta (N, n, 4), weight (N,)).

    ``sqrts`` is a float or a per-event tensor.  With masses, the momenta are
    rescaled by Newton iterations stopping, like the reference, for the whole
    batch as soon as one event converges (``newton_rule=NEWTON_PER_EVENT``
    lets every event converge on its own).
    """
    if check_physical and masses is not None and isinstance(sqrts, float) and sum(masses) > sqrts:
        raise ValueError(f"Not enough energy ({sqrts}) to generate particles of mass: {masses}")
    x = to_device(xrand)
    N = x.shape[0]
    if x.shape[1] < 4 * n_particles:
        raise ValueError(f"rambo needs {4 * n_particles} random numbers per event, got {x.shape[1]}")
    xs = x[:, : 4 * n_particles].T.contiguous()
    if isinstance(sqrts, (int, float)):
        sq = torch.full((1,), float(sqrts), dtype=DTYPE, device=device())
        sstride = 0
    else:
        sq = to_device(sqrts).reshape(-1)
        sstride = 1
    p = torch.empty((n_particles, 4, N), dtype=DTYPE, device=device())
    w = torch.empty(N, dtype=DTYPE, device=device())
    _lib.call("mf_rambo", xs.data_ptr(), N, n_particles, sq.data_ptr(), sstride, _masses_arg(masses, n_particles),
              newton_rule, p.data_ptr(), w.data_ptr(), stream_ptr())
    return p.permute(2, 0, 1).contiguous(), w


def ramboflow(xrand, nparticles, com_sqrts, masses=None, newton_rule=NEWTON_BATCH):
    """ramboflow (phasespace.py:257-319): x1, x2 from the first two numbers,
    RAMBO for the outgoing particles, flux factor in pb.

    Returns (momenta (N, nparticles, 4), weight, x1, x2)."""
    if nparticles < 4:
        raise NotImplementedError("the 2 -> 1 on-shell mapping (phasespace.py:236-254) is not on the GPU path")
    x = to_device(xrand)
    N = x.shape[0]
    nd = 4 * (nparticles - 2) + 2
    xs = x[:, :nd].T.contiguous()
    p = torch.empty((nparticles, 4, N), dtype=DTYPE, device=device())
    w, x1, x2 = (torch.empty(N, dtype=DTYPE, device=device()) for _ in range(3))
    _lib.call("mf_ramboflow", xs.data_ptr(), N, nparticles, float(com_sqrts), _masses_arg(masses, nparticles - 2),
              newton_rule, p.data_ptr(), w.data_ptr(), x1.data_ptr(), x2.data_ptr(), stream_ptr())
    return p.permute(2, 0, 1).contiguous(), w, x1, x2


def boost_to_lab(p_com, x1, x2):
    """_boost_to_lab (phasespace.py:322-356)."""
    p = to_device(p_com)
    N, n = p.shape[0], p.shape[1]
    ps = p.permute(1, 2, 0).contiguous()
    _lib.call("mf_boost_to_lab", ps.data_ptr(), N, n, to_device(x1).data_ptr(), to_device(x2).data_ptr(), stream_ptr())
    return ps.permute(2, 0, 1).contiguous()


def _fourdot(f1, f2):
    return f1[..., 0] * f2[..., 0] - (f1[..., 1:] * f2[..., 1:]).sum(-1)


def _invariant_mass(fm):
    return _fourdot(fm, fm)


class PhaseSpaceGenerator:
    """Phase-space generator with cuts (phasespace.py:359-520).

    Cuts registered with ``register_cut(variable, particle, min_val, max_val)``
    select events exactly as the reference (strict inequalities, thresholds
    held as float_me values); passing events are compacted and their indices
    returned.  ``variable`` is one of the static methods pt, mt, mt2, eta.
    """

    def __init__(self, nparticles, com_sqrts, masses=None, com_output=True, algorithm="ramboflow"):
        if masses is None:
            masses = [0.0] * (nparticles - 2)
        if len(masses) != (nparticles - 2):
            raise ValueError(
                "Missmatch in PhaseSpaceGenerator between particles and masses"
                f" {len(masses)} given for {nparticles - 2} outgoing particles"
            )
        if algorithm != "ramboflow":
            raise ValueError(f"PS algorithm {algorithm} not understood")
        # float_me(com_sqrts): the reference holds sqrt(s) through float32
        self._sqrts = float(torch.tensor(float(com_sqrts), dtype=torch.float32))
        self._masses = list(masses)
        self._nparticles = nparticles
        self._cuts = []
        self._cuts_info = []
        self._cut_specs = []
        self._com_output = com_output

    def clear_cuts(self):
        self._cuts = []
        self._cuts_info = []
        self._cut_specs = []

    def cut_table(self):
        """The registered cuts as (variable, particle, min_val, max_val), the
        form FusedIntegrand(cuts=...) takes."""
        return list(self._cut_specs)

    @staticmethod
    def mt2(ps_point):
        return _invariant_mass(ps_point) + PhaseSpaceGenerator.pt(ps_point) ** 2

    @staticmethod
    def mt(ps_point):
        return torch.sqrt(PhaseSpaceGenerator.mt2(ps_point))

    @staticmethod
    def pt(ps_point):
        return torch.sqrt(ps_point[..., 1] ** 2 + ps_point[..., 2] ** 2)

    @staticmethod
    def eta(ps_point):
        pabs = torch.sqrt((ps_point[..., 1:] ** 2).sum(-1))
        return 0.5 * torch.log((pabs + ps_point[..., 3]) / (pabs - ps_point[..., 3]))

    def register_cut(self, variable, particle=None, min_val=None, max_val=None):
        fun = getattr(self, variable, None)
        if fun is None or variable not in ("pt", "mt", "mt2", "eta"):
            raise ValueError(f"{variable} is not implemented")
        if particle is not None and particle >= self._nparticles:
            raise ValueError(f"Cannot apply cuts to particle {particle}, python idx starts at 0!")
        f32 = lambda v: None if v is None else float(torch.tensor(v, dtype=torch.float32))

        lo, hi = f32(min_val), f32(max_val)

        def cut_function(ps):
            if particle is not None:
                ps = ps[:, particle, :]
            val = fun(ps)
            ok = torch.ones_like(val, dtype=torch.bool)
            if lo is not None:
                ok &= val > lo
            if hi is not None:
                ok &= val < hi
            return ok

        self._cuts.append(cut_function)
        self._cuts_info.append(f"{min_val} < {variable}({particle}) < {max_val}")
        self._cut_specs.append((variable, particle, min_val, max_val))

    def __call__(self, xrand):
        ps, wgt, x1, x2 = ramboflow(xrand, self._nparticles, self._sqrts, self._masses)
        if self._cuts:
            passing = torch.stack([c(ps) for c in self._cuts]).all(dim=0)
            idx = torch.nonzero(passing).to(torch.int32)
            ps, wgt, x1, x2 = ps[passing], wgt[passing], x1[passing], x2[passing]
        else:
            idx = torch.tensor(1, dtype=torch.int32)
        if not self._com_output:
            ps = boost_to_lab(ps, x1, x2)
        return ps, wgt, x1, x2, idx
