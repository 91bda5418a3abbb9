"""Model parameters (madflow parameters.py): couplings as functions of
alpha_s, frozen or per event."""
import math

import torch

from .config import DTYPE, DTYPECOMPLEX


def _alphas_to_gs(alpha_s):
    """g_s = 2 sqrt(pi alpha_s) (parameters.py:13-15)."""
    a = torch.as_tensor(alpha_s, dtype=DTYPE)
    return (2.0 * torch.sqrt(math.pi * a)).to(DTYPECOMPLEX)


class Model:
    """Constants of the model plus the couplings that depend on g_s
    (parameters.py:18-98)."""

    def __init__(self, constants, functions):
        self._tuple_constants = constants
        self._tuple_functions = functions
        self._constants = list(constants)
        self._to_evaluate = list(functions)
        self._frozen = []

    @property
    def frozen(self):
        return bool(self._frozen)

    def freeze_alpha_s(self, alpha_s):
        if self.frozen:
            raise ValueError("The model is already frozen")
        # float_me([alpha_s]): the reference holds the value through float32
        a32 = float(torch.tensor([alpha_s], dtype=torch.float32)[0])
        self._frozen = self._evaluate(torch.tensor([a32], dtype=DTYPE))

    def unfreeze(self):
        self._frozen = []

    def _evaluate(self, alpha_s):
        gs = _alphas_to_gs(alpha_s)
        results = [fun(gs) for fun in self._to_evaluate]
        if not results:
            return self._constants
        if not self._constants:
            return results
        return self._constants + results

    def get_masses(self):
        return [v for k, v in self._tuple_constants._asdict().items() if k.startswith("mdl_M")]

    def parse_parameter(self, name):
        if name == "ZERO":
            return 0.0
        if hasattr(self._tuple_constants, name):
            return getattr(self._tuple_constants, name)
        if hasattr(self._tuple_functions, name):
            return getattr(self._tuple_functions, name)
        raise AttributeError(f"The model class does not contain parameter {name}")

    def evaluate(self, alpha_s=None):
        if self.frozen:
            return self._frozen
        return self._evaluate(alpha_s)


def sm_top_model(mdl_MT=173.0, mdl_WT=1.4915000200271606):
    """The SM parameters a g g > t t~ + gluons module needs: constants
    (mdl_MT, mdl_WT) and GC_10 = -g_s, GC_11 = i g_s, GC_12 = i g_s^2."""
    import collections

    Const = collections.namedtuple("constants", ["mdl_MT", "mdl_WT"])
    Func = collections.namedtuple("functions", ["GC_10", "GC_11", "GC_12"])
    f10 = lambda gs: -gs
    f11 = lambda gs: 1j * gs
    f12 = lambda gs: 1j * gs * gs
    return Model(Const(mdl_MT, mdl_WT), Func(f10, f11, f12))
