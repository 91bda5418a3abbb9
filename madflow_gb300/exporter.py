"""Process output in the layout of madflow's PyOut exporter.

madflow has MG5_aMC run ``generate <process>`` and ``output pyout <folder>``
(scripts/madflow_exec.py:81-112).  The PyOut plugin
(madgraph_plugin/PyOut_exporter.py:125-285) fills the template
madgraph_plugin/template_files/matrix_method_python.inc once per subprocess
and writes ``matrix_1_<proc>.py`` plus ``Cards/param_card.dat``; madflow then
imports every ``matrix_*.py`` of the folder and takes from each module the
class ``Matrix_1_<proc>`` and ``get_model_param(model, param_card_path)``
(scripts/madflow_exec.py:115-137).

``export`` writes the same folder for the processes this library evaluates,
without MG5_aMC:

- one ``matrix_1_<proc>.py`` per subprocess.  Its class keeps the generated
  module's attributes (nexternal, ndiags, ncomb, helicities, denominator,
  initial_states, mirror_initial_states) as literals and its
  ``smatrix(all_ps, <masses/widths>, <couplings>)`` call, which the CUDA
  kernels evaluate.  ``get_model_param`` reads the param card and returns a
  ``parameters.Model`` with the constants and the g_s-dependent couplings the
  call takes, in the exporter's order (sorted masses/widths, then sorted
  couplings, PyOut_exporter.py:244);
- ``Cards/param_card.dat`` (SLHA) with the SM values the processes use;
- for g g > t t~ + gluons, ``csrc/ttng<k>.cuh``: the generated CUDA program
  of the process (colour numerators, helicity table, the helicity-recycling
  recursion), the same source the library's kernels are compiled from.

``import_matrices`` loads such a folder the way madflow does.
"""
import importlib.util
import os
import re
import struct
import types
from pathlib import Path

from . import codegen

# subprocess name -> (base class in madflow_gb300.matrix, parameters of smatrix, description)
_TTNG_PARAMS = {2: ["mdl_MT", "mdl_WT", "GC_10", "GC_11"]}
_SUBPROCESSES = {}
for _k in (2, 3, 4, 5):
    _SUBPROCESSES[codegen.process_name(_k)] = (
        f"Matrix_1_{codegen.process_name(_k)}",
        _TTNG_PARAMS.get(_k, ["mdl_MT", "mdl_WT", "GC_10", "GC_11", "GC_12"]),
        "g g > t t~" + " g" * (_k - 2),
    )
_SUBPROCESSES.update({
    "uux_ttx": ("Matrix_1_uux_ttx", ["mdl_MT", "mdl_WT", "GC_11"], "q q~ > t t~ (q = u c d s)"),
    "uux_ttxg": ("Matrix_1_uux_ttxg", ["mdl_MT", "mdl_WT", "GC_10", "GC_11"], "q q~ > t t~ g (q = u c d s)"),
    "ug_ttxu": ("Matrix_1_ug_ttxu", ["mdl_MT", "mdl_WT", "GC_10", "GC_11"], "q g > t t~ q (q = u c d s)"),
    "uxg_ttxux": ("Matrix_1_uxg_ttxux", ["mdl_MT", "mdl_WT", "GC_10", "GC_11"], "q~ g > t t~ q~ (q = u c d s)"),
})

# the SM couplings of these processes as functions of G = g_s (MG5 SM UFO:
# GC_10 = -G, GC_11 = i G, GC_12 = i G^2)
_COUPLING_EXPR = {"GC_10": "-G", "GC_11": "1j * G", "GC_12": "1j * G * G"}

_QUARKS = ("u", "c", "d", "s")


def subprocesses(process):
    """The subprocess modules a process string expands to, in MG5_aMC's
    syntax: ``g g > t t~`` + up to three `` g``; ``q q~ > t t~ [g]``,
    ``q g > t t~ q``, ``q~ g > t t~ q~`` for q in u c d s (one module for the
    four flavours, as MadGraph groups them); ``p p > t t~``,
    ``p p > t t~ g`` and ``p p > t t~ j`` (p = j = g u c d s and their
    antiquarks).  Anything else raises ValueError."""
    toks = process.split()
    if ">" not in toks:
        raise ValueError(f"not a process string: {process!r}")
    i = toks.index(">")
    ini, fin = toks[:i], toks[i + 1:]
    if len(ini) != 2 or fin[:2] != ["t", "t~"]:
        raise ValueError(f"unsupported process {process!r}: initial state of two partons and t t~ first")
    extra = fin[2:]
    if ini == ["p", "p"]:
        if extra == []:
            return ["gg_ttx", "uux_ttx"]
        if extra == ["g"]:
            return ["gg_ttxg", "uux_ttxg"]
        if extra == ["j"]:
            return ["gg_ttxg", "uux_ttxg", "ug_ttxu", "uxg_ttxux"]
        raise ValueError(f"unsupported process {process!r}: p p > t t~ with nothing, g or j after it")
    if ini == ["g", "g"] and all(t == "g" for t in extra) and len(extra) <= 3:
        return [codegen.process_name(2 + len(extra))]
    a, b = ini
    if a in _QUARKS and b == a + "~" and extra in ([], ["g"]):
        return ["uux_ttx" if not extra else "uux_ttxg"]
    if a in _QUARKS and b == "g" and extra == [a]:
        return ["ug_ttxu"]
    if a.endswith("~") and a[:-1] in _QUARKS and b == "g" and extra == [a]:
        return ["uxg_ttxux"]
    raise ValueError(f"unsupported process {process!r}")


def _f32(x):
    """A Python float held through float32, as madflow's float_me does with
    the param-card values."""
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def read_param_card(path):
    """The blocks of an SLHA param card: {block: {pdg or index: value}};
    DECAY lines go to the block "DECAY"."""
    blocks = {}
    current = None
    for line in Path(path).read_text().splitlines():
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        toks = line.split()
        head = toks[0].upper()
        if head == "BLOCK":
            current = blocks.setdefault(toks[1].upper(), {})
        elif head == "DECAY":
            blocks.setdefault("DECAY", {})[int(toks[1])] = float(toks[2])
            current = None
        elif current is not None and len(toks) >= 2:
            current[int(toks[0])] = float(toks[1])
    return blocks


def _param_card(mt, wt, alpha_s):
    return "\n".join([
        "######################################################################",
        "## PARAM_CARD: the SM parameters of the exported processes        ####",
        "######################################################################",
        "BLOCK MASS #",
        f"      6 {mt:.6e} # MT",
        "BLOCK SMINPUTS #",
        f"      3 {alpha_s:.6e} # aS",
        f"DECAY   6 {wt:.6e} # WT",
        "",
    ])


def _module_source(name, process):
    base, params, desc = _SUBPROCESSES[name]
    consts = [p for p in params if p.startswith("mdl_")]
    coups = [p for p in params if p.startswith("GC_")]
    if name in {codegen.process_name(k) for k in (2, 3, 4, 5)}:
        k = len(name) - len("gg_ttx") + 2
        nexternal, ncomb = k + 2, 2 ** (k + 2)
        ndiags = codegen.diagram_count(k)
        hels = codegen.helicities(k)
        den = float(codegen.denominator(k))
        ini, mirror = [(21, 21)], False
        num, cden = codegen.colour_matrix(k)
        colour = f"    colour_matrix = np.array({num!r}, dtype=np.float64) / {float(cden)!r}\n"
    else:
        from . import matrix as _m

        cls = getattr(_m, base)
        nexternal, ncomb, ndiags = int(cls.nexternal), int(cls.ncomb), int(cls.ndiags)
        hels = cls(precision=0).helicities.tolist()  # host-side table, no device work
        den = float(cls.denominator)
        ini, mirror = list(cls.initial_states), bool(cls.mirror_initial_states)
        colour = ""
    hel_lines = ",\n        ".join("[" + ", ".join(f"{int(v)}" for v in h) + "]" for h in hels)
    func_lines = "\n".join(f"    {c} = lambda G: {_COUPLING_EXPR[c]}" for c in coups)
    sig = ", ".join(params)
    return f'''"""Process {desc}, exported from the process string {process!r} by
madflow_gb300.exporter in the layout of madflow's PyOut output.  The matrix
element runs in the CUDA kernels of madflow_gb300."""
import collections

import numpy as np

from madflow_gb300 import matrix as _matrix
from madflow_gb300.exporter import _f32, read_param_card, import_ufo  # noqa: F401
from madflow_gb300.parameters import Model

ModelParamTupleConst = collections.namedtuple("constants", {consts!r})
ModelParamTupleFunc = collections.namedtuple("functions", {coups!r})


def get_model_param(model, param_card_path):
    """The model parameters smatrix takes ({sig}), read from the param card;
    the couplings as functions of G = g_s.  ``model`` (MG5's UFO model in
    madflow) is not needed."""
    card = read_param_card(param_card_path)
    mdl_MT = card["MASS"][6]
    mdl_WT = card["DECAY"][6]
{func_lines}
    constants = ModelParamTupleConst({", ".join(f"_f32({c})" for c in consts)})
    functions = ModelParamTupleFunc({", ".join(coups)})
    return Model(constants, functions)


class Matrix_1_{name}(_matrix.{base}):
    """{desc}: smatrix(all_ps, {sig})."""

    process_string = "1_{name}"
    nexternal = {float(nexternal)!r}
    ndiags = {float(ndiags)!r}
    ncomb = {float(ncomb)!r}
    initial_states = {ini!r}
    mirror_initial_states = {mirror!r}
    helicities = [
        {hel_lines}]
    denominator = {den!r}
{colour}
    def __str__(self):
        return "1_{name}"
'''


def export(process, output_folder, mdl_MT=173.0, mdl_WT=1.4915, alpha_s=0.118):
    """Write the PyOut-style output of ``process`` into ``output_folder``
    (created if needed).  Returns the paths of the written matrix modules."""
    out = Path(output_folder)
    (out / "Cards").mkdir(parents=True, exist_ok=True)
    (out / "Cards" / "param_card.dat").write_text(_param_card(mdl_MT, mdl_WT, alpha_s))
    paths = []
    for name in subprocesses(process):
        path = out / f"matrix_1_{name}.py"
        path.write_text(_module_source(name, process))
        paths.append(path)
        if name.startswith("gg_ttx"):
            k = len(name) - len("gg_ttx") + 2
            (out / "csrc").mkdir(exist_ok=True)
            (out / "csrc" / f"ttng{k}.cuh").write_text(codegen.emit_process_header(k))
    (out / "proc_card.dat").write_text(f"generate {process}\noutput pyout {out.name}\n")
    return paths


def _import_ufo_model(path):
    """Stand-in for MG5's ``models.import_ufo.import_model``: madflow's loader
    calls it before ``get_model_param``, which here needs no UFO model."""
    return None


import_ufo = types.SimpleNamespace(import_model=_import_ufo_model)


def import_matrices(output_folder):
    """Load every ``matrix_*.py`` of an exported folder as madflow does
    (scripts/madflow_exec.py:115-137): returns (matrices, models), one
    instance of each module's Matrix class and its get_model_param result."""
    out = Path(output_folder)
    re_name = re.compile(r"\w{3,}")
    matrices, models = [], []
    for path in sorted(out.glob("matrix_*.py")):
        mod_name = re_name.findall(path.name)[0]
        spec = importlib.util.spec_from_file_location(mod_name, path)
        module = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(module)
        matrices.append(getattr(module, mod_name.capitalize())())
        model = module.import_ufo.import_model(os.fspath(out))
        models.append(module.get_model_param(model, os.fspath(out / "Cards" / "param_card.dat")))
    return matrices, models
