"""The PyOut-style process output (madflow_gb300.exporter): the folder
madflow's driver loads (scripts/madflow_exec.py:115-137), the generated
module's attributes (template_files/matrix_method_python.inc:56-66), the
param card and model parameters, and on the GPU the exported modules'
smatrix against the library classes."""
import os

import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, ROOT, WT
from madflow_gb300 import codegen
from madflow_gb300.exporter import export, import_matrices, read_param_card, subprocesses
from madflow_gb300.parameters import sm_top_model
from madflow_gb300.utilities import generate_initial_states


def test_subprocesses():
    assert subprocesses("g g > t t~") == ["gg_ttx"]
    assert subprocesses("g g > t t~ g g g") == ["gg_ttxggg"]
    assert subprocesses("p p > t t~") == ["gg_ttx", "uux_ttx"]
    assert subprocesses("p p > t t~ j") == ["gg_ttxg", "uux_ttxg", "ug_ttxu", "uxg_ttxux"]
    assert subprocesses("d d~ > t t~ g") == ["uux_ttxg"]
    assert subprocesses("c g > t t~ c") == ["ug_ttxu"]
    assert subprocesses("s~ g > t t~ s~") == ["uxg_ttxux"]
    for bad in ("g g > t t~ g g g g", "e+ e- > t t~", "p p > t t~ j j", "g g t t~", "u d~ > t t~"):
        with pytest.raises(ValueError):
            subprocesses(bad)


def _load(path):
    import importlib.util

    spec = importlib.util.spec_from_file_location(path.stem, path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_export_ttng_module(tmp_path, k):
    proc = "g g > t t~" + " g" * (k - 2)
    (path,) = export(proc, tmp_path)
    name = codegen.process_name(k)
    assert path.name == f"matrix_1_{name}.py"
    mod = _load(path)
    cls = getattr(mod, f"Matrix_1_{name}")
    assert cls.nexternal == k + 2 and cls.ncomb == 2 ** (k + 2)
    assert cls.ndiags == codegen.KNOWN_DIAGRAMS[k]
    assert cls.denominator == 256 * np.prod(range(1, k - 1))
    assert cls.helicities == codegen.helicities(k)
    assert cls.initial_states == [(21, 21)] and cls.mirror_initial_states is False
    num, den = codegen.colour_matrix(k)
    np.testing.assert_array_equal(cls.colour_matrix, np.array(num) / den)
    if k == 2:  # madflow's gg > tt~ module (tests/mockup_debug_me.py:506-507)
        np.testing.assert_allclose(cls.colour_matrix, np.array([[16, -2], [-2, 16]]) / 3, rtol=1e-15)
    # the exported CUDA program is the one the library is compiled from
    hdr = (tmp_path / "csrc" / f"ttng{k}.cuh").read_text()
    assert hdr == codegen.emit_process_header(k)
    built = os.path.join(ROOT, "madflow_gb300", "csrc", "generated", f"ttng{k}.cuh")
    if os.path.exists(built):
        assert open(built).read() == hdr


def test_param_card_and_model(tmp_path):
    (path,) = export("g g > t t~ g g", tmp_path)
    card = read_param_card(tmp_path / "Cards" / "param_card.dat")
    assert card["MASS"][6] == 173.0 and card["DECAY"][6] == 1.4915 and card["SMINPUTS"][3] == 0.118
    model = _load(path).get_model_param(None, str(tmp_path / "Cards" / "param_card.dat"))
    ref = sm_top_model()
    # constants held through float32, as madflow's float_me does (mdl_WT = 1.4915000200271606)
    assert model.parse_parameter("mdl_MT") == MT and model.parse_parameter("mdl_WT") == WT
    model.freeze_alpha_s(0.118)
    ref.freeze_alpha_s(0.118)
    got, want = model.evaluate(), ref.evaluate()
    assert len(got) == 5
    assert got[:2] == want[:2]
    for g, w, c in zip(got[2:], want[2:], (GC10, GC11, GC12)):
        assert complex(g.item()) == complex(w.item())
        assert abs(complex(g.item()) - c) < 1e-6 * abs(c)  # g_s of float32(0.118)
    # per-event couplings (running alpha_s)
    import torch

    a = torch.tensor([0.11, 0.118, 0.13], dtype=torch.float64)
    m2 = _load(path).get_model_param(None, str(tmp_path / "Cards" / "param_card.dat"))
    per = m2.evaluate(a)
    gs = 2.0 * np.sqrt(np.pi * a.numpy())
    np.testing.assert_allclose(per[2].numpy(), -gs, rtol=1e-15)
    np.testing.assert_allclose(per[4].numpy(), 1j * gs * gs, rtol=1e-15)


def test_pp_ttxj_folder(tmp_path):
    paths = export("p p > t t~ j", tmp_path)
    assert [p.name for p in paths] == ["matrix_1_gg_ttxg.py", "matrix_1_uux_ttxg.py", "matrix_1_ug_ttxu.py",
                                       "matrix_1_uxg_ttxux.py"]
    classes = [getattr(_load(p), p.stem.capitalize()) for p in paths]
    assert [c.nexternal for c in classes] == [5.0] * 4
    assert [c.denominator for c in classes] == [256.0, 36.0, 96.0, 96.0]
    # the initial states madflow's integrand sums over (utilities.py:25-39)
    flav = generate_initial_states(classes)
    assert flav[0] == ((21,), (21,))
    assert set(zip(*flav[1])) == {(2, -2), (4, -4), (1, -1), (3, -3), (-2, 2), (-4, 4), (-1, 1), (-3, 3)}
    assert set(zip(*flav[2])) == {(q, 21) for q in (1, 2, 3, 4)} | {(21, q) for q in (1, 2, 3, 4)}
    quark = _load(paths[1])
    m = quark.get_model_param(None, str(tmp_path / "Cards" / "param_card.dat"))
    assert list(m._tuple_functions._fields) == ["GC_10", "GC_11"]


def test_import_matrices_quark_folder(tmp_path):
    """The madflow-style loader on a folder whose modules need no device at
    construction (q q~ > t t~)."""
    export("u u~ > t t~", tmp_path)
    matrices, models = import_matrices(tmp_path)
    assert [str(m) for m in matrices] == ["1_uux_ttx"]
    assert matrices[0].nexternal == 4.0 and matrices[0].ncomb == 16.0
    assert [p for p in models[0]._tuple_constants._fields] == ["mdl_MT", "mdl_WT"]
    assert list(models[0]._tuple_functions._fields) == ["GC_11"]


@pytest.mark.gpu
def test_exported_smatrix_equals_library(cuda, tmp_path):
    """Each exported module evaluates the same kernels as the library class:
    identical |M|^2 on the same momenta, with the couplings from its own
    get_model_param at frozen alpha_s."""
    import torch

    from madflow_gb300 import matrix as M
    from madflow_gb300.phasespace import ramboflow

    export("p p > t t~ j", tmp_path / "ppj")
    export("g g > t t~ g g", tmp_path / "gg4")
    export("p p > t t~", tmp_path / "pp")
    for folder in ("ppj", "gg4", "pp"):
        matrices, models = import_matrices(tmp_path / folder)
        for mat, model in zip(matrices, models):
            model.freeze_alpha_s(0.118)
            params = model.evaluate()
            n = int(mat.nexternal)
            x = torch.rand((512, 4 * (n - 2) + 2), dtype=torch.float64, device="cuda",
                           generator=torch.Generator(device="cuda").manual_seed(n))
            ps, *_ = ramboflow(x, n, 13000.0, [MT, MT] + [0.0] * (n - 4))
            lib_cls = getattr(M, type(mat).__mro__[1].__name__)
            lib = lib_cls(precision=0)
            got = mat.smatrix(ps, *params).cpu().numpy()
            want = lib.smatrix(ps, *params).cpu().numpy()
            assert np.all(np.isfinite(got)) and np.all(got > 0), str(mat)
            np.testing.assert_array_equal(got, want)
            # madflow's --custom_op path calls cusmatrix with the same arguments
            np.testing.assert_array_equal(mat.cusmatrix(ps, *params).cpu().numpy(), got)
