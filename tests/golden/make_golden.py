"""Generate golden input/output vectors by running madflow's own Python source.

madflow's hot-path modules (``phasespace.py``, ``wavefunctions_flow.py``,
``parameters.py`` and the frozen gg->tt~ module ``tests/mockup_debug_me.py``)
import TensorFlow and pdfflow, which are not installed here.  ``tfshim.py``
supplies numpy stand-ins for the handful of TF calls they make (with TF's
float32 conversion of Python floats), so the reference code itself produces the
outputs stored in ``golden.npz``.

Run (in a checkout that has the reference source)::

    python tests/golden/make_golden.py /path/to/madflow

The fixture is committed; the tests only read it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, HERE)
    import tfshim

    tfshim.install()
    sys.path.insert(0, os.path.join(ref_root, "python_package"))
    import warnings

    warnings.filterwarnings("ignore")
    from madflow import phasespace as ps
    from madflow import wavefunctions_flow as wf
    from madflow import parameters
    from madflow.tests import mockup_debug_me as mk

    rng = np.random.default_rng(20240607)
    out = {}

    # --- constants as the reference sees them
    out["const_PI"] = np.float64(ps.PI)
    out["const_ACC"] = np.float64(ps.ACC)
    out["const_SQH"] = np.float64(wf.SQH)

    # --- rambo, massless, n = 2..7, fixed sqrt(s) (test_ps.py:59-67)
    for n in range(2, 8):
        x = rng.uniform(size=(7, 4 * n))
        p, w = ps.rambo(x, n, 7e3, masses=None)
        out[f"rambo0_n{n}_x"] = x
        out[f"rambo0_n{n}_p"] = p
        out[f"rambo0_n{n}_w"] = w
    # per-event sqrt(s)
    x = rng.uniform(size=(13, 4 * 5))
    sq = rng.uniform(size=13) * 7e3
    p, w = ps.rambo(x, 5, sq, masses=None)
    out["rambo0_var_x"], out["rambo0_var_sqrts"], out["rambo0_var_p"], out["rambo0_var_w"] = x, sq, p, w

    # --- rambo, massive (Newton rescaling with the batch-wide stopping rule)
    cases = {
        "tt": (2, [173.0, 173.0], 1000.0, 64),
        "ttg": (3, [173.0, 173.0, 0.0], 1500.0, 64),
        "ttgg": (4, [173.0, 173.0, 0.0, 0.0], 2000.0, 64),
        "ttggg": (5, [173.0, 173.0, 0.0, 0.0, 0.0], 2500.0, 64),
        "zh": (2, [50.0, 125.0], 7000.0, 16),
        "single": (4, [173.0, 173.0, 0.0, 0.0], 800.0, 1),
    }
    for name, (n, m, sq, nev) in cases.items():
        x = rng.uniform(size=(nev, 4 * n))
        p, w = ps.rambo(x, n, sq, masses=m)
        out[f"rambom_{name}_x"] = x
        out[f"rambom_{name}_p"] = p
        out[f"rambom_{name}_w"] = w
        out[f"rambom_{name}_meta"] = np.array([n, sq] + m, dtype=np.float64)

    # --- ramboflow (x1, x2 + rambo + flux), nparticles 4..7
    flows = {
        "gg_ttx": (4, 13000.0, [173.0, 173.0]),
        "gg_ttxg": (5, 13000.0, [173.0, 173.0, 0.0]),
        "gg_ttxgg": (6, 13000.0, [173.0, 173.0, 0.0, 0.0]),
        "gg_ttxggg": (7, 13000.0, [173.0, 173.0, 0.0, 0.0, 0.0]),
        "massless5": (5, 7000.0, None),
    }
    for name, (npar, sq, m) in flows.items():
        x = rng.uniform(size=(32, (npar - 2) * 4 + 2))
        p, w, x1, x2 = ps.ramboflow(x, npar, sq, masses=m)
        out[f"flow_{name}_x"] = x
        out[f"flow_{name}_p"] = p
        out[f"flow_{name}_w"] = w
        out[f"flow_{name}_x1"] = x1
        out[f"flow_{name}_x2"] = x2
        out[f"flow_{name}_meta"] = np.array([npar, sq] + (m or [0.0] * (npar - 2)), dtype=np.float64)

    # --- PhaseSpaceGenerator with a pT window cut on particle 3 (test_ps.py:70-93)
    gen = ps.PhaseSpaceGenerator(5, 7e3, algorithm="ramboflow")
    gen.register_cut("pt", particle=3, min_val=60, max_val=300.0)
    x = rng.uniform(size=(2000, 14))
    cps, cw, cx1, cx2, idx = gen(x)
    out["psgen_cut_x"], out["psgen_cut_p"], out["psgen_cut_w"] = x, cps, cw
    out["psgen_cut_x1"], out["psgen_cut_x2"], out["psgen_cut_idx"] = cx1, cx2, idx
    # massive + lab-frame output (test_ps.py:96-106 plus _boost_to_lab)
    gen2 = ps.PhaseSpaceGenerator(4, 7e3, masses=[50.0, 125.0], com_output=False)
    x = rng.uniform(size=(50, 10))
    lps, lw, lx1, lx2, _ = gen2(x)
    out["psgen_lab_x"], out["psgen_lab_p"], out["psgen_lab_w"] = x, lps, lw
    out["psgen_lab_x1"], out["psgen_lab_x2"] = lx1, lx2

    # --- external wavefunctions on a momentum set with the special cases
    p_set = []
    for _ in range(6):  # generic massive
        v = rng.normal(size=3) * 300
        p_set.append([np.sqrt(173.0**2 + v @ v), *v])
    for _ in range(4):  # generic massless
        v = rng.normal(size=3) * 300
        p_set.append([np.sqrt(v @ v), *v])
    p_set.append([500.0, 0.0, 0.0, 500.0])  # along +z (pt = 0)
    p_set.append([500.0, 0.0, 0.0, -500.0])  # along -z (pp3 = 0 / sqp0p3 = 0)
    p_set.append([173.0, 0.0, 0.0, 0.0])  # at rest (pp = 0, massive)
    p_set.append([np.sqrt(173.0**2 + 40.0**2), 0.0, 0.0, -40.0])  # massive along -z
    p_set.append([np.sqrt(173.0**2 + 40.0**2), 0.0, 0.0, 40.0])  # massive along +z
    pw = np.array(p_set, dtype=np.float64)
    out["wf_p"] = pw
    f64 = np.float64
    for mass in (0.0, 173.0):
        for nhel in (-1.0, 1.0):
            for nsf in (-1.0, 1.0):
                tag = f"m{int(mass)}_h{int(nhel)}_s{int(nsf)}"
                out[f"wf_ix_{tag}"] = wf.ixxxxx(pw, f64(mass), f64(nhel), f64(nsf))
                out[f"wf_ox_{tag}"] = wf.oxxxxx(pw, f64(mass), f64(nhel), f64(nsf))
    for mass in (0.0, 91.0):
        hels = (-1.0, 1.0, 4.0) if mass == 0.0 else (-1.0, 0.0, 1.0, 4.0)
        for nhel in hels:
            for nsv in (-1.0, 1.0):
                tag = f"m{int(mass)}_h{int(nhel)}_s{int(nsv)}"
                out[f"wf_vx_{tag}"] = wf.vxxxxx(pw, f64(mass), f64(nhel), f64(nsv))
    # sxxxxx (wavefunctions_flow.py:34-51) is not exercised: it calls
    # tf.expand_dims on a rank-0 tensor with axis=1, which TensorFlow rejects,
    # so the reference routine has no output to pin.

    # --- ALOHA routines of the mock-up module on external wavefunctions
    fin = wf.ixxxxx(pw, f64(173.0), f64(1.0), f64(-1.0))
    fout = wf.oxxxxx(pw[::-1].copy(), f64(173.0), f64(-1.0), f64(1.0))
    v1 = wf.vxxxxx(pw, f64(0.0), f64(1.0), f64(-1.0))
    v2 = wf.vxxxxx(pw[::-1].copy(), f64(0.0), f64(-1.0), f64(1.0))
    gc10, gc11 = mk.GC_10, mk.GC_11
    out["aloha_fin"], out["aloha_fout"], out["aloha_v1"], out["aloha_v2"] = fin, fout, v1, v2
    out["aloha_FFV1_0"] = mk.FFV1_0(fin, fout, v1, gc11)
    out["aloha_FFV1_1"] = mk.FFV1_1(fout, v1, gc11, f64(173.0), f64(mk.mdl_WT))
    out["aloha_FFV1_2"] = mk.FFV1_2(fin, v1, gc11, f64(173.0), f64(mk.mdl_WT))
    out["aloha_VVV1P0_1"] = mk.VVV1P0_1(v1, v2, gc10, f64(0.0), f64(0.0))

    # --- the frozen gg -> tt~ matrix element (mockup_debug_me.py:419-543)
    m = mk.Matrix_1_gg_ttx()
    x = rng.uniform(size=(256, 8))
    p, w = ps.rambo(x, 2, 1000.0, masses=[173.0, 173.0])
    zero = np.zeros((256, 1))
    pa = np.stack([zero + 500.0, zero, zero, zero + 500.0], axis=-1)
    pb = np.stack([zero + 500.0, zero, zero, zero - 500.0], axis=-1)
    allp = np.concatenate([pa, pb, p], axis=1)
    out["me_ggttx_p"] = allp
    out["me_ggttx_smatrix"] = m.smatrix(allp, *mk.model_params)
    hel_me = np.stack([np.real(m.matrix(allp[:8], h, *mk.model_params)) for h in m.helicities])
    out["me_ggttx_matrix_hel"] = hel_me  # (16, 8)
    out["me_ggttx_helicities"] = np.asarray(m.helicities)
    out["me_ggttx_params"] = np.array(
        [mk.mdl_MT, mk.mdl_WT, mk.GC_10.real, mk.GC_10.imag, mk.GC_11.real, mk.GC_11.imag]
    )
    # ramboflow at 13 TeV through smatrix (a full integrand point without PDF)
    pf = out["flow_gg_ttx_p"]
    out["me_flow_ggttx_smatrix"] = m.smatrix(pf, *mk.model_params)

    # --- couplings from alpha_s (parameters.py:13-15) and a frozen Model
    a_s = np.array([0.118, 0.1, 0.2], dtype=np.float64)
    out["param_alphas"] = a_s
    out["param_gs"] = parameters._alphas_to_gs(a_s)
    model = parameters.Model((mk.mdl_MT, mk.mdl_WT), (lambda gs: -gs, lambda gs: 1j * gs))
    model.freeze_alpha_s(0.118)
    fz = model.evaluate()
    out["param_frozen_gc10"] = np.asarray(fz[2])
    out["param_frozen_gc11"] = np.asarray(fz[3])

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MADFLOW_REFERENCE", ""))
