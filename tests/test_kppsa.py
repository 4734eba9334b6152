"""KPP-Standalone state files (GeosCore/kppsa_interface_mod.F90:569-870
layout): write -> read round trip, reaction rates, batch assembly."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def test_state_file_round_trip(tmp_path):
    import gcchem.inputs as inputs
    import gcchem.kppsa as kppsa
    import gcchem.mechanism as mechanism
    import ir_eval

    ir = mechanism.load_ir()
    cells = inputs.box_cells(3, seed=2)
    atol_v, rtol = inputs.tolerances()
    nspec, nvar = ir["dims"]["nspec"], ir["dims"]["nvar"]
    atol = np.r_[atol_v, np.ones(nspec - nvar)]
    rconst = np.random.default_rng(1).lognormal(-20, 5, ir["dims"]["nreact"])
    icntrl, rcntrl = inputs.default_controls()
    rcntrl = rcntrl.copy()
    rcntrl[2] = 12.5
    paths = []
    for k in range(3):
        p = str(tmp_path / ("cell%d.txt" % k))
        meta = {"location": "box%d" % k, "timestamp": "2019-07-01 12:00", "lon": -70.25, "lat": 40.5, "level": 3,
                "press": 850.0, "temp": 280.5, "numden": 2.1e19, "h2o_vmr": 0.004, "cldf": 0.0, "suncos": 0.7,
                "h_init": 12.5, "h_exit": 300.0, "dt": 600.0, "steps": 7}
        kppsa.write_state(p, cells["c"][:, k], rconst, atol, meta, icntrl, rcntrl, ir)
        paths.append(p)
        st = kppsa.read_state(p, ir)
        assert np.array_equal(st["c"], cells["c"][:, k])          # 17 significant digits: exact
        assert np.array_equal(st["rconst"], rconst)
        assert np.allclose(st["atol"], atol, rtol=1e-2)            # ES10.2 tolerances
        assert np.array_equal(st["icntrl"], icntrl)
        assert np.allclose(st["rcntrl"], rcntrl)
        assert st["meta"]["level"] == 3 and st["meta"]["steps"] == 7 and st["meta"]["location"] == "box%d" % k
        assert np.isclose(st["meta"]["temp"], 280.5) and np.isclose(st["meta"]["numden"], 2.1e19, rtol=1e-4)
        # A(r): the Fun products, against the statement-by-statement IR evaluation
        V, F = cells["c"][:nvar, k], cells["c"][nvar:, k]
        ref = np.array([ir_eval._prod(toks, V, F, rconst) for toks in ir["fun"]["A"]])
        assert np.array_equal(st["a"], np.array([float(kppsa.fortran_es(v)) for v in ref]))
    c, r, metas = kppsa.cells_from_states(paths, ir)
    assert c.shape == (nspec, 3) and r.shape == (ir["dims"]["nreact"], 3)
    assert np.array_equal(c, cells["c"]) and [m["location"] for m in metas] == ["box0", "box1", "box2"]


def test_fortran_es_format():
    import gcchem.kppsa as kppsa

    assert kppsa.fortran_es(12345.678) == "1.2345678000000000E+004"
    assert kppsa.fortran_es(-0.5) == "-5.0000000000000000E-001"
    assert kppsa.fortran_es(-1.5e-300).endswith("E-300") and float(kppsa.fortran_es(-1.5e-300)) == -1.5e-300
    assert kppsa.fortran_es(0.0) == "0.0000000000000000E+000"
    assert kppsa.fortran_es(1e-2, 2, 2) == "1.00E-02"
