"""KPP-Standalone state files (GeosCore/kppsa_interface_mod.F90:569-870
layout): write -> read round trip, reaction rates, batch assembly."""
import os
import re
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


def _field(desc):
    """Regex of one output field of a Fortran edit descriptor (i6, f11.4,
    e11.4, es25.16e3, es10.2e2, i0)."""
    m = re.fullmatch(r"(?i)(es|e|f|i)(\d+)(?:\.(\d+))?(?:e(\d+))?", desc)
    kind, w = m.group(1).lower(), int(m.group(2))
    d = int(m.group(3) or 0)
    if kind == "i":  # the width is checked by _fits
        return r" *-?\d+"
    if kind == "f":
        return r" *-?\d*\.\d{%d}" % d
    if kind == "e":  # 0.ddddE+ee (or +eee without the E)
        return r" *-?0\.\d{%d}(?:E[+-]\d\d|[+-]\d{3})" % d
    e = int(m.group(4))
    return r" *-?\d\.\d{%d}E[+-]\d{%d}" % (d, e)


def _fits(value, desc):
    w = int(re.search(r"\d+", desc).group())
    return (w == 0 or len(value) == w) and re.fullmatch(_field(desc), value) is not None


def test_writer_follows_the_reference_layout(tmp_path):
    """The header lines from 'Meteorological and general grid cell metadata'
    on, and every CSV row, in the order and edit descriptors of the
    reference writer (tests/golden/kppsa_layout.json, extracted from
    GeosCore/kppsa_interface_mod.F90 by tests/golden/make_kppsa_layout.py)."""
    import json

    import gcchem.inputs as inputs
    import gcchem.kppsa as kppsa
    import gcchem.mechanism as mechanism

    layout = json.load(open(os.path.join(ROOT, "tests", "golden", "kppsa_layout.json")))
    ir = mechanism.load_ir()
    cells = inputs.box_cells(1, seed=4)
    nspec = ir["dims"]["nspec"]
    atol = np.r_[inputs.tolerances()[0], np.ones(nspec - ir["dims"]["nvar"])]
    rconst = np.random.default_rng(2).lognormal(-20, 5, ir["dims"]["nreact"])
    ic, rc = inputs.default_controls()
    meta = {"location": "cell_A", "timestamp": "20190701_1200z", "lon": -70.25, "lat": 40.5, "level": 3,
            "press": 850.123, "temp": 280.567, "numden": 2.1e19, "h2o_vmr": 0.004, "cldf": 0.0, "suncos": -0.7,
            "h_init": 12.5, "h_exit": 300.0, "dt": 600.0, "steps": 7}
    path = str(tmp_path / "cell.txt")
    kppsa.write_state(path, cells["c"][:, 0], rconst, atol, meta, ic, rc, ir)
    lines = open(path).read().splitlines()
    name_at = lines.index("Name,   Value,   Absolute Tolerance")
    assert int(lines[0]) == name_at + 1  # the first line counts the header lines
    k = lines.index(layout["lines"][0]["text"])
    for entry in layout["lines"]:
        fmt, text = entry["format"].strip("()"), entry["text"]
        parts = fmt.split(",")
        if parts[0] == "/":
            assert lines[k] == "", (k, lines[k])
            k += 1
            parts = parts[1:]
        line = lines[k]
        if parts[0] == "a" and len(parts) > 1 and parts[1] not in ("/",):
            w = len(text)
            assert line[:w] == text, (line, text)
            if parts[1] != "a":
                assert _fits(line[w:], parts[1]), (line, parts[1])
        elif parts[0] == "a":
            assert line == ("=" * 76 if text is None else text), (line, text)
        else:  # 10i6, 5F13.6: repeated fields
            n, desc = re.fullmatch(r"(\d+)(\w+\.?\d*)", parts[0]).groups()
            w = int(re.search(r"\d+", desc).group())
            assert len(line) == int(n) * w
            assert all(_fits(line[j:j + w], desc) for j in range(0, len(line), w)), line
        k += 1
        if parts[-1] == "/":
            assert lines[k] == ""
            k += 1
    assert k == name_at + 1
    # CSV rows: species (FORMAT 130; 120 for unmapped species), R (140), A (150)
    f = layout["csv_formats"]
    desc = lambda fmt: re.findall(r"(?i)\b(es\d+\.\d+e\d+|i0|a)\b", re.sub(r'"[^"]*"', "", fmt))
    assert desc(f["130"]) == ["a", "es25.16e3", "es10.2e2"] and desc(f["120"]) == ["i0", "es25.16e3", "es10.2e2"]
    assert desc(f["140"]) == desc(f["150"]) == ["i0", "es25.16e3"]
    rows = lines[name_at + 1:]
    nreact = ir["dims"]["nreact"]
    assert len(rows) == nspec + 2 * nreact
    for row, name in zip(rows[:nspec], ir["species"]):
        nm, v, t = row.split(",")
        assert nm == name and _fits(v, "es25.16e3") and _fits(t, "es10.2e2"), row
    for pre, rows_ in (("R", rows[nspec:nspec + nreact]), ("A", rows[nspec + nreact:])):
        assert f["140" if pre == "R" else "150"].startswith('"%s"' % pre)
        for n, row in enumerate(rows_):
            key, v = row.split(",")
            assert key == "%s%d" % (pre, n + 1) and _fits(v, "es25.16e3"), row


def test_fortran_e_format():
    import gcchem.kppsa as kppsa

    # Ew.d: 0.dddd mantissa, two exponent digits (E dropped beyond 99)
    assert kppsa.fortran_e(2.1e19) == " 0.2100E+20"
    assert kppsa.fortran_e(0.004) == " 0.4000E-02"
    assert kppsa.fortran_e(-1.5e-5) == "-0.1500E-04"
    assert kppsa.fortran_e(0.0) == " 0.0000E+00"
    assert kppsa.fortran_e(999995.0) == " 0.1000E+07"
    assert kppsa.fortran_e(1e-120) == " 0.1000-119"
