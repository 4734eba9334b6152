"""KPP-Standalone chemical-state files: read and write.

GEOS-Chem writes one text file per sampled grid cell and chemistry step
(GeosCore/kppsa_interface_mod.F90:569-870, KppSa_Write_Samples): a first line
with the number of header lines, a free-text header with the cell's
meteorological metadata ("Label:  value" lines) and the integrator options
(ICNTRL in two rows of 10 integers, RCNTRL in four rows of 5 reals), then CSV
rows after a "Name, Value, Absolute Tolerance" line:

    <species name>,<initial concentration>,<ATOL>      (NSPEC rows, KPP order;
    C<n>,<value>,<ATOL>                                 unmapped species)
    R<n>,<rate constant>                               (NREACT rows)
    A<n>,<instantaneous reaction rate>                 (NREACT rows)

Such files turn cells of a real model run into inputs of this solver
(`cells_from_states`) and fixtures of its tests.  `write_state` produces the
same layout, with numbers in the writer's formats (ES25.16E3 values, ES10.2E2
tolerances, the metadata's I6, F11.4, F11.2 and E11.4 fields).
"""
import re

import numpy as np

from . import mechanism

RULE = "=" * 76

META_LABELS = {
    "location": "Location:",
    "timestamp": "Timestamp:",
    "lon": "Longitude (degrees):",
    "lat": "Latitude (degrees):",
    "level": "GEOS-Chem Vertical Level:",
    "press": "Pressure (hPa):",
    "temp": "Temperature (K):",
    "numden": "Dry air density (molec/cm3):",
    "h2o_vmr": "Water vapor mixing ratio (vol H2O/vol dry air):",
    "cldf": "Cloud fraction:",
    "suncos": "Cosine of solar zenith angle:",
    "h_init": "Init KPP Timestep (seconds):",
    "h_exit": "Exit KPP Timestep (seconds):",
    "dt": "Chemistry operator timestep (seconds):",
    "steps": "Number of internal timesteps:",
}
_NUMERIC = {"lon", "lat", "press", "temp", "numden", "h2o_vmr", "cldf", "suncos", "h_init", "h_exit", "dt"}
_INTEGER = {"level", "steps"}


def fortran_e(x, width=11, digits=4):
    """A real in Fortran Ew.d form, as the writer's e11.4 fields print it:
    0.ddddE+ee (mantissa in [0.1, 1), two exponent digits; for 99 < |e| <=
    999 the E is dropped, +eee), right-justified in `width` columns."""
    x = float(x)
    if x == 0.0:
        body = "0." + "0" * digits + "E+00"
    else:
        m, e = ("%.*E" % (digits - 1, abs(x))).split("E")
        ev = int(e) + 1
        exp = ("E%s%02d" % ("-" if ev < 0 else "+", abs(ev)) if abs(ev) <= 99
               else "%s%03d" % ("-" if ev < 0 else "+", abs(ev)))
        body = ("-" if x < 0 else "") + "0." + m.replace(".", "") + exp
    return body.rjust(width)


def fortran_es(x, digits=16, expdigits=3):
    """A real in Fortran ESw.dEe form: d.ddd...E+eee (no leading blanks)."""
    x = float(x)
    if x == 0.0:
        return "0." + "0" * digits + "E+" + "0" * expdigits
    m, e = ("%.*E" % (digits, x)).split("E")
    ev = int(e)
    return "%sE%s%0*d" % (m, "-" if ev < 0 else "+", expdigits, abs(ev))


def reaction_rates(c, rconst, ir=None):
    """A(r) = RCT(r) * product of its reactant concentrations, the Aout of
    KPP's Fun (KPP/fullchem/gckpp_Function.F90), for one cell."""
    ir = ir or mechanism.load_ir()
    nvar = ir["dims"]["nvar"]
    out = np.empty(len(ir["fun"]["A"]))
    for r, factors in enumerate(ir["fun"]["A"]):
        v = 1.0
        for f in factors:
            kind, rest = f[0], f[1:]
            if kind == "R":
                v = v * rconst[int(rest)]
            elif kind == "V":
                v = v * c[int(rest)]
            elif kind == "F":
                v = v * c[nvar + int(rest)]
            else:
                v = v * float(f.replace("d", "e").replace("D", "e"))
        out[r] = v
    return out


def write_state(path, c, rconst, atol, meta=None, icntrl=None, rcntrl=None, ir=None, rates=None):
    """Write one cell's state (c [NSPEC], rconst [NREACT], atol [NSPEC])."""
    ir = ir or mechanism.load_ir()
    names = ir["species"]
    meta = dict(meta or {})
    icntrl = np.zeros(20, np.int64) if icntrl is None else np.asarray(icntrl)
    rcntrl = np.zeros(20) if rcntrl is None else np.asarray(rcntrl)
    a = reaction_rates(c, rconst, ir) if rates is None else rates
    head = [RULE, "", "                  KPP Standalone Atmospheric Chemical State", "File Description:",
            "This file contains the atmospheric chemical state of one grid cell, written",
            "in the layout of GEOS-Chem's KPP Standalone interface: concentrations, rate",
            "constants and KPP-specific fields; other fields are for reference.  The",
            "first line holds the number of header lines.", "",
            "Meteorological and general grid cell metadata    ", ""]
    for key, label in META_LABELS.items():
        if key in ("h_init",):
            head += ["", "KPP Integrator-specific parameters               ", ""]
        v = meta.get(key, "" if key in ("location", "timestamp") else 0)
        # the writer's formats: i6, e11.4, f11.2 (temperature), f11.4
        if key in _INTEGER:
            txt = "%6d" % int(v)
        elif key in ("numden", "h2o_vmr", "cldf", "suncos"):
            txt = fortran_e(v)
        elif key == "temp":
            txt = "%11.2f" % float(v)
        elif key in _NUMERIC:
            txt = "%11.4f" % float(v)
        else:
            txt = str(v)
        head.append("%-49s%s" % (label, txt))  # the writer's labels are 49 characters
    head.append("ICNTRL integrator options used:")
    head.append("".join("%6d" % int(v) for v in icntrl[:10]))
    head.append("".join("%6d" % int(v) for v in icntrl[10:20]))
    head.append("RCNTRL integrator options used:")
    for k in range(0, 20, 5):
        head.append("".join("%13.6f" % float(v) for v in rcntrl[k:k + 5]))
    head += ["", "CSV data of full chemical state, including species concentrations,",
             "rate constants (R) and instantaneous reaction rates (A).",
             "All concentration units are in molec/cm3 and rates in molec/cm3/s.", "", RULE,
             "Name,   Value,   Absolute Tolerance"]
    lines = [str(len(head) + 1)] + head
    for n, name in enumerate(names):
        lines.append("%s,%25s,%10s" % (name, fortran_es(c[n]), fortran_es(atol[n], 2, 2)))
    for n, v in enumerate(rconst):
        lines.append("R%d,%25s" % (n + 1, fortran_es(v)))
    for n, v in enumerate(a):
        lines.append("A%d,%25s" % (n + 1, fortran_es(v)))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _num(s):
    return float(s.strip().replace("d", "E").replace("D", "E"))


def read_state(path, ir=None):
    """One state file -> dict(meta, icntrl, rcntrl, names, c, atol, rconst, a)."""
    ir = ir or mechanism.load_ir()
    with open(path) as f:
        lines = f.read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.replace(" ", "").lower().startswith("name,value"))
    meta = {}
    for ln in lines[1:start]:
        for key, label in META_LABELS.items():
            if ln.startswith(label):
                v = ln[len(label):].strip()
                if key in _INTEGER:
                    meta[key] = int(v)
                elif key in _NUMERIC:
                    meta[key] = _num(v)
                else:
                    meta[key] = v
    icntrl = rcntrl = None
    for i, ln in enumerate(lines[:start]):
        if ln.startswith("ICNTRL"):
            icntrl = np.array([int(v) for v in (lines[i + 1] + " " + lines[i + 2]).split()], np.int32)
        if ln.startswith("RCNTRL"):
            rcntrl = np.array([_num(v) for v in " ".join(lines[i + 1:i + 5]).split()])
    names, c, atol, rconst, a = [], [], [], {}, {}
    index = {n: i for i, n in enumerate(ir["species"])}
    for ln in lines[start + 1:]:
        if not ln.strip():
            continue
        parts = ln.split(",")
        key = parts[0].strip()
        m = re.fullmatch(r"([RA])(\d+)", key)
        if m and len(parts) == 2:
            (rconst if m.group(1) == "R" else a)[int(m.group(2)) - 1] = _num(parts[1])
            continue
        names.append(key)
        c.append(_num(parts[1]))
        atol.append(_num(parts[2]))
    nspec = len(ir["species"])
    cv = np.zeros(nspec)
    av = np.zeros(nspec)
    for i, (n, v, t) in enumerate(zip(names, c, atol)):
        k = index.get(n)
        if k is None:
            mc = re.fullmatch(r"C(\d+)", n)
            k = int(mc.group(1)) - 1 if mc else i
        cv[k] = v
        av[k] = t
    nreact = ir["dims"]["nreact"]
    rv = np.array([rconst.get(k, 0.0) for k in range(nreact)])
    avr = np.array([a.get(k, 0.0) for k in range(nreact)])
    return {"meta": meta, "icntrl": icntrl, "rcntrl": rcntrl, "names": names, "c": cv, "atol": av,
            "rconst": rv, "a": avr}


def cells_from_states(paths, ir=None):
    """Several state files -> cell-interleaved c [NSPEC, n], rconst
    [NREACT, n] (the solver's batch layout), plus each file's metadata."""
    states = [read_state(p, ir) for p in paths]
    c = np.ascontiguousarray(np.stack([s["c"] for s in states], axis=1))
    r = np.ascontiguousarray(np.stack([s["rconst"] for s in states], axis=1))
    return c, r, [s["meta"] for s in states]
