"""Generate the golden fixtures of the parity tests (run from the repo root).

The reference ships no golden vectors for the KPP solve and its Fortran cannot
be compiled here, so these fixtures are produced by the CPU oracle (the C
restatement, strict build) and committed: they pin the oracle against
regressions and give the GPU tests fixed inputs and outputs.

    python tests/golden/make_golden.py

Cases (seeded synthetic box-model cells, inputs + outputs):
  box16_rodas3_600s   16 cells, one 600 s Rodas3 step at the default controls
  box8_methods        8 cells x {Ros2, Ros3, Ros4, Rodas4, Rang3}, 300 s
  box8_options        8 cells, non-autonomous + scalar tolerances + clamping
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402


def make():
    __graft_entry__.load_package()
    import gcchem.inputs as inputs

    orc = __graft_entry__.load_oracle()
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    out = {}

    cells = inputs.box_cells(16, seed=123)
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    c, ist, rst, ierr = orc.integrate(cells["c"], r, atol, rtol, 0.0, 600.0, icntrl, rcntrl)
    out["box16_rodas3_600s"] = dict(met=cells["met"], photol=cells["photol"], c_in=cells["c"], rconst=r, c_out=c,
                                    istatus=ist, rstatus=rst, ierr=ierr, icntrl=icntrl, rcntrl=rcntrl,
                                    atol=atol, rtol=rtol, tout=np.array(600.0))

    cells = inputs.box_cells(8, seed=321)
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    for name, meth in [("ros2", 1), ("ros3", 2), ("ros4", 3), ("rodas4", 5), ("rang3", 6)]:
        ic = icntrl.copy()
        ic[2] = meth
        c, ist, rst, ierr = orc.integrate(cells["c"], r, atol, rtol, 0.0, 300.0, ic, rcntrl)
        out["box8_%s" % name] = dict(c_in=cells["c"], rconst=r, c_out=c, istatus=ist, rstatus=rst, ierr=ierr,
                                     icntrl=ic, rcntrl=rcntrl, atol=atol, rtol=rtol, tout=np.array(300.0))

    ic = icntrl.copy()
    ic[0] = 0      # non-autonomous: ros_FunTimeDerivative path
    ic[1] = 1      # scalar tolerances
    ic[15] = 1     # clamp negatives on acceptance
    rc = rcntrl.copy()
    rc[2] = 0.5    # Hstart
    rc[4] = 4.0    # FacMax
    c, ist, rst, ierr = orc.integrate(cells["c"], r, atol[:1] * 10, rtol[:1] * 2, 0.0, 300.0, ic, rc)
    out["box8_options"] = dict(c_in=cells["c"], rconst=r, c_out=c, istatus=ist, rstatus=rst, ierr=ierr, icntrl=ic,
                               rcntrl=rc, atol=atol[:1] * 10, rtol=rtol[:1] * 2, tout=np.array(300.0))

    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, "ierr", d["ierr"], "steps", d["istatus"][2])


if __name__ == "__main__":
    make()
