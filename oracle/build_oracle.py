"""Build the CPU oracle shared libraries -- TEST INFRASTRUCTURE.

* ``_build/liboracle_strict.so``  -O2 -ffp-contract=off: the parity oracle,
  the reference's arithmetic without contraction.
* ``_build/liboracle_fast.so``    -O3 with the compiler's default contraction:
  the timed CPU baseline (OpenMP cell loop).

Plain gcc, no -march=native (the same recipe builds on x86-64 and aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
GEN = os.path.join(HERE, "_gen")

VARIANTS = {
    "strict": ["-O2", "-ffp-contract=off"],
    "fast": ["-O3"],
}


MECHANISMS = ("fullchem", "Hg")


def lib_path(variant="strict", mech="fullchem"):
    name = "liboracle_%s.so" % variant if mech == "fullchem" else "liboracle_%s_%s.so" % (mech, variant)
    return os.path.join(BUILD, name)


def build(verbose=False, mechs=MECHANISMS):
    sys.path.insert(0, HERE)
    import gen_oracle  # noqa: E402

    os.makedirs(BUILD, exist_ok=True)
    procs = []
    for mech in mechs:
        gen = os.path.join(GEN, mech)
        gen_oracle.write(gen, mech)
        procs += _compile(gen, mech, verbose)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), out.decode()))
    return {(m, v): lib_path(v, m) for m in mechs for v in VARIANTS}


def _compile(gen, mech, verbose):
    srcs = [os.path.join(HERE, "kpp_oracle.c"), os.path.join(gen, "kpp_mech_oracle.c"),
            os.path.join(gen, "kpp_rates_oracle.c"), os.path.join(HERE, "het_state.c")]
    deps = srcs + [os.path.join(HERE, f) for f in ("kpp_oracle.h", "rate_laws.h", "het_laws.h")] + \
        [os.path.join(gen, "kpp_dims.h"), os.path.join(gen, "oracle_het_layout.h")]
    procs = []
    for variant, flags in VARIANTS.items():
        out = lib_path(variant, mech)
        if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
            continue
        cmd = ["gcc", "-shared", "-fPIC", "-fopenmp", "-std=gnu11", "-I", HERE, "-I", gen] + flags + srcs + \
            ["-o", out, "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    return procs


if __name__ == "__main__":
    print(build(verbose=True))
