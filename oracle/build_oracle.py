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


def lib_path(variant="strict"):
    return os.path.join(BUILD, "liboracle_%s.so" % variant)


def build(verbose=False):
    sys.path.insert(0, HERE)
    import gen_oracle  # noqa: E402

    gen_oracle.write(GEN)
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "kpp_oracle.c"), os.path.join(GEN, "kpp_mech_oracle.c"),
            os.path.join(GEN, "kpp_rates_oracle.c")]
    deps = srcs + [os.path.join(HERE, f) for f in ("kpp_oracle.h", "rate_laws.h")] + [os.path.join(GEN, "kpp_dims.h")]
    procs = []
    for variant, flags in VARIANTS.items():
        out = lib_path(variant)
        if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
            continue
        cmd = ["gcc", "-shared", "-fPIC", "-fopenmp", "-std=gnu11", "-I", HERE] + flags + srcs + ["-o", out, "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), out.decode()))
    return {v: lib_path(v) for v in VARIANTS}


if __name__ == "__main__":
    print(build(verbose=True))
