"""Build the CUDA libraries in-tree for sm_103a.

Steps: lower each mechanism's IR (``mechanism/<name>.json``) to device tables
(``csrc/_gen/<name>``), compile the Rosenbrock kernels once per arithmetic
variant (strict: ``-fmad=false``; fast: default contraction; 1, 2 and 4 cells
per thread), the rate, utility and MLP kernels once, the C ABI once per
mechanism, and link ``lib/libgckpp_gb300.so`` (fullchem) and
``lib/libgckpp_gb300_<name>.so`` (the other mechanisms).  The kernels are
table-driven, so every mechanism shares them.  Translation units are compiled
in parallel; nothing here needs CMake.
"""
import os
import shutil
import subprocess
import sys

from . import rates_program, tables

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
GEN = os.path.join(CSRC, "_gen")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "libgckpp_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH


def nvcc():
    for cand in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


MECHANISMS = ("fullchem", "Hg")  # KPP mechanisms with a library each (mechanism/<name>.json)


def lib_path(mech="fullchem"):
    """libgckpp_gb300.so (fullchem) or libgckpp_gb300_<mech>.so."""
    return os.path.join(LIBDIR, LIBNAME if mech == "fullchem" else "libgckpp_gb300_%s.so" % mech)


def _units():
    k = os.path.join(CSRC, "kpp_kernels.cu")
    return [
        (k, "kpp_kernels_strict.o", ["-DGCKPP_STRICT=1", "-DGCKPP_VARIANT=strict", "-fmad=false"]),
        (k, "kpp_kernels_fast.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast", "-DGCKPP_NC=1"]),
        (k, "kpp_kernels_fast2.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast2", "-DGCKPP_NC=2"]),
        (k, "kpp_kernels_fast4.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast4", "-DGCKPP_NC=4"]),
        (os.path.join(CSRC, "kpp_rates.cu"), "kpp_rates.o", []),
        (os.path.join(CSRC, "kpp_util.cu"), "kpp_util.o", []),
        # no FMA contraction: the producer's arithmetic rounds as the Fortran's
        (os.path.join(CSRC, "het_state.cu"), "het_state.o", ["-fmad=false"]),
        (os.path.join(CSRC, "kpp_mlp.cu"), "kpp_mlp.o", []),
        (os.path.join(CSRC, "gckpp_mlp_capi.cu"), "gckpp_mlp_capi.o", []),
        (os.path.join(CSRC, "gckpp_learned_capi.cu"), "gckpp_learned_capi.o", []),
    ]


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    from . import mechanism

    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    deps += [os.path.join(PKG, "..", "include", f) for f in ("gckpp_gb300.h", "gckpp_gb300_mlp.h")]
    units = list(_units())
    # the mechanism enters only through the tables that gckpp_capi.cu uploads:
    # one C ABI object (and library) per mechanism, every kernel object shared
    mech_objs = {}
    for mech in MECHANISMS:
        gen = os.path.join(GEN, mech)
        ir = mechanism.load_ir(mech)
        tables.write_generated(gen, ir)
        rates_program.write_generated(gen, ir)
        gen_deps = [os.path.join(gen, f) for f in os.listdir(gen)]
        objs = ["gckpp_capi_%s.o" % mech, "rates_direct_%s.o" % mech]
        units.append((os.path.join(CSRC, "gckpp_capi.cu"), objs[0], ["-I", gen], gen_deps))
        units.append((os.path.join(CSRC, "rates_direct.cu"), objs[1], ["-I", gen], gen_deps))
        mech_objs[mech] = objs
    exe = nvcc()
    procs = []
    shared = []
    for unit in units:
        src, obj, extra = unit[:3]
        extra_deps = unit[3] if len(unit) > 3 else []
        obj = os.path.join(BUILD, obj)
        if not any(os.path.basename(obj) in objs for objs in mech_objs.values()):
            shared.append(obj)
        if force or _stale(obj, deps + extra_deps):
            cmd = [exe] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode()))
        if verbose and out:
            print(out.decode())
    links = []
    for mech, own in mech_objs.items():
        lib = lib_path(mech)
        objs = shared + [os.path.join(BUILD, o) for o in own]
        if force or procs or not os.path.exists(lib):
            cmd = [exe] + ARCH + ["-shared", "-cudart", "shared", "-o", lib] + objs
            links.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in links:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), out.decode()))
    # profiling aid: the mechanism routines one launch each (not the C ABI)
    rb = routines_path()
    rb_src = os.path.join(CSRC, "routine_bench.cu")
    rb_deps = deps + [os.path.join(GEN, "fullchem", f) for f in os.listdir(os.path.join(GEN, "fullchem"))]
    if force or _stale(rb, rb_deps):
        cmd = [exe] + NVCC_FLAGS + ["-I", os.path.join(GEN, "fullchem"), "-shared", "-cudart", "shared", rb_src,
                                    "-o", rb]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("routine bench build failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    lib = lib_path()
    probe = probe_path()
    src = os.path.join(CSRC, "fp64_probe.cu")
    if force or not os.path.exists(probe) or os.path.getmtime(src) > os.path.getmtime(probe):
        cmd = [exe] + NVCC_FLAGS + ["-shared", "-cudart", "shared", src, "-o", probe]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("probe build failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    return lib


def phase_cycles_path():
    """Profiling copy of the fullchem library whose split block-per-cell
    kernel counts its cycles per phase (gc_kpp_phase_cycles); not built by
    build()."""
    return os.path.join(LIBDIR, "libgckpp_gb300_phases.so")


def build_phase_cycles(verbose=False):
    """Builds phase_cycles_path(): the objects of build() with the fast
    one-cell-per-thread kernels recompiled with -DGCKPP_PHASE_CYCLES."""
    lib = build(verbose=verbose)
    exe = nvcc()
    obj = os.path.join(BUILD, "kpp_kernels_fast_phases.o")
    src, name, extra = next(u for u in _units() if u[1] == "kpp_kernels_fast.o")
    cmd = [exe] + NVCC_FLAGS + extra + ["-DGCKPP_PHASE_CYCLES", "-c", src, "-o", obj]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    objs = [os.path.join(BUILD, u[1]) for u in _units() if u[1] != name] + [obj]
    objs += [os.path.join(BUILD, o) for o in ("gckpp_capi_fullchem.o", "rates_direct_fullchem.o")]
    out = phase_cycles_path()
    cmd = [exe] + ARCH + ["-shared", "-cudart", "shared", "-o", out] + objs
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    if verbose:
        print(out)
    return lib, out


def routines_path():
    """Per-routine launches of the fullchem tables for profiling, not part of the C ABI."""
    return os.path.join(LIBDIR, "libgckpp_routines.so")


def probe_path():
    """FP64 throughput probe library (the roofline denominator), not part of the C ABI."""
    return os.path.join(LIBDIR, "libgckpp_probe.so")


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
