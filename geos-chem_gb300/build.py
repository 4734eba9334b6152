"""Build the CUDA library ``libgckpp_gb300.so`` in-tree for sm_103a.

Steps: lower the mechanism IR to device tables (``csrc/_gen``), compile the
Rosenbrock kernels twice (strict: ``-fmad=false``; fast: default contraction),
compile the C ABI, link a shared library into ``lib/``.  Translation units are
compiled in parallel; nothing here needs CMake.
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


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _units():
    k = os.path.join(CSRC, "kpp_kernels.cu")
    return [
        (k, "kpp_kernels_strict.o", ["-DGCKPP_STRICT=1", "-DGCKPP_VARIANT=strict", "-fmad=false"]),
        (k, "kpp_kernels_fast.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast", "-DGCKPP_NC=1"]),
        (k, "kpp_kernels_fast2.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast2", "-DGCKPP_NC=2"]),
        (k, "kpp_kernels_fast4.o", ["-DGCKPP_STRICT=0", "-DGCKPP_VARIANT=fast4", "-DGCKPP_NC=4"]),
        (os.path.join(CSRC, "kpp_rates.cu"), "kpp_rates.o", []),
        (os.path.join(CSRC, "kpp_util.cu"), "kpp_util.o", []),
        (os.path.join(CSRC, "kpp_mlp.cu"), "kpp_mlp.o", []),
        (os.path.join(CSRC, "gckpp_mlp_capi.cu"), "gckpp_mlp_capi.o", []),
        (os.path.join(CSRC, "gckpp_capi.cu"), "gckpp_capi.o", []),
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
    tables.write_generated(GEN)
    rates_program.write_generated(GEN)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    deps += [os.path.join(GEN, f) for f in os.listdir(GEN)]
    deps += [os.path.join(PKG, "..", "include", f) for f in ("gckpp_gb300.h", "gckpp_gb300_mlp.h")]
    exe = nvcc()
    procs = []
    objs = []
    for src, obj, extra in _units():
        obj = os.path.join(BUILD, obj)
        objs.append(obj)
        if force or _stale(obj, deps):
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
    lib = lib_path()
    if force or procs or not os.path.exists(lib):
        cmd = [exe] + ARCH + ["-shared", "-cudart", "shared", "-o", lib] + objs
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    probe = probe_path()
    src = os.path.join(CSRC, "fp64_probe.cu")
    if force or not os.path.exists(probe) or os.path.getmtime(src) > os.path.getmtime(probe):
        cmd = [exe] + NVCC_FLAGS + ["-shared", "-cudart", "shared", src, "-o", probe]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("probe build failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    return lib


def probe_path():
    """FP64 throughput probe library (the roofline denominator), not part of the C ABI."""
    return os.path.join(LIBDIR, "libgckpp_probe.so")


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
