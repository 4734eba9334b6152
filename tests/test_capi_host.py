"""The C-ABI library loads and exports every entry point include/*.h declares
(no GPU needed; nothing here launches a kernel)."""
import ctypes
import glob
import os
import re

import pytest

import gcchem.build as build
import gcchem.capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(build.lib_path()):
        build.build()
    return capi.load_library()


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(gc_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert "gc_kpp_integrate_batch" in names and "gc_kpp_update_rconst_batch" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(capi.EXPORTED) <= set(names)


def test_mechanism_dims_without_gpu(lib):
    assert capi.dims() == {"nspec": 356, "nvar": 353, "nfix": 3, "nreact": 1058, "lu_nonzero": 5683}


def test_null_arguments_are_rejected(lib):
    assert lib.gc_kpp_ctx_create(None, 0) == capi.GC_KPP_EINVAL
    assert lib.gc_kpp_last_error() != b""
    assert lib.gc_kpp_integrate_batch(None, 1, 0.0, 1.0, None, 1, None, 1, None, None, None, None, None, None,
                                      None, 1, None, 0, None) == capi.GC_KPP_EINVAL
    assert lib.gc_kpp_ctx_destroy(None) == capi.GC_KPP_OK


def test_ctx_create_without_gpu_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = ctypes.c_void_p()
    rc = lib.gc_kpp_ctx_create(ctypes.byref(ctx), 0)
    assert rc == capi.GC_KPP_ECUDA
    assert not ctx.value


def _header_ints():
    vals = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for name, v in re.findall(r"^#define\s+(GC_\w+)\s+\(?(-?\d+)\)?", open(h).read(), re.M):
            vals[name] = int(v)
    return vals


def test_binding_constants_match_the_header():
    """Every status code, memory kind and option key of the ctypes binding
    has the value the C header gives it, and every option key of the header
    is bound."""
    vals = _header_ints()
    for name in ("GC_KPP_OK", "GC_KPP_EINVAL", "GC_KPP_ECUDA", "GC_KPP_ENOMEM", "GC_KPP_EUNSUPPORTED"):
        assert getattr(capi, name) == vals[name], name
    assert (capi.MEM_HOST, capi.MEM_DEVICE) == (vals["GC_KPP_MEM_HOST"], vals["GC_KPP_MEM_DEVICE"])
    opts = {k[len("GC_KPP_OPT_"):]: v for k, v in vals.items() if k.startswith("GC_KPP_OPT_")}
    assert len(set(opts.values())) == len(opts)  # distinct keys
    for k, v in opts.items():
        assert getattr(capi, "OPT_" + k) == v, k
