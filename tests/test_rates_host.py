"""The product's Update_RCONST (the generated straight-line rate code of
rates_direct_kernel with the GPU rate laws of rate_laws.cuh and
het_rates.cuh), built for the host with g++ on glibc's libm, against the
oracle's restatement (oracle/rate_laws.h, oracle/het_laws.h and the
generated kpp_rates_oracle.c): the same arithmetic gives the same rates bit
for bit, gas phase and heterogeneous, so the only GPU/oracle differences
left are those of CUDA's exp/log10/pow (bounded in the GPU tests)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "geos-chem_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    import gcchem.rates_program as rp
    from gcchem.mechanism import load_ir

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    tmp = tmp_path_factory.mktemp("rates_host")
    gen = tmp / "gen"
    rp.write_generated(str(gen), load_ir())
    (tmp / "fake").mkdir()
    (tmp / "fake" / "cuda_runtime.h").write_text("#pragma once\ntypedef int cudaError_t;\ntypedef void* cudaStream_t;\n")
    exe = str(tmp / "rates")
    subprocess.check_call([gxx, "-O1", "-std=c++17", "-ffp-contract=off", "-I", str(tmp / "fake"), "-I", CSRC,
                           "-I", str(gen), os.path.join(ROOT, "tests", "host", "rates_direct_host.cpp"), "-o", exe])
    prog = rp.build_program(load_ir())
    for name, key in (("hsind", "hs_ind"), ("hsmw", "hs_mw"), ("hssr", "hs_srmw"), ("hsk0", "hs_hk0"),
                      ("hscr", "hs_hcr")):
        np.array(prog[key], np.float64).tofile(str(tmp / (name + ".bin")))
    return tmp, exe


def _run(harness, cells, het):
    tmp, exe = harness
    n = cells["c"].shape[1]
    for name, arr in (("met", cells["met"]), ("photol", cells["photol"]), ("c", cells["c"])):
        np.ascontiguousarray(arr, np.float64).tofile(str(tmp / (name + ".bin")))
    if het is not None:
        np.ascontiguousarray(het, np.float64).tofile(str(tmp / "het.bin"))
    subprocess.check_call([exe, str(n), str(cells["c"].shape[0]), "1058", "1" if het is not None else "0"],
                          cwd=str(tmp))
    return np.fromfile(str(tmp / "out.bin")).reshape(1058, n)


@pytest.mark.parametrize("with_het", [False, True])
def test_product_rates_equal_oracle_on_the_same_libm(harness, with_het):
    import gcchem.hetstate as hs
    import gcchem.inputs as inputs
    import oracle

    cells = inputs.box_cells(512, seed=13)
    # nonzero K_MT/K_CLD and SRHOCl/SRHOBr rows, so that every rate reads a real input
    rng = np.random.default_rng(14)
    cells["met"][4:18] = rng.uniform(0.0, 1e-3, (14, 512))
    het = hs.het_cells(512, seed=15) if with_het else None
    got = _run(harness, cells, het)
    ref = oracle.update_rconst(cells["met"], cells["photol"], cells["c"], het=het)
    bad = np.nonzero(~((got == ref) | (np.isnan(got) & np.isnan(ref))))
    assert bad[0].size == 0, (bad[0][:5], got[bad][:5], ref[bad][:5])
