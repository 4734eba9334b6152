"""gc_kpp_copy_rows: the row copies that stage host-memory calls.  Page-locked
host memory is read and written by the SMs (16-, 8- or 4-byte accesses by
the alignment of pointers, pitches and width); pageable memory goes through
cudaMemcpy2DAsync.  Every form must equal a plain copy byte for byte and
leave the padding of pitched rows untouched."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,width,pad", [("float64", 4096, 0), ("float64", 1001, 3), ("int32", 777, 5),
                                             ("int32", 1024, 4), ("float64", 1, 0)])
@pytest.mark.parametrize("host", ["pinned", "pageable"])
def test_copy_rows_round_trip(dtype, width, pad, host):
    import torch
    import gcchem.capi as capi

    tdt = getattr(torch, dtype)
    rows = 37
    g = torch.Generator().manual_seed(width + pad)
    src = (torch.rand((rows, width + pad), generator=g, dtype=torch.float64) * 1e6).to(tdt)
    if host == "pinned":
        src = src.pin_memory()
    dev = torch.full((rows, width + 2 * pad + 2), -1, dtype=tdt, device="cuda")
    capi.copy_rows(dev[:, :width], src[:, :width])
    back = torch.full((rows, width + pad), -7, dtype=tdt)
    if host == "pinned":
        back = back.pin_memory()
    capi.copy_rows(back[:, :width], dev[:, :width])
    torch.cuda.synchronize()
    assert torch.equal(dev[:, :width].cpu(), src[:, :width])
    assert torch.all(dev[:, width:].cpu() == -1)
    assert torch.equal(back[:, :width], src[:, :width])
    assert torch.all(back[:, width:] == -7)


def test_copy_rows_rejects_bad_shapes():
    import ctypes
    import torch
    import gcchem.capi as capi

    lib = capi.load_library()
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = lib.gc_kpp_copy_rows(ctypes.c_void_p(a.data_ptr()), 8, ctypes.c_void_p(a.data_ptr()), 8, 16, 1, None)
    assert rc == capi.GC_KPP_EINVAL  # width above the pitch
    rc = lib.gc_kpp_copy_rows(None, 8, ctypes.c_void_p(a.data_ptr()), 8, 8, 1, None)
    assert rc == capi.GC_KPP_EINVAL


def test_photol_rows_of_the_mechanism():
    import gcchem.capi as capi
    import gcchem.stream as stream

    mask = capi.photol_rows()
    runs = stream.photol_runs()
    want = np.zeros(200, bool)
    for a, b in runs:
        want[a:b] = True
    assert np.array_equal(mask, want) and mask.sum() == 168


def test_copy_rows_other_layouts_fall_back_to_torch():
    import torch
    import gcchem.capi as capi

    src = torch.arange(3 * 50, dtype=torch.float64).reshape(50, 3).pin_memory().t()  # column-major [3, 50]
    assert src.stride(1) != 1
    dev = torch.empty((3, 50), dtype=torch.float64, device="cuda")
    capi.copy_rows(dev, src)
    torch.cuda.synchronize()
    assert torch.equal(dev.cpu(), src)
