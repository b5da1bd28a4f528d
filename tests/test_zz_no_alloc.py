"""The no-allocation pyramid entry point, for callers that cannot allocate
device memory (frameworks owning every device buffer, real-time loops,
fixed memory budgets).  It must give exactly the levels of the allocating
entry point, call after call, although every call reuses one fixed device
array.  Collected last so that a run stopping at the first failure has
already run every other test.  Device buffers here come from torch: the
caller owns input and output memory, the entry point allocates nothing."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    lib = mvkit_gb300.load()
    f = lib.mvg_ncc_pyramid_level_noalloc
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                  C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]
    f.restype = C.c_int32
    return lib


def noalloc_level(lib, image: np.ndarray, level: int) -> np.ndarray:
    import torch
    src = torch.from_numpy(np.ascontiguousarray(image)).cuda()
    h, w = image.shape
    for _ in range(level):
        w, h = max(1, w // 2), max(1, h // 2)
    out = torch.full((h, w), -1.0, dtype=torch.float32, device="cuda")
    ow, oh = C.c_int64(), C.c_int64()
    torch.cuda.synchronize()
    st = lib.mvg_ncc_pyramid_level_noalloc(src.data_ptr(), 1 if image.dtype == np.uint16 else 0, image.shape[1],
                                           image.shape[0], image.strides[0], level, out.data_ptr(), out.numel(),
                                           C.byref(ow), C.byref(oh), None)
    assert st == 0, lib.mvg_last_error()
    assert (ow.value, oh.value) == (w, h)
    return out.cpu().numpy()


def allocating_level(image: np.ndarray, level: int, tsize: int, levels: int) -> np.ndarray:
    import mvkit_gb300 as mg
    from mvkit_gb300 import workloads as W
    tmpl = W.make_workload(5, 4 * tsize, 4 * tsize, tsize, 1, maxval=4095 if image.dtype == np.uint16 else 255).template
    model = mg.create_ncc_model(tmpl, levels, 0.0, 0.0, "auto", "use_polarity")
    lev, _ = mg.pyramid_level(image, model, levels, level)
    return lev


def test_two_calls_in_a_row_match_the_allocating_entry_point(lib):
    from mvkit_gb300 import workloads as W
    a = W.make_workload(41, 600, 800, 64, 2, angle_range=(-math.radians(10), math.radians(10))).image
    b = W.make_workload(42, 517, 389, 48, 1, maxval=4095, noise_sigma=20).image  # odd sizes, uint16
    got_a = noalloc_level(lib, a, 3)
    got_b = noalloc_level(lib, b, 2)
    np.testing.assert_array_equal(got_a, allocating_level(a, 3, 64, 4))
    np.testing.assert_array_equal(got_b, allocating_level(b, 2, 48, 3))
    # the shared scratch keeps the previous call's levels; a repeat still matches
    np.testing.assert_array_equal(noalloc_level(lib, a, 3), got_a)


def test_rejects_images_beyond_the_fixed_scratch(lib):
    import torch
    big = torch.zeros((4096, 4096), dtype=torch.uint8, device="cuda")
    out = torch.zeros(512 * 512, dtype=torch.float32, device="cuda")
    ow, oh = C.c_int64(), C.c_int64()
    st = lib.mvg_ncc_pyramid_level_noalloc(big.data_ptr(), 0, 4096, 4096, 4096, 3, out.data_ptr(), out.numel(),
                                           C.byref(ow), C.byref(oh), None)
    assert st == -103
    assert b"scratch" in lib.mvg_last_error()
