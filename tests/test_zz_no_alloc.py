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


def test_level_zero_matches_the_allocating_entry_point(lib):
    # level 0 is written straight into the caller's buffer; the scratch is unused
    from mvkit_gb300 import workloads as W
    a = W.make_workload(43, 300, 413, 48, 1).image
    np.testing.assert_array_equal(noalloc_level(lib, a, 0), allocating_level(a, 0, 48, 3))


def test_lower_levels_that_exactly_fill_the_scratch(lib):
    # 2048 x 3072 bytes: level 0 is exactly the 6 Mi floats of the scratch
    from mvkit_gb300 import workloads as W
    a = W.make_workload(44, 3072, 2048, 64, 1).image
    assert a.shape == (3072, 2048)
    np.testing.assert_array_equal(noalloc_level(lib, a, 1), allocating_level(a, 1, 64, 3))
    # one row more no longer fits
    import torch
    big = torch.zeros((3073, 2048), dtype=torch.uint8, device="cuda")
    out = torch.zeros(1536 * 1024, dtype=torch.float32, device="cuda")
    ow, oh = C.c_int64(), C.c_int64()
    st = lib.mvg_ncc_pyramid_level_noalloc(big.data_ptr(), 0, 2048, 3073, 2048, 1, out.data_ptr(), out.numel(),
                                           C.byref(ow), C.byref(oh), None)
    assert st == -103, lib.mvg_last_error()


def test_inexact_uint16_sums_are_unsupported_on_both_entry_points(lib):
    # 4^5 x 65535 exceeds 2^24: the level-5 sums are not exact in float
    import torch
    import mvkit_gb300 as mg
    from mvkit_gb300 import workloads as W
    img = np.full((256, 256), 65535, np.uint16)
    src = torch.from_numpy(img).cuda()
    out = torch.zeros(64, dtype=torch.float32, device="cuda")
    ow, oh = C.c_int64(), C.c_int64()
    st = lib.mvg_ncc_pyramid_level_noalloc(src.data_ptr(), 1, 256, 256, 512, 5, out.data_ptr(), out.numel(),
                                           C.byref(ow), C.byref(oh), None)
    assert st == -6, lib.mvg_last_error()
    tmpl = W.make_workload(5, 1024, 1024, 256, 1, maxval=4095).template  # 256^2 allows 6 levels
    model = mg.create_ncc_model(tmpl, 6, 0.0, 0.0, "auto", "use_polarity")
    with pytest.raises(mg.MvError) as e:
        mg.pyramid_level(img, model, 6, 5)
    assert e.value.status == -6


def test_host_and_misaligned_pointers_are_refused_before_any_launch(lib):
    import torch
    host = np.zeros((64, 64), np.uint8)
    dev = torch.zeros((64, 64), dtype=torch.uint16, device="cuda")
    out = torch.zeros(64 * 64, dtype=torch.float32, device="cuda")
    host_out = np.zeros(64 * 64, np.float32)
    ow, oh = C.c_int64(), C.c_int64()
    f = lib.mvg_ncc_pyramid_level_noalloc
    assert f(host.ctypes.data, 0, 64, 64, 64, 1, out.data_ptr(), out.numel(), C.byref(ow), C.byref(oh), None) == -1
    assert b"pixels" in lib.mvg_last_error()
    assert f(dev.data_ptr(), 1, 64, 64, 128, 1, host_out.ctypes.data, host_out.size, C.byref(ow), C.byref(oh),
             None) == -1
    assert b"out" in lib.mvg_last_error()
    assert f(dev.data_ptr() + 1, 1, 63, 64, 128, 1, out.data_ptr(), out.numel(), C.byref(ow), C.byref(oh),
             None) == -1
    assert f(dev.data_ptr(), 1, 64, 64, 128, 1, out.data_ptr() + 2, out.numel() - 1, C.byref(ow), C.byref(oh),
             None) == -1


def test_rejects_images_beyond_the_fixed_scratch(lib):
    import torch
    big = torch.zeros((4096, 4096), dtype=torch.uint8, device="cuda")
    out = torch.zeros(512 * 512, dtype=torch.float32, device="cuda")
    ow, oh = C.c_int64(), C.c_int64()
    st = lib.mvg_ncc_pyramid_level_noalloc(big.data_ptr(), 0, 4096, 4096, 4096, 3, out.data_ptr(), out.numel(),
                                           C.byref(ow), C.byref(oh), None)
    assert st == -103
    assert b"scratch" in lib.mvg_last_error()
