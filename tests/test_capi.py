"""CPU checks of the drop-in boundary: the library loads, exports every symbol
the header declares, and the host-side mirror validates controls like the
reference C API (no GPU call is made here)."""
import re
from pathlib import Path

import numpy as np
import pytest

import mvkit_gb300 as mg
from mvkit_gb300 import ncc

HEADER = Path(__file__).resolve().parents[1] / "include" / "mvkit_gb300_ncc.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"MVG_API\s+[\w\s\*]+?\b(mvg_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_symbols()
    for n in ("mvg_create_ncc_model", "mvg_find_ncc_model", "mvg_get_ncc_model_params", "mvg_clear_ncc_model",
              "mvg_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = mg.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_last_error_is_empty_initially():
    assert mg.load().mvg_last_error() in (b"",) or isinstance(mg.load().mvg_last_error(), bytes)


@pytest.mark.parametrize("kwargs,status", [
    (dict(num_levels="many"), -1),
    (dict(num_levels=17), -1),
    (dict(num_levels=2.5), -1),
    (dict(angle_step=0.5), -1),
    (dict(angle_step="fine"), -1),
    (dict(metric="use_polarityx"), -1),
    (dict(metric=3), -3),
    (dict(num_levels=[3, 4]), -1),
])
def test_create_controls_rejected_like_reference(kwargs, status):
    t = np.zeros((16, 16), np.uint8)
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(t, **kwargs)
    assert e.value.status == status


def test_create_rejects_non_gray_types():
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(np.zeros((16, 16), np.float32))
    assert e.value.status == -3
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(np.zeros((16, 16, 3), np.uint8))
    assert e.value.status == -3


@pytest.mark.parametrize("over,status", [
    (dict(min_score=1.5), -1),
    (dict(min_score=-0.1), -1),
    (dict(max_overlap=2.0), -1),
    (dict(angle_extent=-0.1), -1),
    (dict(angle_extent=7.0), -1),
    (dict(num_matches=-1), -1),
    (dict(num_matches=1.5), -1),
    (dict(subpixel=True), -3),
    (dict(subpixel="yes"), -1),
    (dict(num_levels=[1, 2, 3]), -1),
    (dict(num_levels=-1), -1),
    (dict(min_score=[0.5, 0.6]), -1),
])
def test_find_controls_rejected_like_reference(over, status):
    ctl = dict(angle_start=0.0, angle_extent=0.0, min_score=0.5, num_matches=1, max_overlap=0.5,
               subpixel="true", num_levels=0)
    ctl.update(over)
    with pytest.raises(mg.MvError) as e:
        ncc._find_controls("find_ncc_model", **ctl)
    assert e.value.status == status


def test_find_controls_accept_level_pair():
    r = ncc._find_controls("find_ncc_model", 0.0, 0.1, 0.7, 0, 0.5, "false", [3, 2])
    assert r == (0.0, 0.1, 0.7, 0, 0.5, 0, 3, 2)


def test_noalloc_pyramid_refuses_misaligned_and_host_pointers_without_launching():
    """The no-allocation pyramid checks its pointers on the host: misaligned
    pointers are refused before any CUDA call, host memory before any launch
    (here, without a GPU, the pointer query itself fails)."""
    import ctypes as C
    lib = mg.load()
    f = lib.mvg_ncc_pyramid_level_noalloc
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                  C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]
    f.restype = C.c_int32
    img = np.zeros(64 * 64 + 8, np.uint16)
    out = np.zeros(64 * 64 + 4, np.float32)
    ow, oh = C.c_int64(), C.c_int64()
    base, obase = img.ctypes.data, out.ctypes.data
    assert f(base + 1, 1, 64, 64, 128, 1, obase, 64 * 64, C.byref(ow), C.byref(oh), None) == -1
    assert b"aligned" in lib.mvg_last_error()
    assert f(base, 1, 64, 64, 128, 1, obase + 2, 64 * 64, C.byref(ow), C.byref(oh), None) == -1
    assert b"aligned" in lib.mvg_last_error()
    assert f(base, 0, 64, 600000, 64, 0, obase, 64 * 64, C.byref(ow), C.byref(oh), None) == -103
    st = f(base, 1, 64, 64, 128, 1, obase, 64 * 64, C.byref(ow), C.byref(oh), None)
    assert st in (-1, -1000) and lib.mvg_last_error()


def test_launch_shape_settings_checked():
    """The tensor-core weight lookahead is a launch-shape setting: values out
    of range are refused with InvalidArgument (-1), values in range are taken
    (no device needed)."""
    for bad in (0, 65, -3):
        with pytest.raises(mg.MvError) as e:
            ncc.set_tc_weight_lookahead(bad)
        assert e.value.status == -1
    for good in (1, 8, 24, 64):
        ncc.set_tc_weight_lookahead(good)
    ncc.set_tc_weight_lookahead(8)
