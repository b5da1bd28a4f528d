"""FindNccModels control checks (NccControls and ncc_models,
src/c_api/ncc_matching_api.cpp:112-162): cardinalities and ranges are
rejected with the reference's statuses before any device work, so these run
without a GPU."""
from __future__ import annotations

import numpy as np
import pytest

import mvkit_gb300 as mg
from mvkit_gb300 import ncc


@pytest.fixture(scope="module")
def models():
    try:
        mg.load()
    except mg.MvError as e:
        pytest.skip(str(e))
    rng = np.random.default_rng(3)
    return [mg.create_ncc_model(rng.integers(0, 255, (20, 20), dtype=np.uint8), 2, -0.2, 0.4, "auto",
                                "use_polarity") for _ in range(3)]


IMG = np.zeros((64, 64), np.uint8)
OK = dict(angle_start=[-0.2], angle_extent=[0.4], min_score=[0.7], num_matches=[0], max_overlap=[0.5],
          subpixel=["true"], num_levels=[2])


def call(models, **over):
    c = dict(OK)
    c.update(over)
    return mg.find_ncc_models(IMG, models, c["angle_start"], c["angle_extent"], c["min_score"], c["num_matches"],
                              c["max_overlap"], c["subpixel"], c["num_levels"])


@pytest.mark.parametrize("over,status", [
    (dict(num_matches=[1, 2]), ncc.MV_STATUS_INVALID_ARGUMENT),          # neither 1 nor 3 values
    (dict(angle_start=[0.0, 0.1]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(num_levels=[2, 1, 2, 1]), ncc.MV_STATUS_INVALID_ARGUMENT),     # 4 is not 1, 2, 3 or 6
    (dict(angle_extent=[7.0]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(min_score=[0.5, 1.5, 0.5]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(max_overlap=[-0.1]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(num_matches=[-1]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(subpixel=["yes"]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(subpixel=[1]), ncc.MV_STATUS_TYPE_MISMATCH),
    (dict(num_levels=[-1]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(min_score=["a"]), ncc.MV_STATUS_TYPE_MISMATCH),
])
def test_control_errors(models, over, status):
    with pytest.raises(mg.MvError) as e:
        call(models, **over)
    assert e.value.status == status


def test_model_list_errors(models):
    with pytest.raises(mg.MvError) as e:
        call([])
    assert e.value.status == ncc.MV_STATUS_INVALID_ARGUMENT
    with pytest.raises(mg.MvError) as e:
        call([models[0], "x"])
    assert e.value.status == ncc.MV_STATUS_TYPE_MISMATCH


def test_c_abi_cardinality(models):
    """The C entry checks the same rules on raw arrays (ctypes caller)."""
    import ctypes as C
    lib = mg.load()
    ids = (C.c_void_p * 3)(*[m.handle for m in models])
    d = np.array([0.5, 0.5], dtype=np.float64)
    one = np.array([0.5], dtype=np.float64)
    q = np.array([0], dtype=np.int64)
    sp = np.array([1], dtype=np.int32)
    lv = np.array([2], dtype=np.int32)
    cnt = C.c_int64()
    st = lib.mvg_find_ncc_models(IMG.ctypes.data, 0, 64, 64, 64, 0, None, ids, 3, one.ctypes.data, 1, one.ctypes.data, 1,
                                 one.ctypes.data, 1, q.ctypes.data, 1, d.ctypes.data, 2, sp.ctypes.data, 1,
                                 lv.ctypes.data, 1, None, None, None, None, None, 0, C.byref(cnt), None)
    assert st == ncc.MV_STATUS_INVALID_ARGUMENT
    st = lib.mvg_find_ncc_models(IMG.ctypes.data, 0, 64, 64, 64, 0, None, ids, 4097, one.ctypes.data, 1, one.ctypes.data,
                                 1, one.ctypes.data, 1, q.ctypes.data, 1, one.ctypes.data, 1, sp.ctypes.data, 1,
                                 lv.ctypes.data, 1, None, None, None, None, None, 0, C.byref(cnt), None)
    assert st == ncc.MV_STATUS_INVALID_ARGUMENT
