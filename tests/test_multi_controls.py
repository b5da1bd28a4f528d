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


def batch(models, images, workers=2, **over):
    c = dict(OK)
    c.update(over)
    return mg.find_ncc_models_batch(images, models, c["angle_start"], c["angle_extent"], c["min_score"],
                                    c["num_matches"], c["max_overlap"], c["subpixel"], c["num_levels"],
                                    workers=workers)


@pytest.mark.parametrize("over,status", [
    (dict(num_matches=[1, 2]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(angle_extent=[7.0]), ncc.MV_STATUS_INVALID_ARGUMENT),
    (dict(subpixel=[1]), ncc.MV_STATUS_TYPE_MISMATCH),
    (dict(num_levels=[2, 1, 2, 1]), ncc.MV_STATUS_INVALID_ARGUMENT),
])
def test_batch_control_errors(models, over, status):
    """The batched operator checks the FindNccModels controls the same way."""
    with pytest.raises(mg.MvError) as e:
        batch(models, [IMG, IMG], **over)
    assert e.value.status == status


def c_batch(models, n_images, workers, n_matches_values=1):
    """mvg_find_ncc_models_batch called directly (the C side's own checks)."""
    import ctypes as C
    _, ids, arrs, _ = ncc._models_controls("t", models, OK["angle_start"], OK["angle_extent"], OK["min_score"],
                                           OK["num_matches"], OK["max_overlap"], OK["subpixel"], OK["num_levels"])
    arrs = list(arrs)
    arrs[3] = np.zeros(n_matches_values, dtype=np.int64)
    args = []
    for a in arrs:
        args += [a.ctypes.data, len(a)]
    imgs = (C.c_void_p * max(1, n_images))(*([IMG.ctypes.data] * n_images))
    types = np.zeros(max(1, n_images), np.int32)
    dims = np.full(max(1, n_images), 64, np.int64)
    out = [np.zeros(8) for _ in range(4)] + [np.zeros(8, np.int64)]
    offsets = np.full(n_images + 1, -1, np.int64)
    statuses = np.full(max(1, n_images), 7, np.int32)
    cnt = C.c_int64(-1)
    st = mg.load().mvg_find_ncc_models_batch(imgs, types.ctypes.data, dims.ctypes.data, dims.ctypes.data,
                                             dims.ctypes.data, n_images, 0, None, ids, len(models), *args, workers,
                                             *[o.ctypes.data for o in out], 8, offsets.ctypes.data,
                                             statuses.ctypes.data, C.byref(cnt))
    return st, cnt.value, offsets


def test_batch_c_entry_checks(models):
    """An empty batch succeeds with no matches; a worker count outside 1..256
    and a control cardinality that fits neither one nor every model are
    InvalidArgument, before any device work."""
    st, cnt, offsets = c_batch(models, 0, 4)
    assert st == 0 and cnt == 0 and offsets[0] == 0
    for workers in (0, 257):
        st, cnt, _ = c_batch(models, 2, workers)
        assert st == ncc.MV_STATUS_INVALID_ARGUMENT and cnt == 0
        assert b"workers" in mg.load().mvg_last_error()
    st, _, _ = c_batch(models, 2, 4, n_matches_values=2)
    assert st == ncc.MV_STATUS_INVALID_ARGUMENT
    assert b"NumMatches" in mg.load().mvg_last_error()


def test_batch_python_checks(models):
    with pytest.raises(mg.MvError) as e:
        batch(models, [IMG], workers=0)
    assert e.value.status == ncc.MV_STATUS_INVALID_ARGUMENT
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_models_batch([IMG], models, *[OK[k] for k in ("angle_start", "angle_extent", "min_score",
                                                                   "num_matches", "max_overlap", "subpixel",
                                                                   "num_levels")], domains=[None, None])
    assert e.value.status == ncc.MV_STATUS_INVALID_ARGUMENT
    assert batch(models, []) == []
