"""CreateNccModel's rotated rasters (src/ncc_matching/model.cpp:39-242: every
level, every trained angle, plus the unrotated level-0 raster): sample rows,
columns, FP64 weights, weight sums, angles and origins equal the oracle's
bit for bit, and the compiled reference's where its build exists.  The host
build runs without a GPU (mvg_ncc_model_raster reads the model's host
rasters)."""
from __future__ import annotations

import math

import numpy as np
import pytest

import mvkit_gb300 as mg
import oracle_lib
from mvkit_gb300 import ncc

D = math.radians


def disc(h, w):
    y, x = np.mgrid[:h, :w]
    return ((y - (h - 1) / 2) ** 2 + (x - (w - 1) / 2) ** 2 <= (min(h, w) / 2 - 1) ** 2).astype(np.uint8)


def template(seed, shape, dtype, maxval):
    rng = np.random.default_rng(seed)
    base = rng.integers(0, maxval, size=(shape[0] // 4 + 2, shape[1] // 4 + 2))
    t = np.kron(base, np.ones((4, 4), dtype=np.int64))[: shape[0], : shape[1]]
    t = t + rng.integers(0, max(2, maxval // 16), size=shape)
    return np.clip(t, 0, maxval).astype(dtype)


CASES = {
    "u8_rot": dict(t=(1, (40, 44), np.uint8, 255), levels=3, a0=-0.3, ext=0.6, step=0.0),
    "u8_step": dict(t=(2, (33, 27), np.uint8, 255), levels=2, a0=D(-15), ext=D(30), step=0.04),
    "u8_auto_levels": dict(t=(3, (64, 64), np.uint8, 255), levels=0, a0=D(-10), ext=D(20), step=0.0),
    "u8_one_angle": dict(t=(4, (30, 50), np.uint8, 255), levels=2, a0=0.0, ext=0.0, step=0.0),
    "u16_12bit": dict(t=(5, (36, 36), np.uint16, 4095), levels=3, a0=D(-45), ext=D(90), step=0.0),
    "masked": dict(t=(6, (48, 48), np.uint8, 255), levels=3, a0=-0.2, ext=0.4, step=0.0, mask=True),
    "polarity": dict(t=(7, (32, 40), np.uint8, 255), levels=2, a0=-0.25, ext=0.5, step=0.0, ignore=True),
    "full_circle": dict(t=(8, (24, 24), np.uint8, 255), levels=2, a0=-math.pi, ext=2 * math.pi, step=0.0),
}


@pytest.fixture(scope="module")
def host_build():
    try:
        mg.load()
    except mg.MvError as e:
        pytest.skip(str(e))
    mg.ncc.set_model_build("host")
    yield
    mg.ncc.set_model_build("device")


def same(a, b, label):
    for k in ("angle", "origin_row", "origin_column", "weight_sum"):
        assert a[k] == b[k], f"{label}: {k} {a[k]!r} vs {b[k]!r}"
    for k in ("rows", "cols", "weights"):
        assert np.array_equal(a[k], b[k]), f"{label}: {k} differ"


@pytest.mark.parametrize("name", sorted(CASES))
def test_rasters_equal_oracle_and_reference(host_build, name):
    c = CASES[name]
    t = template(*c["t"])
    mask = disc(*t.shape) if c.get("mask") else None
    model = mg.create_ncc_model(t, c["levels"] or "auto", c["a0"], c["ext"], c["step"] or "auto",
                                "ignore_global_polarity" if c.get("ignore") else "use_polarity", domain=mask)
    checkers = [oracle_lib.oracle()]
    ref = oracle_lib.reference("scalar")
    if ref is not None:
        checkers.append(ref)
    levels = mg.get_ncc_model_params(model)[0]
    for chk in checkers:
        om = chk.create(t, levels=c["levels"], angle_start=c["a0"], angle_extent=c["ext"], angle_step=c["step"],
                        ignore_polarity=c.get("ignore", False), mask=mask)
        info = om.info()
        assert info["levels"] == levels
        # the operator reports step 0 for a model without angle range
        # (src/c_api/ncc_matching_api.cpp:85-96)
        step = mg.get_ncc_model_params(model)[3]
        assert step == (info["angle_step"] if c["ext"] != 0 else 0.0)
        same(ncc.ncc_model_raster(model, -1), om.patch(-1, 0), f"{name} original")
        per_level = info["patches"]  # one raster per trained angle on every level
        for lv in range(levels):
            for k in range(per_level):
                same(ncc.ncc_model_raster(model, lv, k), om.patch(lv, k), f"{name} level {lv} raster {k}")
            with pytest.raises(mg.MvError):
                ncc.ncc_model_raster(model, lv, per_level)
    with pytest.raises(mg.MvError) as e:
        ncc.ncc_model_raster(model, levels, 0)
    assert e.value.status == ncc.MV_STATUS_INVALID_ARGUMENT


def test_extended_sample_budget(host_build):
    """A 160^2 template over a full circle needs more than the reference's 16
    million raster samples: refused (LimitExceeded, as by the reference) under
    the default budget; under a raised budget every raster equals the
    oracle's with the same budget, bit for bit.  The model keeps its budget."""
    t = template(9, (160, 160), np.uint8, 255)
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(t, 4, -math.pi, 2 * math.pi, "auto", "use_polarity")
    assert e.value.status == -103 and "raster budget" in e.value.message
    orc = oracle_lib.oracle()
    with pytest.raises(oracle_lib.CheckerError) as oe:
        orc.create(t, levels=4, angle_start=-math.pi, angle_extent=2 * math.pi)
    assert oe.value.status == -103
    with mg.extended_budgets(samples=100_000_000):
        model = mg.create_ncc_model(t, 4, -math.pi, 2 * math.pi, "auto", "use_polarity")
    assert mg.get_budgets()["samples"] == 16_000_000
    oracle_lib.set_oracle_budgets(samples=100_000_000)
    try:
        om = orc.create(t, levels=4, angle_start=-math.pi, angle_extent=2 * math.pi)
    finally:
        oracle_lib.set_oracle_budgets()
    info = om.info()
    total = 0
    for lv in range(4):
        for k in range(info["patches"]):
            a = ncc.ncc_model_raster(model, lv, k)
            same(a, om.patch(lv, k), f"extended level {lv} raster {k}")
            total += len(a["rows"])
    assert total > 16_000_000


def test_budget_arguments():
    with pytest.raises(mg.MvError) as e:
        mg.set_budgets(candidates=1 << 22)
    assert e.value.status == -1
    with mg.extended_budgets(samples=5, pixels=7, candidates=11):
        assert mg.get_budgets() == {"samples": 5, "pixels": 7, "candidates": 11}
    assert mg.get_budgets() == {"samples": 16_000_000, "pixels": 32_000_000, "candidates": 10_000}
