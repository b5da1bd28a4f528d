"""CreateNccModel's errors without a GPU (host build).  Errors of the model
build (mv::ncc_matching::create, src/ncc_matching/model.cpp) give the same
status and message as the oracle and, where its build exists, the compiled
reference.  The operator-level checks give mv_create_ncc_model's own
messages (src/c_api/ncc_matching_api.cpp:46-54; finite numbers,
src/c_api/tuple_input.cpp:99)."""
from __future__ import annotations

import math

import numpy as np
import pytest

import mvkit_gb300 as mg
import oracle_lib
from mvkit_gb300 import ncc

RNG = np.random.default_rng(1)
GOOD = RNG.integers(0, 255, (32, 32)).astype(np.uint8)
BUILD = {
    "flat": (np.full((32, 32), 9, np.uint8), dict(levels=2)),
    "degenerate_rotation": (np.array([[10, 200], [30, 90]], np.uint8), dict(levels=1, angle_extent=1.0)),
    "too_many_levels": (GOOD, dict(levels=9)),
    "negative_extent": (GOOD, dict(levels=2, angle_extent=-0.1)),
    "extent_over_2pi": (GOOD, dict(levels=2, angle_extent=7.0)),
    "empty_domain": (GOOD, dict(levels=2, mask=np.zeros((32, 32), np.uint8))),
    "small_domain": (GOOD, dict(levels=2, mask=np.pad(np.ones((2, 2), np.uint8), 15))),
    "one_row": (RNG.integers(0, 255, (1, 64)).astype(np.uint8), dict(levels=1)),
    "raster_budget": ((np.arange(700 * 700) % 251).astype(np.uint8).reshape(700, 700),
                      dict(levels=1, angle_start=-math.pi, angle_extent=2 * math.pi, angle_step=0.01)),
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


def ours(t, kw):
    lv, st = kw.get("levels", 0), kw.get("angle_step", 0.0)
    try:
        mg.create_ncc_model(t, lv or "auto", kw.get("angle_start", 0.0), kw.get("angle_extent", 0.0), st or "auto",
                            "use_polarity", domain=kw.get("mask"))
        return 0, ""
    except mg.MvError as e:
        return e.status, e.message


def theirs(chk, t, kw):
    try:
        chk.create(t, levels=kw.get("levels", 0), angle_start=kw.get("angle_start", 0.0),
                   angle_extent=kw.get("angle_extent", 0.0), angle_step=kw.get("angle_step", 0.0),
                   mask=kw.get("mask"))
        return 0, ""
    except oracle_lib.CheckerError as e:
        return e.status, e.message


@pytest.mark.parametrize("name", sorted(BUILD))
def test_build_errors_equal_reference(host_build, name):
    t, kw = BUILD[name]
    got = ours(t, kw)
    assert got == theirs(oracle_lib.oracle(), t, kw)
    ref = oracle_lib.reference("scalar")
    if ref is not None:
        assert got == theirs(ref, t, kw)


@pytest.mark.parametrize("kw,message", [
    (dict(levels=17), "levels must be 0..16 or auto"),
    (dict(levels=2, angle_extent=1.0, angle_step=0.5), "angle step must be in [0,pi/16] or auto"),
    (dict(levels=2, angle_start=float("nan")), "finite control value required"),
])
def test_operator_checks(host_build, kw, message):
    assert ours(GOOD, kw) == (ncc.MV_STATUS_INVALID_ARGUMENT, message)
