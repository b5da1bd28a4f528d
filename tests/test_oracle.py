"""The oracle restatement against the golden vectors of the reference, the
scene generator's determinism, and (where the reference was compiled in this
container) the oracle against the reference on fresh seeds."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from golden.cases import CASES, LARGE, make_inputs, search_domain

GOLDEN = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())["cases"]


@pytest.fixture(scope="module")
def orc():
    return oracle_lib.oracle()


def run(checker, case, wl, mask, **over):
    c = case["create"]
    model = checker.create(wl.template, levels=c["levels"], angle_start=c["angle_start"],
                           angle_extent=c["angle_extent"], angle_step=c.get("angle_step", 0.0),
                           ignore_polarity=c.get("ignore_polarity", False), mask=mask)
    f = dict(case["find"])
    f.update(over)
    return model, checker.find(model, wl.image, f["angle_start"], f["angle_extent"], f["min_score"],
                               f["num_matches"], f["max_overlap"], f["subpixel"], f["highest"], f["lowest"],
                               domain=search_domain(case, wl))


@pytest.mark.parametrize("name", sorted(CASES))
def test_generator_digest(name):
    wl, _ = make_inputs(CASES[name])
    assert wl.digest() == GOLDEN[name]["digest"], "scene generator drifted from the golden inputs"


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(orc, name):
    """Bit-exact: the restatement follows the reference's FP64 expression order;
    where the reference rejects the search, the oracle returns the same status."""
    wl, mask = make_inputs(CASES[name])
    if "status" in GOLDEN[name]:
        with pytest.raises(oracle_lib.CheckerError) as err:
            run(orc, CASES[name], wl, mask)
        assert err.value.status == GOLDEN[name]["status"]
        return
    model, res = run(orc, CASES[name], wl, mask)
    ref = np.array(GOLDEN[name]["matches"]).reshape(-1, 4)
    assert res.shape == ref.shape
    np.testing.assert_array_equal(res, ref)
    assert model.info()["levels"] == GOLDEN[name]["levels"]
    assert model.info()["angle_step"] == GOLDEN[name]["angle_step"]


@pytest.mark.slow
@pytest.mark.parametrize("name", list(LARGE))
def test_oracle_matches_reference_golden_large(orc, name):
    case = LARGE[name]
    wl, mask = make_inputs(case)
    assert wl.digest() == GOLDEN[name]["digest"]
    _, res = run(orc, case, wl, mask)
    np.testing.assert_array_equal(res, np.array(GOLDEN[name]["matches"]).reshape(-1, 4))


def test_avx2_reference_agrees_with_scalar_within_fp64_noise():
    """The reference's own two builds differ only in FP64 rounding order."""
    for name, g in GOLDEN.items():
        if "matches_avx2" not in g or "status" in g:
            continue
        a, b = np.array(g["matches"]).reshape(-1, 4), np.array(g["matches_avx2"]).reshape(-1, 4)
        assert a.shape == b.shape, name
        assert np.abs(a - b).max(initial=0) < 1e-9, name


def test_golden_matches_near_ground_truth():
    """Sanity of the fixtures: each pasted pose is found within a pixel."""
    for name in ("cfg1_s1", "cfg1_s2", "cfg1_s3", "rot_l4_2", "cfg2_s1"):
        g = GOLDEN[name]
        m = np.array(g["matches"]).reshape(-1, 4)
        for t in g["truth"]:
            d = np.hypot(m[:, 0] - t[0], m[:, 1] - t[1])
            i = int(np.argmin(d))
            assert d[i] < 1.0, name
            assert abs(m[i, 2] - t[2]) < math.radians(0.5), name


def test_oracle_pyramid_is_exact_integer_sums(orc):
    """Level k of the matcher pyramid is (sum of 4^k pixels)/4^k - dc exactly."""
    wl, _ = make_inputs(CASES["rot_l4_2"])
    model = orc.create(wl.template, levels=4, angle_start=-0.3, angle_extent=0.6)
    img = wl.image.astype(np.int64)
    for level in range(4):
        lev, geom = orc.pyramid(model, wl.image, 4, level)
        h, w = lev.shape
        k = 1 << level
        sums = img[: h * k, : w * k].reshape(h, k, w, k).sum(axis=(1, 3))
        np.testing.assert_array_equal(lev, sums / float(k * k) - geom[4])


def test_oracle_rejects_like_reference(orc):
    wl, _ = make_inputs(CASES["cfg1_s1"])
    with pytest.raises(oracle_lib.CheckerError) as e:
        orc.create(wl.template, levels=9)
    assert e.value.status == -1
    with pytest.raises(oracle_lib.CheckerError) as e:
        orc.create(np.full((32, 32), 7, np.uint8))
    assert e.value.status == -1
    model = orc.create(wl.template, levels=3)
    with pytest.raises(oracle_lib.CheckerError) as e:
        orc.find(model, wl.image, 0.0, 0.0, 1.5, 1, 0.5)
    assert e.value.status == -1
    big = np.zeros((8001, 4001), np.uint8)
    with pytest.raises(oracle_lib.CheckerError) as e:
        orc.find(model, big, 0.0, 0.0, 0.5, 1, 0.5)
    assert e.value.status == -103


@pytest.mark.skipif(oracle_lib.reference("scalar") is None, reason="reference not compiled in this container")
@pytest.mark.parametrize("seed", [101, 102, 103, 104])
def test_oracle_matches_reference_fresh_seeds(orc, seed):
    ref = oracle_lib.reference("scalar")
    case = dict(gen=dict(seed=seed, height=360, width=480, tsize=48, n_poses=2,
                         angle_range=(-math.radians(15), math.radians(15))),
                create=dict(levels=3, angle_start=-math.radians(15), angle_extent=math.radians(30)),
                find=dict(angle_start=-math.radians(15), angle_extent=math.radians(30), min_score=0.6,
                          num_matches=0, max_overlap=0.5, subpixel=True, highest=3, lowest=1))
    wl, mask = make_inputs(case)
    _, a = run(orc, case, wl, mask)
    _, b = run(ref, case, wl, mask)
    np.testing.assert_array_equal(a, b)
