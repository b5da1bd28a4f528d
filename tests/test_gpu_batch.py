"""Batched FindNccModels (mvg_find_ncc_models_batch): scenes of uneven size
searched for one model set on the library's host threads, several finds in
flight.  Each image's status and matches equal the reference's find_models
on that image (golden/batch.json; tolerances as test_gpu_parity: same count,
order and model indices, |drow|,|dcol| <= 0.05 px, |dangle| <= 0.05 deg,
|dscore| <= 1e-4) and, bit for bit, the single-image find_ncc_models."""
import json
from pathlib import Path

import numpy as np
import pytest

from golden.batch_cases import BATCH_CASES, make_batch_inputs
from golden.make_batch import template_digest
from test_gpu_parity import assert_same_matches

pytestmark = pytest.mark.gpu

BATCH = json.loads((Path(__file__).parent / "golden" / "batch.json").read_text())["cases"]


@pytest.fixture(scope="module")
def mg():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    mvkit_gb300.load()
    return mvkit_gb300


def batch_models(mg, case, batch):
    c = case["create"]
    return [mg.create_ncc_model(t, c["levels"], c["angle_start"], c["angle_extent"], "auto", "use_polarity")
            for t in batch[0].templates]


def controls(case):
    f = case["find"]
    return (f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"], f["max_overlap"], f["subpixel"],
            f["num_levels"])


@pytest.mark.parametrize("name", sorted(BATCH_CASES))
def test_batch_matches_reference(mg, name):
    case = BATCH_CASES[name]
    batch = make_batch_inputs(case)
    want = BATCH[name]
    assert template_digest(batch[0].templates) == want["templates"]
    assert [wl.digest() for wl in batch] == [w["digest"] for w in want["images"]]
    models = batch_models(mg, case, batch)
    got = mg.find_ncc_models_batch([wl.image for wl in batch], models, *controls(case), workers=4,
                                   raise_errors=False)
    assert len(got) == len(batch)
    for i, (g, w) in enumerate(zip(got, want["images"])):
        label = f"{name} image {i}"
        if w["status"] != 0:
            assert isinstance(g, mg.MvError) and g.status == w["status"], f"{label}: {g} vs status {w['status']}"
            continue
        assert not isinstance(g, mg.MvError), f"{label}: {g}"
        wm = np.array(w["matches"]).reshape(-1, 5)
        assert list(g[4]) == [int(x) for x in wm[:, 4]], f"{label}: model indices {list(g[4])} vs {wm[:, 4]}"
        assert_same_matches(g[:4], wm[:, :4], label)


def test_batch_equals_single_finds(mg):
    """Every image of a batch, host or device memory, one or eight workers,
    with and without a domain: the single-image result, bit for bit."""
    case = BATCH_CASES["batch_uneven"]
    batch = make_batch_inputs(case)
    models = batch_models(mg, case, batch)
    ctl = controls(case)
    images = [wl.image for wl in batch]
    domains = []
    for k, im in enumerate(images):
        d = None
        if k % 2:
            d = np.zeros(im.shape, np.uint8)
            d[:, : im.shape[1] * 2 // 3] = 1
        domains.append(d)
    single = [mg.find_ncc_models(im, models, *ctl, domain=d) for im, d in zip(images, domains)]
    dev = [mg.DeviceImage(im) for im in images]
    for imgs, workers in ((images, 1), (images, 8), (dev, 3)):
        got = mg.find_ncc_models_batch(imgs, models, *ctl, domains=domains, workers=workers)
        for i, (g, s) in enumerate(zip(got, single)):
            assert len(g[0]) == len(s[0]) and len(s[0]) > 0, f"image {i}, {workers} workers"
            for x, y in zip(g, s):
                np.testing.assert_array_equal(x, y)


def test_batch_errors(mg):
    """A failed image: its status per image, or the first failure raised
    with its index; bad batch arguments raise the reference's statuses."""
    case = BATCH_CASES["batch_360"]
    batch = make_batch_inputs(case)
    models = batch_models(mg, case, batch)
    images = [wl.image for wl in batch]
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_models_batch(images, models, *controls(case), workers=2)
    first = next(i for i, w in enumerate(BATCH["batch_360"]["images"]) if w["status"] != 0)
    assert e.value.status == -103 and f"image {first}:" in e.value.message
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_models_batch(images, models, *controls(case), workers=0)
    assert e.value.status == -1
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_models_batch(images[:1], models, *controls(case), domains=[None, None])
    assert e.value.status == -1
    assert mg.find_ncc_models_batch([], models, *controls(case)) == []


def test_single_model_batch_equals_find(mg):
    """One model: every image's matches are find_ncc_model's, bit for bit
    (find_models with one model is find)."""
    case = BATCH_CASES["batch_uneven"]
    batch = make_batch_inputs(case)
    model = batch_models(mg, case, batch)[1]
    f = case["find"]
    ctl = (f["angle_start"][0], f["angle_extent"][0], f["min_score"][0], 0, f["max_overlap"][0], "true",
           f["num_levels"][0])
    got = mg.find_ncc_models_batch([wl.image for wl in batch], [model], *ctl, workers=4)
    for i, wl in enumerate(batch):
        one = mg.find_ncc_model(wl.image, model, *ctl)
        assert len(one[0]) > 0 and (got[i][4] == 0).all()
        for x, y in zip(got[i][:4], one):
            np.testing.assert_array_equal(x, y)


def test_batch_empty_image(mg):
    """An empty image in a batch finds nothing (the operator commits empty
    outputs); the other images are unaffected."""
    case = BATCH_CASES["batch_uneven"]
    batch = make_batch_inputs(case)[:2]
    models = batch_models(mg, case, batch)
    ctl = controls(case)
    imgs = [batch[0].image, np.zeros((0, 0), np.uint8), batch[1].image]
    got = mg.find_ncc_models_batch(imgs, models, *ctl, workers=2)
    assert len(got) == 3 and all(len(x) == 0 for x in got[1])
    for g, im in zip((got[0], got[2]), (batch[0].image, batch[1].image)):
        s = mg.find_ncc_models(im, models, *ctl)
        assert len(s[0]) > 0
        for x, y in zip(g, s):
            np.testing.assert_array_equal(x, y)


def test_merged_tensor_core_launches_equal_per_find_launches(mg):
    """A batch merges its finds' tensor-core launches (fewer launches than
    find jobs); every image's matches equal those of the same batch with one
    launch per find, bit for bit."""
    case = BATCH_CASES["batch_uneven"]
    batch = make_batch_inputs(case)
    models = batch_models(mg, case, batch)
    ctl = controls(case)
    images = [wl.image for wl in batch]
    mg.set_batch_merge(1)  # all four workers in one cohort
    try:
        mg.batch_profile_reset()
        merged = mg.find_ncc_models_batch(images, models, *ctl, workers=4)
        st = mg.batch_profile_read()
        assert st["jobs"] > st["launches"] > 0, st
        mg.set_batch_merge(0)
        mg.batch_profile_reset()
        separate = mg.find_ncc_models_batch(images, models, *ctl, workers=4)
        assert mg.batch_profile_read()["launches"] == 0
        mg.set_batch_merge(2)  # two cohorts of two
        cohorts = mg.find_ncc_models_batch(images, models, *ctl, workers=4)
    finally:
        mg.set_batch_merge(0)
    for i, (a, b, c) in enumerate(zip(merged, separate, cohorts)):
        assert len(a[0]) > 0, f"image {i}"
        for x, y, z in zip(a, b, c):
            np.testing.assert_array_equal(x, y)
            np.testing.assert_array_equal(x, z)


def test_merged_batch_of_2048_scenes(mg):
    """Eight 2048^2 scenes sharing one 128^2 template (5 poses each, +-30
    degrees: the throughput workload) in one batch with merged tensor-core
    launches: every image's matches equal find_ncc_model's on it, bit for
    bit, and, for two of them, the FP64 oracle's (count, order, 0.05 px,
    0.05 deg, 1e-4)."""
    import math
    from concurrent.futures import ThreadPoolExecutor

    import oracle_lib
    from mvkit_gb300 import workloads as W
    D = math.radians
    gen = dict(height=2048, width=2048, tsize=128, n_poses=5, angle_range=(-D(30), D(30)))
    wls = [W.make_workload(2000 + i, template_seed=1, **gen) for i in range(8)]
    model = mg.create_ncc_model(wls[0].template, 4, -D(30), D(60), "auto", "use_polarity")
    ctl = (-D(30), D(60), 0.7, 5, 0.5, "true", 4)
    mg.set_batch_merge(2)
    try:
        mg.batch_profile_reset()
        got = mg.find_ncc_models_batch([w.image for w in wls], [model], *ctl, workers=8)
        st = mg.batch_profile_read()
    finally:
        mg.set_batch_merge(0)
    assert st["jobs"] > st["launches"] > 0 and st["macs"] > 0, st
    for i, w in enumerate(wls):
        one = mg.find_ncc_model(w.image, model, *ctl)
        assert len(one[0]) == 5, f"scene {i}"
        for x, y in zip(got[i][:4], one):
            np.testing.assert_array_equal(x, y)
    orc = oracle_lib.oracle()
    om = orc.create(wls[0].template, levels=4, angle_start=-D(30), angle_extent=D(60))
    with ThreadPoolExecutor(2) as ex:
        want = list(ex.map(lambda w: orc.find(om, w.image, -D(30), D(60), 0.7, 5, 0.5, True, 4, 1), wls[:2]))
    for i in range(2):
        assert_same_matches(got[i][:4], want[i], f"scene {i} vs oracle")
