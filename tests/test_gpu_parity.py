"""GPU parity: the CUDA find path against the reference's golden matches and the
oracle restatement, through the C ABI (ctypes) of libmvkit_gb300.so.

Tolerances (final matches): identical count and order, |drow|,|dcol| <= 0.05 px,
|dangle| <= 0.05 deg, |dscore| <= 1e-4.  Pyramid levels are compared bit-exact.
Candidate stages are compared as sets of poses (exact FP64 equality of
row/column/angle): the CUDA path scores windows in FP32 from exact integer
moments, so a stage may differ from the FP64 oracle only by near-ties."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from golden.cases import CASES, LARGE, make_inputs, search_domain
from golden.multi_cases import MULTI_CASES, make_multi_inputs

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())["cases"]
TOL_PX = 0.05
TOL_ANGLE = math.radians(0.05)
TOL_SCORE = 1e-4


@pytest.fixture(scope="module")
def mg():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    mvkit_gb300.load()
    return mvkit_gb300


@pytest.fixture(scope="module")
def orc():
    return oracle_lib.oracle()


def gpu_model(mg, case, wl, mask):
    c = case["create"]
    return mg.create_ncc_model(wl.template, c["levels"], c["angle_start"], c["angle_extent"],
                               c.get("angle_step", "auto") or "auto",
                               "ignore_global_polarity" if c.get("ignore_polarity") else "use_polarity", domain=mask)


def gpu_find(mg, model, image, case, domain=None, **over):
    f = dict(case["find"])
    f.update(over)
    return mg.find_ncc_model(image, model, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                             f["max_overlap"], "true" if f["subpixel"] else "false", [f["highest"], f["lowest"]],
                             domain=domain)


def assert_same_matches(got, want_internal, label=""):
    want = oracle_lib.to_halcon(np.array(want_internal).reshape(-1, 4))
    g = np.stack(got, axis=1) if len(got[0]) else np.zeros((0, 4))
    assert g.shape == want.shape, f"{label}: {len(g)} matches vs reference {len(want)}\n{g}\n{want}"
    if len(g):
        d = np.abs(g - want)
        assert d[:, 0].max() <= TOL_PX and d[:, 1].max() <= TOL_PX, f"{label} position\n{g}\n{want}"
        assert d[:, 2].max() <= TOL_ANGLE, f"{label} angle\n{g}\n{want}"
        assert d[:, 3].max() <= TOL_SCORE, f"{label} score\n{g}\n{want}"


@pytest.mark.parametrize("name", sorted(CASES))
def test_find_matches_reference(mg, name):
    case = CASES[name]
    wl, mask = make_inputs(case)
    assert wl.digest() == GOLDEN[name]["digest"]
    model = gpu_model(mg, case, wl, mask)
    if "status" in GOLDEN[name]:
        # the reference rejects this search (coarse candidate budget): same status
        with pytest.raises(mg.MvError) as err:
            gpu_find(mg, model, wl.image, case)
        assert err.value.status == GOLDEN[name]["status"]
        return
    got = gpu_find(mg, model, wl.image, case, domain=search_domain(case, wl))
    assert_same_matches(got, GOLDEN[name]["matches"], name)


@pytest.mark.parametrize("name", ["tiny16", "rot3_all", "mask_disc", "u16_rot"])
def test_find_with_model_from_file(mg, name, tmp_path):
    """A model read back from its file finds what the reference finds.  For
    tiny16 the file is the reference's own (tests/golden/models/); the other
    cases write ours, whose bytes equal the reference's (test_persist.py)."""
    case = CASES[name]
    wl, mask = make_inputs(case)
    if name == "tiny16":
        path = Path(__file__).parent / "golden" / "models" / "tiny16.ncm"
    else:
        path = tmp_path / f"{name}.ncm"
        mg.write_ncc_model(gpu_model(mg, case, wl, mask), str(path))
    model = mg.read_ncc_model(str(path))
    assert_same_matches(gpu_find(mg, model, wl.image, case), GOLDEN[name]["matches"], name)


MULTI = json.loads((Path(__file__).parent / "golden" / "multi.json").read_text())["cases"]


def multi_models(mg, case, wl):
    models = []
    for spec in case["models"]:
        if "same" in spec:
            models.append(models[spec["same"]])
            continue
        c = spec["create"]
        models.append(mg.create_ncc_model(wl.templates[spec["t"]], c["levels"], c["angle_start"], c["angle_extent"],
                                          "auto", "use_polarity"))
    return models


@pytest.mark.parametrize("name", sorted(MULTI_CASES))
def test_find_models_matches_reference(mg, name):
    """FindNccModels: same matches, order and model indices as the
    reference's find_models on the same control tuples."""
    case = MULTI_CASES[name]
    wl = make_multi_inputs(case)
    assert wl.digest() == MULTI[name]["digest"]
    models = multi_models(mg, case, wl)
    f = case["find"]
    got = mg.find_ncc_models(wl.image, models, f["angle_start"], f["angle_extent"], f["min_score"],
                             f["num_matches"], f["max_overlap"], f["subpixel"], f["num_levels"])
    want = np.array(MULTI[name]["matches"]).reshape(-1, 5)
    assert list(got[4]) == [int(x) for x in want[:, 4]], f"{name}: model indices {list(got[4])} vs {want[:, 4]}"
    assert_same_matches(got[:4], want[:, :4], name)


def test_find_models_with_domain(mg):
    """FindNccModels on a reduced domain: each model's find restricted to
    it, the selection over all (each model crops the image differently)."""
    case = CASES["roi_two"]
    wl, mask = make_inputs(case)
    dom = search_domain(case, wl)
    a = gpu_model(mg, case, wl, mask)
    b = mg.create_ncc_model(wl.template, 2, case["create"]["angle_start"], case["create"]["angle_extent"], "auto",
                            "use_polarity")
    f = case["find"]
    many = mg.find_ncc_models(wl.image, [a, b], f["angle_start"], f["angle_extent"], f["min_score"], [0],
                              [0.5, 0.5], "true", [3, 1, 2, 1], domain=dom)
    for k, m in enumerate((a, b)):
        one = mg.find_ncc_model(wl.image, m, f["angle_start"], f["angle_extent"], f["min_score"], 0, 0.5, "true",
                                [3 if k == 0 else 2, 1], domain=dom)
        sel = many[4] == k
        assert sel.sum() == len(one[0]) and len(one[0]) == 2
        for x, y in zip(one, many[:4]):
            np.testing.assert_allclose(np.sort(x), np.sort(y[sel]), atol=1e-9)


@pytest.fixture
def host_build(mg):
    yield
    mg.ncc.set_model_build("device")


@pytest.mark.parametrize("spec", [
    dict(case="rot3_all"), dict(case="u16_rot"), dict(case="mask_disc"), dict(case="full_circle"),
    dict(case="polarity"), dict(case="tiny16"), dict(case="big160"), dict(case="cfg1_s1"),
    dict(case="rot3_all", levels=0, angle_start=-math.pi, angle_extent=2 * math.pi),
    dict(case="cfg1_s1", levels=0, angle_start=-1.0, angle_extent=2.0, angle_step=0.03)])
def test_device_model_build_bit_identical(mg, spec, host_build):
    """The model built on the GPU has the host FP64 build's tables bit for
    bit (weights, sample and run tables, descriptors)."""
    case = CASES[spec["case"]]
    wl, mask = make_inputs(case)
    c = dict(case["create"])
    c.update({k: v for k, v in spec.items() if k != "case"})
    args = (wl.template, c["levels"] or "auto", c["angle_start"], c["angle_extent"], c.get("angle_step", 0) or "auto",
            "ignore_global_polarity" if c.get("ignore_polarity") else "use_polarity")
    mg.ncc.set_model_build("device")
    dev = mg.create_ncc_model(*args, domain=mask)
    mg.ncc.set_model_build("host")
    host = mg.create_ncc_model(*args, domain=mask)
    assert mg.ncc.model_tables_digest(dev) == mg.ncc.model_tables_digest(host)
    assert mg.get_ncc_model_params(dev) == mg.get_ncc_model_params(host)


def test_device_model_build_errors(mg, host_build):
    """Both builds raise the reference's errors: a raster with fewer than
    four samples, and the 16 M sample budget."""
    tiny = np.array([[10, 200], [30, 90]], np.uint8)
    big = (np.arange(700 * 700) % 251).astype(np.uint8).reshape(700, 700)
    for where in ("device", "host"):
        mg.ncc.set_model_build(where)
        with pytest.raises(mg.MvError) as e:
            mg.create_ncc_model(tiny, 1, 0.0, 1.0, "auto", "use_polarity")
        assert e.value.status == -1 and "degenerate" in e.value.message
        with pytest.raises(mg.MvError) as e:
            mg.create_ncc_model(big, 1, -math.pi, 2 * math.pi, 0.01, "use_polarity")
        assert e.value.status == -103 and "budget" in e.value.message


def test_find_models_single_equals_find(mg):
    """One model through FindNccModels gives FindNccModel's matches."""
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    f = case["find"]
    one = gpu_find(mg, model, wl.image, case)
    many = mg.find_ncc_models(wl.image, [model], f["angle_start"], f["angle_extent"], f["min_score"],
                              f["num_matches"], f["max_overlap"], "true" if f["subpixel"] else "false",
                              [f["highest"], f["lowest"]])
    assert list(many[4]) == [0] * len(one[0])
    for a, b in zip(one, many[:4]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", list(LARGE))
def test_find_matches_reference_2048(mg, name):
    case = LARGE[name]
    wl, mask = make_inputs(case)
    assert wl.digest() == GOLDEN[name]["digest"]
    model = gpu_model(mg, case, wl, mask)
    got = gpu_find(mg, model, wl.image, case)
    assert_same_matches(got, GOLDEN[name]["matches"], name)


@pytest.mark.parametrize("seed", [31, 32, 33])
def test_find_matches_oracle_fresh_seeds(mg, orc, seed):
    case = dict(gen=dict(seed=seed, height=600, width=800, tsize=64, n_poses=3,
                         angle_range=(-math.radians(25), math.radians(25))),
                create=dict(levels=3, angle_start=-math.radians(25), angle_extent=math.radians(50)),
                find=dict(angle_start=-math.radians(25), angle_extent=math.radians(50), min_score=0.7,
                          num_matches=3, max_overlap=0.5, subpixel=True, highest=3, lowest=1))
    wl, mask = make_inputs(case)
    c, f = case["create"], case["find"]
    om = orc.create(wl.template, levels=c["levels"], angle_start=c["angle_start"], angle_extent=c["angle_extent"])
    want = orc.find(om, wl.image, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                    f["max_overlap"], True, 3, 1)
    got = gpu_find(mg, gpu_model(mg, case, wl, mask), wl.image, case)
    assert_same_matches(got, want, f"seed {seed}")


def test_pyramid_levels_bit_exact(mg, orc):
    case = CASES["rot_l4_2"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    om = orc.create(wl.template, levels=4, angle_start=case["create"]["angle_start"],
                    angle_extent=case["create"]["angle_extent"])
    for level in range(4):
        sums, geom = mg.pyramid_level(wl.image, model, 4, level)
        ref, rgeom = orc.pyramid(om, wl.image, 4, level)
        assert sums.shape == ref.shape
        # the reference's FP64 level value is sum / 4^level - dc, exactly
        np.testing.assert_array_equal(sums.astype(np.float64) / float(4 ** level) - rgeom[4], ref)


def pose_set(a):
    return {(float(r[0]), float(r[1]), float(r[2])) for r in np.asarray(a).reshape(-1, 4)}


@pytest.fixture
def path(mg, request):
    mg.set_correlation_path(request.param)
    yield request.param
    mg.set_correlation_path("tensor")


@pytest.mark.parametrize("path", ["tensor", "plain"], indirect=True)
@pytest.mark.parametrize("name", ["cfg1_s1", "rot3_all", "rot_l4_2", "u16_rot", "polarity", "full_circle",
                                  "u16_12bit", "tiny16", "roi_two", "roi_ring", "roi_strips", "roi_no_subpixel",
                                  "cfg2_s1"])
def test_candidate_stages_match_oracle(mg, orc, name, path):
    case = {**CASES, **LARGE}[name]
    wl, mask = make_inputs(case)
    c, f = case["create"], case["find"]
    om = orc.create(wl.template, levels=c["levels"], angle_start=c["angle_start"], angle_extent=c["angle_extent"],
                    ignore_polarity=c.get("ignore_polarity", False), mask=mask)
    model = gpu_model(mg, case, wl, mask)
    ctl = (f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"], f["max_overlap"],
           "true" if f["subpixel"] else "false", [f["highest"], f["lowest"]])
    steps = [0] + list(range(1, f["highest"]))
    dom = search_domain(case, wl)
    for stage in steps:
        want = orc.find(om, wl.image, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                        f["max_overlap"], f["subpixel"], f["highest"], f["lowest"], stage=stage, domain=dom)
        got = mg.find_ncc_model_stage(wl.image, model, *ctl, stage=stage, domain=dom)
        a, b = pose_set(got), pose_set(want)
        sym = len(a ^ b)
        # identical sets on every case measured; at most a near-tie pair
        # (two candidates whose FP32 and FP64 scores order differently) may swap
        assert sym <= 2, f"{name} stage {stage}: {len(a)} vs {len(b)} candidates, {sym} differ"
        # scores of the common candidates agree to FP32 precision
        ws = {(r[0], r[1], r[2]): r[3] for r in want}
        for r in got:
            k = (r[0], r[1], r[2])
            if k in ws:
                assert abs(r[3] - ws[k]) < 2e-5, f"{name} stage {stage} score {r[3]} vs {ws[k]}"
    # full-resolution scores of the sorted candidate list
    want = orc.find(om, wl.image, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                    f["max_overlap"], f["subpixel"], f["highest"], f["lowest"], stage=100, domain=dom)
    got = mg.find_ncc_model_stage(wl.image, model, *ctl, stage=100, domain=dom)
    want = want[np.isfinite(want[:, 3])]   # the find loop skips unscorable candidates
    ws = {(r[0], r[1], r[2]): r[3] for r in want}
    common = [r for r in got if (r[0], r[1], r[2]) in ws]
    assert len(common) >= len(want) - 2 and len(got) <= len(want) + 2
    assert np.all(np.diff(got[:, 3]) <= 0), "sorted by score"
    for r in common:
        assert abs(r[3] - ws[(r[0], r[1], r[2])]) < 1e-4


@pytest.mark.parametrize("path", ["plain"], indirect=True)
@pytest.mark.parametrize("name", ["cfg1_s1", "rot_l4_2", "u16_rot", "polarity", "mask_disc", "full_circle",
                                  "u16_12bit", "big160", "roi_two", "roi_ring", "roi_lowest2"])
def test_find_matches_reference_plain_path(mg, name, path):
    case = CASES[name]
    wl, mask = make_inputs(case)
    got = gpu_find(mg, gpu_model(mg, case, wl, mask), wl.image, case, domain=search_domain(case, wl))
    assert_same_matches(got, GOLDEN[name]["matches"], f"{name} plain")


def test_tensor_core_tracking_runs(mg):
    """The default path scores the tracking windows of a u8 search on the
    tensor cores (the track_tc stage launches), the plain path never does."""
    case = LARGE["cfg2_s1"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    launches = {}
    for p in ("tensor", "plain"):
        mg.set_correlation_path(p)
        mg.profile_enable(True)
        mg.profile_reset()
        got = gpu_find(mg, model, wl.image, case)
        prof = mg.profile_read()
        mg.profile_enable(False)
        launches[p] = prof["track_tc"]["launches"]
        assert_same_matches(got, GOLDEN["cfg2_s1"]["matches"], f"cfg2_s1 {p}")
    mg.set_correlation_path("tensor")
    assert launches["tensor"] > 0 and launches["plain"] == 0, launches


@pytest.mark.parametrize("maxval", [4095, 65535])
def test_uint16_levels_on_tensor_cores(mg, orc, maxval):
    """uint16 level sums need three or four fp16 parts above level 1: the
    coarse scan (level 3) and both tracking steps (levels 2 and 1) run on the
    tensor cores (three track_tc launches per find), and the candidates after
    every stage and the final matches equal the oracle's."""
    from mvkit_gb300 import workloads as W
    wl = W.make_workload(81, 600, 800, 64, 3, angle_range=(-math.radians(20), math.radians(20)), maxval=maxval,
                         noise_sigma=20)
    a0, ext = -math.radians(20), math.radians(40)
    model = mg.create_ncc_model(wl.template, 4, a0, ext, "auto", "use_polarity")
    om = orc.create(wl.template, levels=4, angle_start=a0, angle_extent=ext)
    ctl = (a0, ext, 0.7, 3, 0.5, "true", 4)
    mg.set_correlation_path("tensor")
    mg.profile_enable(True)
    mg.profile_reset()
    got = mg.find_ncc_model(wl.image, model, *ctl)
    prof = mg.profile_read()
    mg.profile_enable(False)
    assert prof["track_tc"]["launches"] == 3 and prof["track_tc"]["work"] > 0, prof["track_tc"]
    want = orc.find(om, wl.image, a0, ext, 0.7, 3, 0.5, True, 4, 1)
    assert len(want) == 3
    assert_same_matches(got, want, f"uint16 max {maxval}")
    for stage in (0, 1, 2):
        w = orc.find(om, wl.image, a0, ext, 0.7, 3, 0.5, True, 4, 1, stage=stage)
        g = mg.find_ncc_model_stage(wl.image, model, *ctl, stage=stage)
        assert len(pose_set(g) ^ pose_set(w)) <= 2, f"stage {stage}"


def test_device_resident_input_and_repeat_calls(mg):
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    a = gpu_find(mg, model, wl.image, case)
    b = gpu_find(mg, model, mg.DeviceImage(wl.image), case)
    c = gpu_find(mg, model, wl.image, case)
    for x, y in ((a, b), (a, c)):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


def test_empty_and_errors(mg):
    case = CASES["cfg1_s1"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    r = mg.find_ncc_model(np.zeros((0, 0), np.uint8), model, 0.0, 0.0, 0.8, 1, 0.5, "true", 3)
    assert all(len(x) == 0 for x in r)
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_model(np.zeros((8001, 4001), np.uint8), model, 0.0, 0.0, 0.8, 1, 0.5, "true", 3)
    assert e.value.status == -103
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(np.full((32, 32), 9, np.uint8))
    assert e.value.status == -1
    with pytest.raises(mg.MvError) as e:
        mg.create_ncc_model(wl.template, num_levels=9)
    assert e.value.status == -1
    # query range outside the trained range: no matches, no error
    r = mg.find_ncc_model(wl.image, model, 1.0, 0.5, 0.8, 1, 0.5, "true", 3)
    assert all(len(x) == 0 for x in r)


def test_model_params(mg):
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    lv, a0, a1, step, metric = mg.get_ncc_model_params(model)
    assert lv == GOLDEN["rot3_all"]["levels"]
    assert a0 == case["create"]["angle_start"] and a1 == case["create"]["angle_extent"]
    assert step == GOLDEN["rot3_all"]["angle_step"]
    assert metric == "use_polarity"


def _sweep_case(seed):
    """A seeded small search: image type, size, template, angle range, levels,
    controls, polarity and an optional search domain drawn from the seed."""
    rng = np.random.default_rng(1000 + seed)
    u16 = bool(rng.integers(0, 4) == 0)
    tsize = int(rng.choice([24, 32, 40, 48]))
    h, w = int(rng.choice([240, 300])), int(rng.choice([320, 400]))
    span = float(rng.choice([0.0, math.radians(20), math.radians(60), 2 * math.pi]))
    start = -span / 2
    levels = int(rng.integers(2, 4)) if tsize >= 40 else 2
    gen = dict(seed=200 + seed, height=h, width=w, tsize=tsize, n_poses=int(rng.integers(1, 4)),
               angle_range=(start * 0.9, (start + span) * 0.9), invert_odd=bool(rng.integers(0, 4) == 0))
    if u16:
        gen.update(maxval=4095, noise_sigma=20)
    create = dict(levels=levels, angle_start=start, angle_extent=span,
                  ignore_polarity=gen["invert_odd"])
    find = dict(angle_start=start, angle_extent=span, min_score=float(rng.choice([0.6, 0.7, 0.8])),
                num_matches=int(rng.integers(0, 4)), max_overlap=float(rng.choice([0.0, 0.3, 0.5])),
                subpixel=bool(rng.integers(0, 5) != 0), highest=levels, lowest=1)
    case = dict(gen=gen, create=create, find=find)
    kind = int(rng.integers(0, 3))  # 0 whole image, 1 rectangle, 2 two rectangles (sparse)
    if kind:
        case["domain"] = [("around", 0, int(rng.integers(10, 60)))] + (
            [("around", min(1, gen["n_poses"] - 1), int(rng.integers(3, 20)))] if kind == 2 else [])
    return case


@pytest.mark.parametrize("seed", list(range(24)))
def test_find_matches_oracle_random_sweep(mg, orc, seed):
    """Seeded random searches against the oracle (bit-exact to the reference's
    scalar build): identical match count and order, poses and scores within
    the tolerances above."""
    case = _sweep_case(seed)
    wl, mask = make_inputs(case)
    dom = search_domain(case, wl)
    c, f = case["create"], case["find"]
    om = orc.create(wl.template, levels=c["levels"], angle_start=c["angle_start"], angle_extent=c["angle_extent"],
                    ignore_polarity=c["ignore_polarity"])
    try:
        want = orc.find(om, wl.image, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                        f["max_overlap"], f["subpixel"], f["highest"], f["lowest"], domain=dom)
    except oracle_lib.CheckerError as e:
        with pytest.raises(mg.MvError) as err:
            gpu_find(mg, gpu_model(mg, case, wl, mask), wl.image, case, domain=dom)
        assert err.value.status == e.status
        return
    got = gpu_find(mg, gpu_model(mg, case, wl, mask), wl.image, case, domain=dom)
    assert_same_matches(got, want, f"sweep {seed}: {case}")


def test_large_configuration_statuses(mg, orc, host_build):
    """The large split-precision configuration (8192x8192 uint16 12-bit
    image; 512x512 template over 360 degrees, NumLevels 6) is outside the
    reference's budgets: the image exceeds its 32 M pixel search budget and
    the model its 16 M raster-sample budget.  Both give the reference's
    status and message here and in the oracle."""
    big = np.zeros((8192, 8192), np.uint16)
    case = CASES["cfg1_s1"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    with pytest.raises(mg.MvError) as e:
        mg.find_ncc_model(big, model, 0.0, 0.0, 0.5, 20, 0.3, "true", 3)
    assert e.value.status == -103 and "pixel budget" in e.value.message
    om = orc.create(wl.template, levels=3)
    with pytest.raises(oracle_lib.CheckerError) as oe:
        orc.find(om, big, 0.0, 0.0, 0.5, 20, 0.3, True, 3, 1)
    assert oe.value.status == -103 and "pixel budget" in oe.value.message
    tmpl = (np.random.default_rng(5).integers(0, 4096, (512, 512))).astype(np.uint16)
    for where in ("device", "host"):
        mg.ncc.set_model_build(where)
        with pytest.raises(mg.MvError) as e:
            mg.create_ncc_model(tmpl, 6, -math.pi, 2 * math.pi, "auto", "use_polarity")
        assert e.value.status == -103 and "budget" in e.value.message
    with pytest.raises(oracle_lib.CheckerError) as oe:
        orc.create(tmpl, levels=6, angle_start=-math.pi, angle_extent=2 * math.pi)
    assert oe.value.status == -103 and "budget" in oe.value.message
