"""Searches through the reference-signature C ABI (include/mvkit_gb300_mv.h)
on the GPU: a C program calling mv_gen_image1 -> mv_reduce_domain ->
mv_create_ncc_model -> mv_find_ncc_model / mv_find_ncc_models, and a C++
program calling mv::FindNccModel, return the matches the same programs
return when linked against the reference's own compiled C ABI
(tests/golden/mv_abi.json): same status, count and order, |drow|, |dcol| <=
0.05 px, |dangle| <= 0.05 deg, |dscore| <= 1e-4."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import mv_abi

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
FIXTURE = json.loads((ROOT / "tests" / "golden" / "mv_abi.json").read_text())


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    from mvkit_gb300 import build
    build.build()
    return mv_abi.compile_probe(mv_abi.OURS, tmp_path_factory.mktemp("probe") / "probe")


def assert_close(got, want):
    got, want = np.array(got), np.array(want)
    assert got.shape == want.shape, (got, want)
    if got.size == 0:
        return
    d = np.abs(got - want)
    assert d[:, 0].max() <= 0.05 and d[:, 1].max() <= 0.05, d
    assert d[:, 2].max() <= math.radians(0.05), d
    assert d[:, 3].max() <= 1e-4, d
    if got.shape[1] == 5:
        assert (got[:, 4] == want[:, 4]).all()


@pytest.mark.parametrize("name", list(mv_abi.FIND_CASES))
def test_find_through_reference_signatures(probe, name):
    want = FIXTURE["find"][name]
    got = mv_abi.run_find(probe, name)
    assert got["status"] == want["status"], got
    assert len(got["matches"]) == len(want["matches"]), (got, want)
    assert_close(got["matches"], want["matches"])


def test_cpp_find(tmp_path):
    from mvkit_gb300 import build
    build.build()
    probe = mv_abi.compile_cpp_probe(mv_abi.OURS, tmp_path / "cpp")
    got, want = mv_abi.run_cpp(probe, "cfg1_s1"), FIXTURE["cpp"]["cfg1_s1"]
    assert [l for l in got if not l.startswith("match")] == [l for l in want if not l.startswith("match")]
    gm = [[float(v) for v in l.split()[1:]] for l in got if l.startswith("match")]
    wm = [[float(v) for v in l.split()[1:]] for l in want if l.startswith("match")]
    assert_close(gm, wm)
