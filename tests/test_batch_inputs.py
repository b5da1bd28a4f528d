"""The batched cases' scenes (mvkit_gb300.workloads.make_batch_workloads)
are the ones the reference's results in golden/batch.json were recorded on,
and the recorded results are self-consistent (CPU only)."""
import json
from pathlib import Path

import numpy as np
import pytest

from golden.batch_cases import BATCH_CASES, make_batch_inputs
from golden.make_batch import template_digest

BATCH = json.loads((Path(__file__).parent / "golden" / "batch.json").read_text())["cases"]


@pytest.mark.parametrize("name", sorted(BATCH_CASES))
def test_batch_inputs_pinned(name):
    case = BATCH_CASES[name]
    batch = make_batch_inputs(case)
    want = BATCH[name]
    assert template_digest(batch[0].templates) == want["templates"]
    assert len(batch) == case["gen"]["n_images"] == len(want["images"])
    for wl, w in zip(batch, want["images"]):
        assert wl.digest() == w["digest"]
        assert list(wl.image.shape) == w["shape"]
        assert tuple(wl.image.shape) in case["gen"]["sizes"]
        # every template pasted 1..max_pastes times with contrast in [0.9, 1.1]
        assert all(1 <= len(p) <= case["gen"]["max_pastes"] for p in wl.poses)
        assert all(0.9 <= q.contrast <= 1.1 for p in wl.poses for q in p)
        if w["status"] != 0:
            assert w["matches"] == [] and w["status"] == -103
        else:
            m = np.array(w["matches"]).reshape(-1, 5)
            assert len(m) > 0 and set(m[:, 4].astype(int)) <= set(range(len(case["gen"]["tsizes"])))
            assert (np.diff(m[:, 3]) <= 0).all()  # final matches by descending score


def test_batch_mixes_outcomes():
    """batch_360 holds both matched scenes and LimitExceeded scenes."""
    st = [w["status"] for w in BATCH["batch_360"]["images"]]
    assert 0 in st and -103 in st
