"""Records the reference's FindNccModels results, image by image, for the
batches of batch_cases.py (find_models, src/ncc_matching/matcher.cpp:
1077-1124, as mv_find_ncc_models calls it), from the reference compiled from
its own sources (oracle/Makefile `ref`).

Run in a container where the reference sources are present:
    make -C oracle ref && python tests/golden/make_batch.py
Writes tests/golden/batch.json: per case the template digest and, per image,
the input digest, the status (0 or the reference's MvStatus) and the matches
(row, column, angle, score in the matcher's pixel-centre convention, model
index)."""
from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))

import oracle_lib  # noqa: E402
from golden.batch_cases import BATCH_CASES, make_batch_inputs  # noqa: E402
from golden.multi_cases import expand  # noqa: E402


def template_digest(templates) -> str:
    h = hashlib.sha256()
    for t in templates:
        h.update(np.ascontiguousarray(t).tobytes())
    return h.hexdigest()[:16]


def main():
    ref = oracle_lib.reference("scalar")
    if ref is None:
        raise SystemExit("reference build missing: make -C oracle ref")
    out = {"source": "reference mvkit find_models compiled from its sources (scalar build), one call per image",
           "cases": {}}
    for name, case in BATCH_CASES.items():
        batch = make_batch_inputs(case)
        c = case["create"]
        models = [ref.create(t, levels=c["levels"], angle_start=c["angle_start"], angle_extent=c["angle_extent"])
                  for t in batch[0].templates]
        opts, sel_n, sel_o = expand(case["find"], len(models))
        images = []
        for wl in batch:
            t0 = time.perf_counter()
            try:
                res = ref.find_models(models, wl.image, opts, sel_n, sel_o)
                status, message = 0, ""
            except oracle_lib.CheckerError as e:
                res, status, message = np.zeros((0, 5)), e.status, e.message
            dt = time.perf_counter() - t0
            images.append({"digest": wl.digest(), "shape": list(wl.image.shape), "status": status,
                           "message": message, "matches": res.tolist(), "seconds_scalar": round(dt, 4)})
            print(name, wl.image.shape, status, len(res), f"{dt:.2f}s", flush=True)
        out["cases"][name] = {"templates": template_digest(batch[0].templates), "images": images}
    (HERE / "batch.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
