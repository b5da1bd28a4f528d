"""Records the reference's FindNccModels results (find_models,
src/ncc_matching/matcher.cpp:1077-1124, as mv_find_ncc_models calls it) for
the cases of multi_cases.py, from the reference compiled from its own sources
(oracle/Makefile `ref`).

Run in a container where the reference sources are present:
    make -C oracle ref && python tests/golden/make_multi.py
Writes tests/golden/multi.json: per case the input digest and the matches
(row, column, angle, score in the matcher's pixel-centre convention, model
index)."""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))

import oracle_lib  # noqa: E402
from golden.multi_cases import MULTI_CASES, expand, make_multi_inputs  # noqa: E402


def build_models(ref, case, wl):
    models = []
    for spec in case["models"]:
        if "same" in spec:
            models.append(models[spec["same"]])
            continue
        c = spec["create"]
        models.append(ref.create(wl.templates[spec["t"]], levels=c["levels"], angle_start=c["angle_start"],
                                 angle_extent=c["angle_extent"], angle_step=c.get("angle_step", 0.0),
                                 ignore_polarity=c.get("ignore_polarity", False)))
    return models


def main():
    ref = oracle_lib.reference("scalar")
    if ref is None:
        raise SystemExit("reference build missing: make -C oracle ref")
    out = {"source": "reference mvkit find_models compiled from its sources (scalar build)", "cases": {}}
    for name, case in MULTI_CASES.items():
        wl = make_multi_inputs(case)
        models = build_models(ref, case, wl)
        opts, sel_n, sel_o = expand(case["find"], len(models))
        t0 = time.perf_counter()
        res = ref.find_models(models, wl.image, opts, sel_n, sel_o)
        dt = time.perf_counter() - t0
        out["cases"][name] = {"digest": wl.digest(), "matches": res.tolist(), "seconds_scalar": round(dt, 4),
                              "truth": [[[p.row, p.column, p.angle] for p in ps] for ps in wl.poses]}
        print(name, len(res), [int(x) for x in res[:, 4]], f"{dt:.3f}s", flush=True)
    (HERE / "multi.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
