"""Generates tests/golden/golden.json from the reference mvkit matcher compiled
from its own sources (oracle/Makefile `ref`, scalar and AVX2 builds).

Run in a container where the reference sources are present:
    make -C oracle ref && python tests/golden/make_golden.py
The fixture holds, per case of tests/golden/cases.py, the input digest, the
reference's final matches (matcher-internal pixel-centre convention), the
same through the AVX2 build, and model facts (level count, angle step)."""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))

import oracle_lib  # noqa: E402
from golden.cases import CASES, LARGE, make_inputs, search_domain  # noqa: E402


def run(checker, case, wl, mask):
    c = case["create"]
    model = checker.create(wl.template, levels=c["levels"], angle_start=c["angle_start"],
                           angle_extent=c["angle_extent"], angle_step=c.get("angle_step", 0.0),
                           ignore_polarity=c.get("ignore_polarity", False), mask=mask)
    f = case["find"]
    t0 = time.perf_counter()
    res = checker.find(model, wl.image, f["angle_start"], f["angle_extent"], f["min_score"], f["num_matches"],
                       f["max_overlap"], f["subpixel"], f["highest"], f["lowest"], domain=search_domain(case, wl))
    dt = time.perf_counter() - t0
    return model, res, dt


def main():
    scalar = oracle_lib.reference("scalar")
    avx2 = oracle_lib.reference("avx2")
    if scalar is None:
        raise SystemExit("reference build missing: make -C oracle ref")
    out = {"source": "reference mvkit matcher compiled from its sources (scalar build)", "cases": {}}
    for name, case in {**CASES, **LARGE}.items():
        wl, mask = make_inputs(case)
        try:
            model, res, dt = run(scalar, case, wl, mask)
        except oracle_lib.CheckerError as e:
            # the reference rejects the search (e.g. coarse candidate budget):
            # the fixture records the status the drop-in must return
            out["cases"][name] = {"digest": wl.digest(), "status": e.status, "message": str(e),
                                  "truth": [[p.row, p.column, p.angle] for p in wl.poses]}
            print(name, "status", e.status, flush=True)
            continue
        info = model.info()
        entry = {"digest": wl.digest(), "matches": res.tolist(), "seconds_scalar": round(dt, 4),
                 "levels": info["levels"], "angle_step": info["angle_step"],
                 "truth": [[p.row, p.column, p.angle] for p in wl.poses]}
        if avx2 is not None:
            _, ra, da = run(avx2, case, wl, mask)
            entry["matches_avx2"] = ra.tolist()
            entry["seconds_avx2"] = round(da, 4)
        out["cases"][name] = entry
        print(name, len(res), f"{dt:.3f}s", flush=True)
    (HERE / "golden.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
