"""Records the reference's model files (src/ncc_matching/persist.cpp) for the
persistence parity tests, from the reference compiled from its own sources
(oracle/Makefile `ref`).

Run in a container where the reference sources are present:
    make -C oracle ref && python tests/golden/make_models.py
Writes:
- tests/golden/models/<name>.ncm: the reference's file for each MODEL_FILES
  entry of model_cases.py;
- tests/golden/models.json: per golden case of cases.py the SHA-256 of the
  reference's file, per MODEL_FILES entry the trained parameters, and per
  EDITS entry the status of the reference's reader (0 = accepted) with the
  SHA-256 of the file the reference writes back for an accepted one."""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))

import oracle_lib  # noqa: E402
from golden.cases import CASES, make_inputs  # noqa: E402
from golden.model_cases import EDIT_BASE, EDITS, MODEL_FILES, sha256, template_of  # noqa: E402


def create(ref, t, mask, c):
    return ref.create(t, levels=c.get("levels", 0), angle_start=c["angle_start"], angle_extent=c["angle_extent"],
                      angle_step=c.get("angle_step", 0.0), ignore_polarity=c.get("ignore_polarity", False),
                      mask=mask)


def main():
    ref = oracle_lib.reference("scalar")
    if ref is None:
        raise SystemExit("reference build missing: make -C oracle ref")
    out = {"source": "reference mvkit serialize/deserialize compiled from its sources (scalar build)",
           "case_sha256": {}, "files": {}, "edits": {}}
    for name, case in CASES.items():
        wl, mask = make_inputs(case)
        m = create(ref, wl.template, mask, case["create"])
        out["case_sha256"][name] = sha256(ref.serialize(m))
    (HERE / "models").mkdir(exist_ok=True)
    files = {}
    for name, spec in MODEL_FILES.items():
        t, mask, c = template_of(spec)
        m = create(ref, t, mask, c)
        b = ref.serialize(m)
        files[name] = b
        (HERE / "models" / f"{name}.ncm").write_bytes(b)
        info = m.info()
        out["files"][name] = {"sha256": sha256(b), "size": len(b), "levels": info["levels"],
                              "angle_step": info["angle_step"], "origin_row": info["origin_row"],
                              "origin_column": info["origin_column"]}
    base = files[EDIT_BASE]
    for name, edit in EDITS.items():
        data = edit(base)
        try:
            m = ref.deserialize(data)
        except oracle_lib.CheckerError as e:
            out["edits"][name] = {"status": e.status, "message": e.message}
        else:
            out["edits"][name] = {"status": 0, "rewritten_sha256": sha256(ref.serialize(m))}
        print(name, out["edits"][name], flush=True)
    (HERE / "models.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
