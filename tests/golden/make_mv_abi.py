"""Generates tests/golden/mv_abi.json from the reference's own C ABI compiled
from its sources (oracle/Makefile `capi`): the output of
tests/capi/mv_abi_probe.c linked against it, for the fixed `cases` table and
for every search of tests/mv_abi.py FIND_CASES, and the output of
tests/capi/mv_cpp_probe.cpp (the header-only C++ functions) linked the same way.

Run in a container where the reference sources are present:
    make -C oracle capi && python tests/golden/make_mv_abi.py
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))

import mv_abi  # noqa: E402


def main():
    if not mv_abi.REFERENCE.exists():
        raise SystemExit("reference C ABI missing: make -C oracle capi")
    out = {"source": "reference mvkit C ABI (mv_*) compiled from its sources (scalar build), "
                     "driven by tests/capi/mv_abi_probe.c", "cases": [], "model_file_sha256": "", "find": {}}
    with tempfile.TemporaryDirectory() as d:
        probe = mv_abi.compile_probe(mv_abi.REFERENCE, Path(d) / "probe_ref")
        work = Path(d) / "cases"
        work.mkdir()
        lines, model = mv_abi.run_cases(probe, work)
        out["cases"] = lines
        out["model_file_sha256"] = hashlib.sha256(model).hexdigest()
        cpp = mv_abi.compile_cpp_probe(mv_abi.REFERENCE, Path(d) / "cpp_ref")
        out["cpp"] = {"empty": mv_abi.run_cpp(cpp, None), "cfg1_s1": mv_abi.run_cpp(cpp, "cfg1_s1")}
        for name in mv_abi.FIND_CASES:
            t0 = time.perf_counter()
            out["find"][name] = mv_abi.run_find(probe, name)
            print(name, out["find"][name]["status"], len(out["find"][name]["matches"]),
                  f"{time.perf_counter() - t0:.1f}s", flush=True)
    (HERE / "mv_abi.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
