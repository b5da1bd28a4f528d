"""Builds and runs tests/capi/mv_abi_probe.c against a library with the
reference's C signatures: this repository's libmvkit_gb300_mv.so, or the
reference's own C ABI compiled from its sources (oracle/_ref/libref_capi.so,
only where the reference sources were present).  Test infrastructure.

FIND_CASES lists the searches the probe's `find` mode runs, each from the
seeded scenes of tests/golden/cases.py, with template and search-image
domains given as mv_gen_rectangle1 rectangles."""
from __future__ import annotations

import math
import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PROBE = ROOT / "tests" / "capi" / "mv_abi_probe.c"
CPP_PROBE = ROOT / "tests" / "capi" / "mv_cpp_probe.cpp"
OURS = ROOT / "mvkit_gb300" / "_lib" / "libmvkit_gb300_mv.so"
REFERENCE = ROOT / "oracle" / "_ref" / "libref_capi.so"
D = math.radians


def compile_probe(lib: Path, out: Path) -> Path:
    cmd = ["gcc", "-std=c99", "-O1", "-I", str(ROOT / "include"), str(PROBE), "-o", str(out),
           f"-L{lib.parent}", f"-l:{lib.name}", f"-Wl,-rpath,{lib.parent}", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def compile_cpp_probe(lib: Path, out: Path) -> Path:
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(CPP_PROBE), "-o", str(out),
           f"-L{lib.parent}", f"-l:{lib.name}", f"-Wl,-rpath,{lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def run_cases(probe: Path, workdir: Path) -> tuple[list[str], bytes]:
    """The probe's `cases` lines and the model file it wrote."""
    r = subprocess.run([str(probe), "cases", str(workdir)], check=True, capture_output=True, text=True,
                       timeout=600)
    return r.stdout.splitlines(), (workdir / "model.ncm").read_bytes()


def _rect(spec):
    return "-" if spec is None else ",".join(str(int(v)) for v in spec)


# name: golden scene, create controls, template rectangle, search rectangle
# (relative to pose `k`: (k, half_size) or None), find controls, models
FIND_CASES = {
    "cfg1_s1": dict(scene="cfg1_s1", levels="3", step="auto"),
    "rot3_all": dict(scene="rot3_all", levels="3", step="auto"),
    "u16_rot": dict(scene="u16_rot", levels="3", step="auto"),
    "polarity": dict(scene="polarity", levels="3", step="auto", metric="ignore_global_polarity"),
    "lowest2": dict(scene="lowest2", levels="3", step="auto", find_levels="3,2"),
    "no_subpixel": dict(scene="no_subpixel", levels="3", step="auto"),
    "auto_levels_step": dict(scene="demo_like", levels="auto", step="0.025", find_levels="0"),
    "template_roi": dict(scene="rot3_all", levels="3", step="auto", template_rect=(4, 6, 57, 60)),
    "search_roi": dict(scene="rot3_all", levels="3", step="auto", search_around=(1, 40)),
    "models_2": dict(scene="rot3_all", levels="3", step="auto", models=2),
    "cfg2_s1": dict(scene="cfg2_s1", levels="4", step="auto"),
}


def scene_case(name: str):
    from golden.cases import CASES, LARGE
    return {**CASES, **LARGE}[name]


def find_args(name: str, workdir: Path) -> list[str]:
    """Writes the case's raw inputs to workdir; returns the probe's arguments."""
    from mvkit_gb300 import workloads as W
    spec = FIND_CASES[name]
    case = scene_case(spec["scene"])
    wl = W.make_workload(**case["gen"])
    img, tpl = np.ascontiguousarray(wl.image), np.ascontiguousarray(wl.template)
    typ = "uint2" if img.dtype == np.uint16 else "byte"
    (workdir / f"{name}_image.raw").write_bytes(img.tobytes())
    (workdir / f"{name}_template.raw").write_bytes(tpl.tobytes())
    c, f = case["create"], case["find"]
    search = None
    if "search_around" in spec:
        k, half = spec["search_around"]
        p = wl.poses[k]
        r, col = int(math.floor(p.row + .5)), int(math.floor(p.column + .5))
        search = (r - half, col - half, r + half, col + half)
    levels = spec.get("find_levels", f"{f['highest']},{f['lowest']}" if f["lowest"] != 1 else str(f["highest"]))
    return [str(workdir / f"{name}_image.raw"), str(img.shape[1]), str(img.shape[0]), typ,
            str(workdir / f"{name}_template.raw"), str(tpl.shape[1]), str(tpl.shape[0]),
            spec["levels"], repr(float(c["angle_start"])), repr(float(c["angle_extent"])), spec["step"],
            spec.get("metric", "use_polarity"), _rect(spec.get("template_rect")), _rect(search),
            repr(float(f["angle_start"])), repr(float(f["angle_extent"])), repr(float(f["min_score"])),
            str(int(f["num_matches"])), repr(float(f["max_overlap"])), "true" if f["subpixel"] else "false",
            levels] + ([str(spec["models"])] if spec.get("models") else [])


def run_find(probe: Path, name: str) -> dict:
    """Runs one find case; returns {"status", "error", "matches"}."""
    with tempfile.TemporaryDirectory() as d:
        args = find_args(name, Path(d))
        r = subprocess.run([str(probe), "find", *args], check=True, capture_output=True, text=True, timeout=900)
    out = {"status": None, "error": "", "matches": []}
    for line in r.stdout.splitlines():
        head, _, rest = line.partition(" ")
        if head == "status":
            out["status"] = int(rest)
        elif head == "error":
            out["error"] = rest
        elif head == "match":
            out["matches"].append([float(v) for v in rest.split()])
    return out


def run_cpp(probe: Path, scene: str | None) -> list[str]:
    """Runs the C++ probe on the scene's template (cfg1_s1) and image (or an
    empty image object for None); returns its output lines."""
    from mvkit_gb300 import workloads as W
    case = scene_case("cfg1_s1")
    wl = W.make_workload(**case["gen"])
    c, f = case["create"], case["find"]
    with tempfile.TemporaryDirectory() as d:
        tp, ip = Path(d) / "t.raw", Path(d) / "i.raw"
        tp.write_bytes(np.ascontiguousarray(wl.template).tobytes())
        ip.write_bytes(np.ascontiguousarray(wl.image).tobytes())
        args = [str(tp), str(wl.template.shape[1]), str(wl.template.shape[0]), str(c["levels"]),
                repr(float(c["angle_start"])), repr(float(c["angle_extent"])),
                str(ip) if scene else "-", str(wl.image.shape[1]), str(wl.image.shape[0]),
                repr(float(f["min_score"])), str(int(f["num_matches"]))]
        r = subprocess.run([str(probe), *args], check=True, capture_output=True, text=True, timeout=600)
    return r.stdout.splitlines()
