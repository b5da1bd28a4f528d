"""The reference-signature C ABI (include/mvkit_gb300_mv.h, libmvkit_gb300_mv.so)
on the CPU: the library exports every declared symbol, and a C program and a
C++ program written against the reference's API print, for a table of
create / params / write / read / find calls with valid and invalid controls,
exactly what they print when linked against the reference's own compiled C
ABI (status, error code, operation, parameter, index, message, output tuples,
model file bytes; tests/golden/mv_abi.json).  No call searches an image."""
import hashlib
import json
import re
from pathlib import Path

import pytest

import mv_abi

ROOT = Path(__file__).resolve().parents[1]
FIXTURE = json.loads((ROOT / "tests" / "golden" / "mv_abi.json").read_text())


@pytest.fixture(scope="module")
def ours():
    from mvkit_gb300 import build
    build.build()
    assert mv_abi.OURS.exists()
    return mv_abi.OURS


def test_library_exports_every_declared_mv_symbol(ours):
    import ctypes
    names = sorted(set(re.findall(r"MV_API\s+MvStatus\s+(mv_\w+)\s*\(", (ROOT / "include" / "mvkit_gb300_mv.h").read_text())))
    for n in ("mv_create_ncc_model", "mv_find_ncc_model", "mv_find_ncc_models", "mv_get_ncc_model_params",
              "mv_read_ncc_model", "mv_write_ncc_model", "mv_gen_image1", "mv_get_last_error"):
        assert n in names
    lib = ctypes.CDLL(str(ours))
    for n in names:
        assert hasattr(lib, n), n


def test_cases_equal_the_reference_c_abi(ours, tmp_path):
    probe = mv_abi.compile_probe(ours, tmp_path / "probe")
    work = tmp_path / "cases"
    work.mkdir()
    lines, model = mv_abi.run_cases(probe, work)
    want = FIXTURE["cases"]
    assert len(lines) == len(want)
    for got, exp in zip(lines, want):
        assert got == exp
    # the model file is the reference's byte for byte
    assert hashlib.sha256(model).hexdigest() == FIXTURE["model_file_sha256"]


@pytest.mark.skipif(not mv_abi.REFERENCE.exists(), reason="reference C ABI not built here (make -C oracle capi)")
def test_cases_equal_the_reference_c_abi_live(ours, tmp_path):
    a = mv_abi.compile_probe(ours, tmp_path / "ours")
    b = mv_abi.compile_probe(mv_abi.REFERENCE, tmp_path / "ref")
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    la, ma = mv_abi.run_cases(a, tmp_path / "a")
    lb, mb = mv_abi.run_cases(b, tmp_path / "b")
    assert la == lb
    assert ma == mb


def test_cpp_functions_on_an_empty_image(ours, tmp_path):
    probe = mv_abi.compile_cpp_probe(ours, tmp_path / "cpp")
    assert mv_abi.run_cpp(probe, None) == FIXTURE["cpp"]["empty"]


def test_raw_find_controls_checked_like_the_reference():
    """The raw ABI's single-model find rejects what NccControls rejects
    (AngleExtent above 2 pi, negative levels) and reads lowest level 0 as 1,
    before any device work."""
    import ctypes as C
    import numpy as np
    import mvkit_gb300 as mg
    from mvkit_gb300 import workloads as W
    lib = mg.load()
    model = mg.create_ncc_model(W.make_workload(3, 128, 128, 32, 1).template, 2, 0.0, 0.0, "auto", "use_polarity")
    img = np.zeros((64, 64), np.uint8)
    out = np.zeros(4)
    cnt = C.c_int64()
    dp = out.ctypes.data_as(C.POINTER(C.c_double))

    def find(extent, highest, lowest, handle):
        return lib.mvg_find_ncc_model(img.ctypes.data, 0, 64, 64, 64, 0, None, handle, 0.0, extent, 0.5, 1, 0.5, 1,
                                      highest, lowest, dp, dp, dp, dp, 1, C.byref(cnt), None)
    assert find(7.0, 0, 1, model.handle) == -1 and b"AngleExtent" in lib.mvg_last_error()
    assert find(0.1, -1, 1, model.handle) == -1 and b"NumLevels" in lib.mvg_last_error()
    assert find(0.1, 0, -1, model.handle) == -1 and b"NumLevels" in lib.mvg_last_error()
    # lowest 0 passes the control checks (a null model handle fails next, before any device work)
    assert find(0.1, 0, 0, None) == -1 and b"not an NCC model" in lib.mvg_last_error()
