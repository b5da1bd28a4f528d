"""Model files (WriteNccModel / ReadNccModel, src/ncc_matching/persist.cpp)
against the reference's own files and reader statuses (tests/golden/models/,
models.json, written by tests/golden/make_models.py from the compiled
reference).  Model building and files are host work: these run without a
GPU through the C ABI."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import mvkit_gb300 as mg
from mvkit_gb300 import ncc
from golden.cases import CASES, make_inputs
from golden.model_cases import EDIT_BASE, EDITS, MODEL_FILES, sha256, template_of

HERE = Path(__file__).resolve().parent
FIX = json.loads((HERE / "golden" / "models.json").read_text())
FILES = HERE / "golden" / "models"


def create(t, mask, c):
    return mg.create_ncc_model(t, c.get("levels", 0) or "auto", c["angle_start"], c["angle_extent"],
                               c.get("angle_step", 0.0) or "auto",
                               "ignore_global_polarity" if c.get("ignore_polarity") else "use_polarity", domain=mask)


@pytest.fixture(scope="module", autouse=True)
def _lib():
    try:
        mg.load()
    except mg.MvError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("name", sorted(MODEL_FILES))
def test_written_file_is_the_references(name, tmp_path):
    t, mask, c = template_of(MODEL_FILES[name])
    m = create(t, mask, c)
    want = (FILES / f"{name}.ncm").read_bytes()
    assert sha256(want) == FIX["files"][name]["sha256"]
    assert mg.serialize_ncc_model(m) == want
    path = tmp_path / f"{name}.ncm"
    mg.write_ncc_model(m, str(path))
    assert path.read_bytes() == want


@pytest.mark.parametrize("name", sorted(MODEL_FILES))
def test_read_reference_file(name):
    m = mg.read_ncc_model(str(FILES / f"{name}.ncm"))
    info = FIX["files"][name]
    lv, a0, ae, st, metric = mg.get_ncc_model_params(m)
    assert lv == info["levels"]
    c = template_of(MODEL_FILES[name])[2]
    assert a0 == c["angle_start"] and ae == c["angle_extent"]
    assert st == (0.0 if ae == 0 else info["angle_step"])
    assert metric == ("ignore_global_polarity" if c.get("ignore_polarity") else "use_polarity")
    # reading and writing back reproduces the file
    assert mg.serialize_ncc_model(m) == (FILES / f"{name}.ncm").read_bytes()


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_case_model_bytes(name):
    """Every parity case's model serialises to the reference's bytes."""
    case = CASES[name]
    wl, mask = make_inputs(case)
    m = create(wl.template, mask, case["create"])
    assert sha256(mg.serialize_ncc_model(m)) == FIX["case_sha256"][name]


@pytest.mark.parametrize("name", sorted(EDITS))
def test_reader_status_matches_reference(name):
    base = (FILES / f"{EDIT_BASE}.ncm").read_bytes()
    data = EDITS[name](base)
    want = FIX["edits"][name]
    if want["status"] == 0:
        m = mg.deserialize_ncc_model(data)
        assert sha256(mg.serialize_ncc_model(m)) == want["rewritten_sha256"]
    else:
        with pytest.raises(mg.MvError) as e:
            mg.deserialize_ncc_model(data)
        assert e.value.status == want["status"], (e.value.message, want["message"])
        assert e.value.message == want["message"]


def test_file_errors(tmp_path):
    t, mask, c = template_of(MODEL_FILES["one_angle"])
    m = create(t, mask, c)
    with pytest.raises(mg.MvError) as e:
        mg.write_ncc_model(m, str(tmp_path / "missing_dir" / "x.ncm"))
    assert e.value.status == ncc.MV_STATUS_IO_ERROR
    with pytest.raises(mg.MvError) as e:
        mg.read_ncc_model(str(tmp_path / "absent.ncm"))
    assert e.value.status == ncc.MV_STATUS_IO_ERROR
    for bad in ("", "a\0b"):
        with pytest.raises(mg.MvError) as e:
            mg.read_ncc_model(bad)
        assert e.value.status == ncc.MV_STATUS_INVALID_ARGUMENT
    with pytest.raises(mg.MvError) as e:
        mg.read_ncc_model(3)
    assert e.value.status == ncc.MV_STATUS_TYPE_MISMATCH
    # a file over the 64 MiB + 128 byte budget is refused before parsing
    big = tmp_path / "big.ncm"
    with open(big, "wb") as f:
        f.truncate(64 * 1024 * 1024 + 129)
    with pytest.raises(mg.MvError) as e:
        mg.read_ncc_model(str(big))
    assert e.value.status == ncc.MV_STATUS_LIMIT_EXCEEDED


def test_reference_reads_our_files():
    """Cross-check with the compiled reference where it exists (this
    container): its reader accepts our bytes and writes them back unchanged."""
    oracle_lib = pytest.importorskip("oracle_lib")
    ref = oracle_lib.reference("scalar")
    if ref is None:
        pytest.skip("reference build absent")
    rng = np.random.default_rng(7)
    for shape, dt in (((21, 19), np.uint8), ((20, 26), np.uint16)):
        t = rng.integers(0, 200, size=shape).astype(dt)
        ours = mg.serialize_ncc_model(mg.create_ncc_model(t, "auto", -0.7, 1.4, "auto", "use_polarity"))
        assert ref.serialize(ref.deserialize(ours)) == ours


@pytest.mark.parametrize("name", ["tiny16", "u16_circle"])
def test_reader_matches_reference_on_mutated_files(name):
    """Seeded mutations of a stored file's body (a byte replaced, a digit
    changed, a byte inserted, the body cut short), re-checksummed so that the
    parser sees them: the status, the message and, for accepted files, the
    bytes written back equal the compiled reference's reader's.  Runs where
    the reference build exists (this container)."""
    oracle_lib = pytest.importorskip("oracle_lib")
    ref = oracle_lib.reference("scalar")
    if ref is None:
        pytest.skip("reference build absent")
    from golden.model_cases import rehash, split

    magic, _, body = split((FILES / f"{name}.ncm").read_bytes())
    digits = [i for i, c in enumerate(body) if 48 <= c <= 57]
    rng = np.random.default_rng(11)

    def ours(data):
        try:
            return 0, "", mg.serialize_ncc_model(mg.deserialize_ncc_model(data))
        except mg.MvError as e:
            return e.status, e.message, None

    def theirs(data):
        try:
            return 0, "", ref.serialize(ref.deserialize(data))
        except oracle_lib.CheckerError as e:
            return e.status, e.message, None

    seen = set()
    for k in range(400):
        b = bytearray(body)
        kind = k % 4
        if kind == 0:
            b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
        elif kind == 1:
            b[digits[int(rng.integers(0, len(digits)))]] = int(rng.integers(48, 58))
        elif kind == 2:
            b.insert(int(rng.integers(0, len(b))), int(rng.choice([10, 32, 43, 45, 46, 48, 49, 101])))
        else:
            b = b[: int(rng.integers(0, len(b)))]
        data = rehash(magic, bytes(b))
        got, want = ours(data), theirs(data)
        assert got == want, (k, kind, got[:2], want[:2])
        seen.add(want[0])
    assert 0 in seen and len(seen) >= 2  # both accepted and rejected files were exercised
