"""Model-file parity cases ("MVKIT_NCC 1", src/ncc_matching/persist.cpp).

Shared by make_models.py (which records the reference's files, digests and
statuses into tests/golden/models/ and models.json) and the tests.

- MODEL_FILES: templates whose reference-written model files are stored.
- Every golden case of cases.py: the SHA-256 of the reference's file bytes.
- EDITS: edits of one stored file (most re-checksummed so that they reach
  the body parser) with the status the reference's reader returns, and for
  files it accepts, the SHA-256 of the file it writes back.
"""
from __future__ import annotations

import hashlib
import math

import numpy as np

from golden.cases import CASES, make_inputs


def template_of(spec: dict):
    """(template, mask, create kwargs) of one MODEL_FILES entry."""
    if "case" in spec:
        case = CASES[spec["case"]]
        wl, mask = make_inputs(case)
        return wl.template, mask, dict(case["create"])
    rng = np.random.default_rng(spec["seed"])
    h, w = spec["shape"]
    hi = spec.get("maxval", 255)
    t = rng.integers(0, hi + 1, size=(h, w)).astype(np.uint16 if spec["dtype"] == "u16" else np.uint8)
    mask = None
    if spec.get("mask") == "ellipse":
        yy, xx = np.mgrid[0:h, 0:w]
        mask = ((((yy - (h - 1) / 2) / (h / 2)) ** 2 + ((xx - (w - 1) / 2) / (w / 2.3)) ** 2) <= 1).astype(np.uint8)
    return t, mask, dict(spec["create"])


MODEL_FILES = {
    # the tiny16 golden case: its reference model file also drives a GPU find
    "tiny16": dict(case="tiny16"),
    "masked_u8": dict(seed=31, shape=(24, 20), dtype="u8", mask="ellipse",
                      create=dict(levels=0, angle_start=-0.3, angle_extent=0.6)),
    "u16_circle": dict(seed=32, shape=(18, 22), dtype="u16", maxval=4095,
                       create=dict(levels=2, angle_start=-math.pi, angle_extent=2 * math.pi, angle_step=0.1,
                                   ignore_polarity=True)),
    "one_angle": dict(seed=33, shape=(16, 17), dtype="u8",
                      create=dict(levels=1, angle_start=-1.0, angle_extent=0.0)),
}


def sha256(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def fnv1a64(b: bytes) -> int:
    h = 14695981039346656037
    for x in b:
        h ^= x
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def split(f: bytes):
    """(magic line, checksum line, body) of a well-formed file."""
    a = f.index(b"\n")
    b = f.index(b"\n", a + 1)
    return f[:a], f[a + 1:b], f[b + 1:]


def rehash(magic: bytes, body: bytes) -> bytes:
    return magic + b"\n" + str(fnv1a64(body)).encode() + b"\n" + body


def _lines(f: bytes):
    m, _, body = split(f)
    return m, body.split(b"\n")


def _edit_line(f: bytes, index: int, fn) -> bytes:
    m, lines = _lines(f)
    lines[index] = fn(lines[index])
    return rehash(m, b"\n".join(lines))


def _field(line: bytes, k: int, value: bytes) -> bytes:
    parts = line.split(b" ")
    parts[k] = value
    return b" ".join(parts)


def _first_masked(f: bytes) -> int:
    _, lines = _lines(f)
    for i in range(3, len(lines)):
        if lines[i].startswith(b"1 "):
            return i
    raise ValueError("no masked sample")


def _bump(line: bytes, k: int, d: float) -> bytes:
    parts = line.split(b" ")
    parts[k] = repr(float(parts[k]) + d).encode()
    return b" ".join(parts)


# name -> edit of the "masked_u8" file
EDITS = {
    "version_2": lambda f: f.replace(b"MVKIT_NCC 1", b"MVKIT_NCC 2", 1),
    "bad_magic": lambda f: f.replace(b"MVKIT_NCC 1", b"MVKIT_NCX 1", 1),
    "empty": lambda f: b"",
    "header_only": lambda f: b"MVKIT_NCC 1\n",
    "checksum_blank_prefix": lambda f: (lambda m, c, b: m + b"\n  " + c + b"\n" + b)(*split(f)),
    "checksum_no_newline": lambda f: (lambda m, c, b: m + b"\n" + c + b" " + b)(*split(f)),
    "checksum_mismatch": lambda f: (lambda m, c, b: m + b"\n" + str(int(c) ^ 1).encode() + b"\n" + b)(*split(f)),
    "body_flip": lambda f: f[:-3] + bytes([f[-3] ^ 1]) + f[-2:],
    "truncated": lambda f: f[:-10],
    "truncated_rehashed": lambda f: (lambda m, c, b: rehash(m, b[:b.rstrip(b"\n").rfind(b"\n") + 1]))(*split(f)),
    "trailing_data": lambda f: (lambda m, c, b: rehash(m, b + b"0 0\n"))(*split(f)),
    "trailing_blanks": lambda f: (lambda m, c, b: rehash(m, b + b" \t\r\n\n"))(*split(f)),
    "crlf": lambda f: (lambda m, c, b: rehash(m, b.replace(b"\n", b"\r\n")))(*split(f)),
    "levels_17": lambda f: _edit_line(f, 0, lambda l: _field(l, 0, b"17")),
    "levels_negative": lambda f: _edit_line(f, 0, lambda l: _field(l, 0, b"-1")),
    "levels_too_many": lambda f: _edit_line(f, 0, lambda l: _field(l, 0, b"6")),
    "polarity_2": lambda f: _edit_line(f, 0, lambda l: _field(l, 1, b"2")),
    "angle_step_zero": lambda f: _edit_line(f, 0, lambda l: _field(l, 4, b"0")),
    "extent_negative": lambda f: _edit_line(f, 0, lambda l: _field(l, 3, b"-0.5")),
    "extent_over_2pi": lambda f: _edit_line(f, 0, lambda l: _field(l, 3, b"6.3")),
    "start_inf": lambda f: _edit_line(f, 0, lambda l: _field(l, 2, b"inf")),
    "width_huge": lambda f: _edit_line(f, 1, lambda l: _field(l, 2, b"2000000")),
    "dims_product": lambda f: _edit_line(f, 1, lambda l: _field(_field(l, 2, b"2048"), 3, b"1024")),
    "width_zero": lambda f: _edit_line(f, 1, lambda l: _field(l, 2, b"0")),
    "origin_half": lambda f: _edit_line(f, 1, lambda l: _bump(l, 0, 0.5)),
    "origin_whole": lambda f: _edit_line(f, 1, lambda l: _bump(l, 0, 3.0)),
    "origin_below": lambda f: _edit_line(f, 1, lambda l: _bump(l, 1, -30.0)),
    "centroid_off": lambda f: _edit_line(f, 2, lambda l: _bump(l, 0, 1e-3)),
    "mask_2": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 0, b"2")),
    "gray_nan": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"nan")),
    "gray_word": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"abc")),
    "gray_exponent": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"2.5e1")),
    "gray_plus": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"+" + l.split(b" ")[1].lstrip(b"-"))),
    "gray_double_plus": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"++1")),
    "mask_plus": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 0, b"+1")),
    "gray_hex": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"0x10")),
    "gray_long_integer": lambda f: _edit_line(f, _first_masked(f), lambda l: _field(l, 1, b"00000000000000000012")),
    "constant": lambda f: (lambda m, lines: rehash(m, b"\n".join(
        lines[:3] + [(_field(x, 1, b"0") if x else x) for x in lines[3:]])))(*_lines(f)),
}
EDIT_BASE = "masked_u8"
