"""Python mirror of mvkit's NCC matching operators over libmvkit_gb300.so.

Names, argument meaning and error behaviour follow the reference C API
(src/c_api/ncc_matching_api.cpp): each control accepts one value (a scalar
or a one-element sequence), strings are checked as the reference checks them
("auto", "true"/"false", metric names), and failures raise MvError carrying
the reference's MvStatus code.  The search itself runs on the GPU through
the C ABI declared in include/mvkit_gb300_ncc.h; there is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path
from typing import Sequence

import numpy as np

from . import build as _build

# MvStatus (include/mvkit/c/mv_status.h:12-24)
MV_STATUS_OK = 0
MV_STATUS_INVALID_ARGUMENT = -1
MV_STATUS_TYPE_MISMATCH = -3
MV_STATUS_OUT_OF_MEMORY = -5
MV_STATUS_UNSUPPORTED = -6
MV_STATUS_INVALID_STATE = -7
MV_STATUS_IO_ERROR = -100
MV_STATUS_DECODE_ERROR = -101
MV_STATUS_LIMIT_EXCEEDED = -103
MV_STATUS_INTERNAL_ERROR = -1000

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class MvError(RuntimeError):
    def __init__(self, status: int, message: str, operator: str = ""):
        super().__init__(f"{operator}: status {status}: {message}" if operator else f"status {status}: {message}")
        self.status = status
        self.message = message


_LIB = None


def library_path() -> Path:
    return _build.LIB


def load() -> C.CDLL:
    """Loads the in-tree CUDA library; raises when it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise MvError(MV_STATUS_INTERNAL_ERROR, f"CUDA extension missing: {path} (run mvkit_gb300.build.build())")
    lib = C.CDLL(str(path))
    lib.mvg_create_ncc_model.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, _u8p, C.c_int32,
                                         C.c_double, C.c_double, C.c_double, C.c_int32, C.POINTER(C.c_void_p)]
    lib.mvg_get_ncc_model_params.argtypes = [C.c_void_p, _i32p, _dp, _dp, _dp, _i32p]
    lib.mvg_clear_ncc_model.argtypes = [C.c_void_p]
    lib.mvg_find_ncc_model.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p,
                                       C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double, C.c_int32,
                                       C.c_int32, C.c_int32, _dp, _dp, _dp, _dp, C.c_int64, _i64p, C.c_void_p]
    lib.mvg_find_ncc_model_stage.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                             C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double,
                                             C.c_int32, C.c_int32, C.c_int32, C.c_int32, _dp, C.c_int64, _i64p]
    lib.mvg_ncc_pyramid_level.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                          C.c_int32, C.c_int32, _fp, C.c_int64, _dp]
    lib.mvg_write_ncc_model.argtypes = [C.c_void_p, C.c_char_p]
    lib.mvg_read_ncc_model.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    lib.mvg_serialize_ncc_model.argtypes = [C.c_void_p, C.c_char_p, C.c_int64, _i64p]
    lib.mvg_deserialize_ncc_model.argtypes = [C.c_char_p, C.c_int64, C.POINTER(C.c_void_p)]
    lib.mvg_find_ncc_models.argtypes = ([C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                        C.c_void_p, C.c_void_p, C.c_int64] + [C.c_void_p, C.c_int64] * 7 +
                                       [C.c_void_p] * 5 + [C.c_int64, _i64p, C.c_void_p])
    lib.mvg_find_ncc_models_batch.argtypes = ([C.c_void_p] * 5 + [C.c_int64, C.c_int32, C.c_void_p, C.c_void_p,
                                                                   C.c_int64] +
                                             [C.c_void_p, C.c_int64] * 7 + [C.c_int32] + [C.c_void_p] * 5 +
                                             [C.c_int64, C.c_void_p, C.c_void_p, _i64p])
    lib.mvg_last_error.restype = C.c_char_p
    lib.mvg_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    lib.mvg_host_free.argtypes = [C.c_void_p]
    lib.mvg_device_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    lib.mvg_device_free.argtypes = [C.c_void_p]
    lib.mvg_copy_to_device.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    lib.mvg_profile_enable.argtypes = [C.c_int32]
    lib.mvg_profile_reset.argtypes = []
    lib.mvg_profile_read.argtypes = [C.c_int32, C.POINTER(C.c_char_p), _dp, _i64p, _dp, _i64p]
    for name in ("mvg_profile_enable", "mvg_profile_reset", "mvg_profile_read"):
        getattr(lib, name).restype = C.c_int32
    for name in ("mvg_create_ncc_model", "mvg_get_ncc_model_params", "mvg_clear_ncc_model", "mvg_find_ncc_model",
                 "mvg_find_ncc_model_stage", "mvg_ncc_pyramid_level", "mvg_host_alloc", "mvg_host_free",
                 "mvg_device_alloc", "mvg_device_free", "mvg_copy_to_device", "mvg_write_ncc_model", "mvg_read_ncc_model",
                 "mvg_serialize_ncc_model", "mvg_deserialize_ncc_model", "mvg_find_ncc_models",
                 "mvg_find_ncc_models_batch"):
        getattr(lib, name).restype = C.c_int32
    _LIB = lib
    return lib


def _check(status: int, op: str) -> None:
    if status != 0:
        msg = (load().mvg_last_error() or b"").decode(errors="replace")
        raise MvError(status, msg, op)


# ---------------------------------------------------------------- controls
def _values(x, op: str, name: str) -> list:
    if isinstance(x, (list, tuple, np.ndarray)):
        return list(x)
    return [x]


def _one(x, op: str, name: str):
    v = _values(x, op, name)
    if len(v) != 1:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, f"{name}: exactly one value required", op)
    return v[0]


def _number(v, op: str, name: str) -> float:
    if isinstance(v, (bool, np.bool_)) or not isinstance(v, (int, float, np.integer, np.floating)):
        raise MvError(MV_STATUS_TYPE_MISMATCH, f"{name}: numeric control value required", op)
    return float(v)


def _integer(v, op: str, name: str) -> int:
    if isinstance(v, (bool, np.bool_)):
        raise MvError(MV_STATUS_TYPE_MISMATCH, f"{name}: integer control value required", op)
    if isinstance(v, (int, np.integer)):
        return int(v)
    if isinstance(v, (float, np.floating)):
        if math.isfinite(v) and float(v).is_integer():
            return int(v)
        raise MvError(MV_STATUS_INVALID_ARGUMENT, f"{name}: integer-valued control required", op)
    raise MvError(MV_STATUS_TYPE_MISMATCH, f"{name}: integer control value required", op)


def _image(img, op: str, name: str):
    a = np.asarray(img)
    if a.ndim != 2 or a.dtype not in (np.uint8, np.uint16):
        raise MvError(MV_STATUS_TYPE_MISMATCH, f"{name}: one byte or uint2 channel required", op)
    if a.strides[1] != a.itemsize:
        a = np.ascontiguousarray(a)
    return a, (1 if a.dtype == np.uint16 else 0)


class NccModel:
    """Handle of a model on the GPU (the reference's NCC model handle)."""

    def __init__(self, handle: C.c_void_p):
        self.handle = handle

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    def clear(self):
        if self.handle:
            load().mvg_clear_ncc_model(self.handle)
            self.handle = None


def create_ncc_model(template, num_levels="auto", angle_start=0.0, angle_extent=0.0, angle_step="auto",
                     metric="use_polarity", domain=None) -> NccModel:
    """CreateNccModel (src/c_api/ncc_matching_api.cpp:29-66)."""
    op = "create_ncc_model"
    t, typ = _image(template, op, "Template")
    lv = _one(num_levels, op, "NumLevels")
    if isinstance(lv, str):
        if lv != "auto":
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "NumLevels: expected auto", op)
        levels = 0
    else:
        levels = _integer(lv, op, "NumLevels")
        if levels < 0 or levels > 16:
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "levels must be 0..16 or auto", op)
    start = _number(_one(angle_start, op, "AngleStart"), op, "AngleStart")
    extent = _number(_one(angle_extent, op, "AngleExtent"), op, "AngleExtent")
    if not math.isfinite(start) or not math.isfinite(extent):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "finite control value required", op)
    st = _one(angle_step, op, "AngleStep")
    if isinstance(st, str):
        if st != "auto":
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "AngleStep: expected auto", op)
        step = 0.0
    else:
        step = _number(st, op, "AngleStep")
        if not math.isfinite(step):
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "finite control value required", op)
        if step < 0 or step > math.pi / 16:
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "angle step must be in [0,pi/16] or auto", op)
    m = _one(metric, op, "Metric")
    if not isinstance(m, str):
        raise MvError(MV_STATUS_TYPE_MISMATCH, "Metric: string control value required", op)
    if m == "ignore_global_polarity":
        metric_id = 1
    elif m == "use_polarity":
        metric_id = 0
    else:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "unsupported NCC metric", op)
    d = None
    if domain is not None:
        d = np.ascontiguousarray(np.asarray(domain) != 0, dtype=np.uint8)
        if d.shape != t.shape:
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "domain must match the template size", op)
    h = C.c_void_p()
    lib = load()
    _check(lib.mvg_create_ncc_model(t.ctypes.data, typ, t.shape[1], t.shape[0], t.strides[0],
                                    d.ctypes.data_as(_u8p) if d is not None else None, levels, start, extent, step,
                                    metric_id, C.byref(h)), op)
    return NccModel(h)


def get_ncc_model_params(model: NccModel):
    """GetNccModelParams (src/c_api/ncc_matching_api.cpp:85-96)."""
    lv = C.c_int32()
    a0, a1, a2 = C.c_double(), C.c_double(), C.c_double()
    mt = C.c_int32()
    _check(load().mvg_get_ncc_model_params(model.handle, C.byref(lv), C.byref(a0), C.byref(a1), C.byref(a2),
                                           C.byref(mt)), "get_ncc_model_params")
    return (lv.value, a0.value, a1.value, a2.value, "ignore_global_polarity" if mt.value else "use_polarity")


def _file_name(name, op: str) -> bytes:
    """FileName control: exactly one nonempty string without NUL
    (src/c_api/ncc_matching_api.cpp:77-83)."""
    v = _one(name, op, "FileName")
    if isinstance(v, Path):
        v = str(v)
    if not isinstance(v, str):
        raise MvError(MV_STATUS_TYPE_MISMATCH, "FileName: string control value required", op)
    if not v or "\0" in v:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "nonempty file name without NUL required", op)
    return v.encode("utf-8")


def write_ncc_model(model: NccModel, file_name) -> None:
    """WriteNccModel (src/c_api/ncc_matching_api.cpp:97-99): the reference's
    "MVKIT_NCC 1" model file, byte-identical to the reference's."""
    op = "write_ncc_model"
    lib = load()
    _check(lib.mvg_write_ncc_model(model.handle, _file_name(file_name, op)), op)


def read_ncc_model(file_name) -> NccModel:
    """ReadNccModel (src/c_api/ncc_matching_api.cpp:101-110)."""
    op = "read_ncc_model"
    lib = load()
    h = C.c_void_p()
    _check(lib.mvg_read_ncc_model(_file_name(file_name, op), C.byref(h)), op)
    return NccModel(h)


def serialize_ncc_model(model: NccModel) -> bytes:
    """The model file's bytes (what write_ncc_model writes)."""
    op = "serialize_ncc_model"
    lib = load()
    n = C.c_int64()
    _check(lib.mvg_serialize_ncc_model(model.handle, None, 0, C.byref(n)), op)
    buf = C.create_string_buffer(max(1, n.value))
    _check(lib.mvg_serialize_ncc_model(model.handle, buf, n.value, C.byref(n)), op)
    return buf.raw[:n.value]


def deserialize_ncc_model(data: bytes) -> NccModel:
    """A model from model-file bytes (what read_ncc_model reads)."""
    op = "deserialize_ncc_model"
    lib = load()
    b = bytes(data)
    h = C.c_void_p()
    _check(lib.mvg_deserialize_ncc_model(b, len(b), C.byref(h)), op)
    return NccModel(h)


def _find_controls(op, angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel, num_levels):
    """Single-model NccControls (src/c_api/ncc_matching_api.cpp:126-162)."""
    vals = {}
    for name, x in (("AngleStart", angle_start), ("AngleExtent", angle_extent), ("MinScore", min_score),
                    ("NumMatches", num_matches), ("MaxOverlap", max_overlap), ("SubPixel", subpixel)):
        vals[name] = _one(x, op, name)

    def number(name, lo, hi):
        v = _number(vals[name], op, name)
        if not math.isfinite(v) or v < lo or v > hi:
            raise MvError(MV_STATUS_INVALID_ARGUMENT, f"{name}: numeric control outside allowed range", op)
        return v

    start = number("AngleStart", -1.7976931348623157e308, 1.7976931348623157e308)
    extent = number("AngleExtent", 0.0, 6.28318530717958647692)
    score = number("MinScore", 0.0, 1.0)
    overlap = number("MaxOverlap", 0.0, 1.0)
    quota = _integer(vals["NumMatches"], op, "NumMatches")
    if quota < 0:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "match count must be nonnegative", op)
    mode = vals["SubPixel"]
    if not isinstance(mode, str):
        raise MvError(MV_STATUS_TYPE_MISMATCH, "SubPixel: string control value required", op)
    if mode not in ("true", "false"):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "expected true or false", op)
    lv = _values(num_levels, op, "NumLevels")
    if len(lv) not in (1, 2):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "highest level or shared/per-model level pairs required", op)
    highest = _integer(lv[0], op, "NumLevels")
    lowest = _integer(lv[1], op, "NumLevels") if len(lv) == 2 else 1
    if highest < 0 or highest > 2**31 - 1 or lowest < 0 or lowest > 2**31 - 1:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "invalid highest/lowest level pair", op)
    return start, extent, score, quota, overlap, 1 if mode == "true" else 0, highest, max(1, lowest)


class DeviceImage:
    """An image already resident in device memory (uint8/uint16, dense rows)."""

    def __init__(self, array: np.ndarray):
        a, typ = _image(array, "device_image", "Image")
        self.shape = a.shape
        self.dtype = a.dtype
        self.type = typ
        self.stride = a.strides[0]
        self.nbytes = a.nbytes
        p = C.c_void_p()
        _check(load().mvg_device_alloc(a.nbytes, C.byref(p)), "device_image")
        self.ptr = p
        _check(load().mvg_copy_to_device(p, a.ctypes.data, a.nbytes), "device_image")

    def __del__(self):
        try:
            if self.ptr:
                load().mvg_device_free(self.ptr)
                self.ptr = None
        except Exception:
            pass


def _domain(domain, shape, op: str):
    """The search image's domain (the reference image object's reduced
    domain) as a contiguous byte mask of the image's shape, or None."""
    if domain is None:
        return None
    d = np.ascontiguousarray(np.asarray(domain) != 0, dtype=np.uint8)
    if d.shape != tuple(shape):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "domain must match the image size", op)
    return d


def find_ncc_model(image, model: NccModel, angle_start, angle_extent, min_score, num_matches, max_overlap,
                   subpixel, num_levels, stream=None, domain=None):
    """FindNccModel (src/c_api/ncc_matching_api.cpp:178-190).

    image: 2-D uint8/uint16 array in host memory, or a DeviceImage.
    domain: the image's reduced domain (ROI) as a mask of the image's shape,
    nonzero inside; None = the whole image.
    Returns (Row, Column, Angle, Score) as float64 arrays in the operator's
    edge-centred convention.  An empty image returns empty outputs."""
    op = "find_ncc_model"
    ctl = _find_controls(op, angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel, num_levels)
    if not isinstance(model, NccModel) or not model.handle:
        raise MvError(MV_STATUS_TYPE_MISMATCH, "ModelID: NCC model handle required", op)
    if isinstance(image, DeviceImage):
        ptr, typ, (h, w), stride, loc = image.ptr, image.type, image.shape, image.stride, 1
    else:
        a, typ = _image(image, op, "Image")
        if a.size == 0:
            e = np.zeros(0)
            return e, e.copy(), e.copy(), e.copy()
        ptr, (h, w), stride, loc = a.ctypes.data, a.shape, a.strides[0], 0
    dom = _domain(domain, (h, w), op)
    cap = 64 if ctl[3] == 0 else int(ctl[3])
    lib = load()
    while True:
        out = [np.zeros(cap) for _ in range(4)]
        cnt = C.c_int64()
        _check(lib.mvg_find_ncc_model(ptr, typ, w, h, stride, loc, None if dom is None else dom.ctypes.data,
                                      model.handle, *ctl,
                                      *[o.ctypes.data_as(_dp) for o in out], cap, C.byref(cnt),
                                      C.c_void_p(stream) if stream else None), op)
        if cnt.value <= cap:
            return tuple(o[: cnt.value] for o in out)
        cap = int(cnt.value)


def _models_controls(op, models, angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel,
                     num_levels):
    """Model handles and control arrays of FindNccModels (NccControls,
    src/c_api/ncc_matching_api.cpp:126-162): (models, ctypes handle array,
    control arrays in C-ABI order, match quotas)."""
    ms = list(models) if isinstance(models, (list, tuple)) else [models]
    if not ms or len(ms) > 4096:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "one model or a nonempty model array (maximum 4096) required", op)
    for m in ms:
        if not isinstance(m, NccModel) or not m.handle:
            raise MvError(MV_STATUS_TYPE_MISMATCH, "control handle is not an NCC model", op)
    n = len(ms)

    def per(x, name):
        v = _values(x, op, name)
        if len(v) not in (1, n):
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "one value or one value per model required", op)
        return v

    def numbers(x, name):
        out = []
        for v in per(x, name):
            out.append(_number(v, op, name))
        return np.array(out, dtype=np.float64)

    starts, extents = numbers(angle_start, "AngleStart"), numbers(angle_extent, "AngleExtent")
    scores, overlaps = numbers(min_score, "MinScore"), numbers(max_overlap, "MaxOverlap")
    quotas = np.array([_integer(v, op, "NumMatches") for v in per(num_matches, "NumMatches")], dtype=np.int64)
    modes = []
    for v in per(subpixel, "SubPixel"):
        if not isinstance(v, str):
            raise MvError(MV_STATUS_TYPE_MISMATCH, "SubPixel: string control value required", op)
        if v not in ("true", "false"):
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "expected true or false", op)
        modes.append(1 if v == "true" else 0)
    modes = np.array(modes, dtype=np.int32)
    lv = _values(num_levels, op, "NumLevels")
    if len(lv) not in (1, 2, n, 2 * n):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "highest level or shared/per-model level pairs required", op)
    levels = np.array([_integer(v, op, "NumLevels") for v in lv], dtype=np.int64)
    if (levels < 0).any() or (levels > 2**31 - 1).any():
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "invalid highest/lowest level pair", op)
    levels = levels.astype(np.int32)
    ids = (C.c_void_p * n)(*[m.handle for m in ms])
    return ms, ids, (starts, extents, scores, quotas, overlaps, modes, levels), quotas


def find_ncc_models(image, models, angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel,
                    num_levels, stream=None, domain=None):
    """FindNccModels (src/c_api/ncc_matching_api.cpp:191-201).

    models: one NccModel or a sequence of 1..4096.  Each control takes one
    value (shared) or one per model; num_levels takes 1, 2, len(models) or
    2*len(models) values.  Returns (Row, Column, Angle, Score, Model), Model
    being the index into `models`."""
    op = "find_ncc_models"
    ms, ids, arrs, quotas = _models_controls(op, models, angle_start, angle_extent, min_score, num_matches,
                                             max_overlap, subpixel, num_levels)
    n = len(ms)
    if isinstance(image, DeviceImage):
        ptr, typ, (h, w), stride, loc = image.ptr, image.type, image.shape, image.stride, 1
    else:
        a, typ = _image(image, op, "Image")
        if a.size == 0:
            e = np.zeros(0)
            return e, e.copy(), e.copy(), e.copy(), np.zeros(0, dtype=np.int64)
        ptr, (h, w), stride, loc = a.ctypes.data, a.shape, a.strides[0], 0
    dom = _domain(domain, (h, w), op)
    lib = load()
    cap = max(64, int(quotas.sum()))
    args = []
    for arr in arrs:
        args += [arr.ctypes.data, len(arr)]
    while True:
        out = [np.zeros(cap) for _ in range(4)] + [np.zeros(cap, dtype=np.int64)]
        cnt = C.c_int64()
        _check(lib.mvg_find_ncc_models(ptr, typ, w, h, stride, loc, None if dom is None else dom.ctypes.data, ids,
                                       n, *args,
                                       *[o.ctypes.data for o in out], cap, C.byref(cnt),
                                       C.c_void_p(stream) if stream else None), op)
        if cnt.value <= cap:
            return tuple(o[: cnt.value] for o in out)
        cap = int(cnt.value)


def find_ncc_models_batch(images, models, angle_start, angle_extent, min_score, num_matches, max_overlap,
                          subpixel, num_levels, domains=None, workers: int = 8, raise_errors: bool = True):
    """FindNccModels over a batch of images of any sizes, several finds in
    flight on the library's own host threads (mvg_find_ncc_models_batch).

    images: 2-D uint8/uint16 host arrays, or DeviceImage objects (not mixed).
    domains: None, or one mask (or None) per image.  Controls as for
    find_ncc_models, shared by all images.  Returns one entry per image:
    (Row, Column, Angle, Score, Model) as find_ncc_models returns it, or,
    with raise_errors=False, the MvError of an image that failed.  With
    raise_errors=True the first failed image's error is raised."""
    op = "find_ncc_models_batch"
    imgs = list(images)
    ms, ids, arrs, quotas = _models_controls(op, models, angle_start, angle_extent, min_score, num_matches,
                                             max_overlap, subpixel, num_levels)
    if isinstance(workers, bool) or not isinstance(workers, (int, np.integer)) or not 1 <= int(workers) <= 256:
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "workers must be 1..256", op)
    n_img = len(imgs)
    if n_img == 0:
        return []
    on_device = [isinstance(x, DeviceImage) for x in imgs]
    if any(on_device) and not all(on_device):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "images must all be in host or all in device memory", op)
    keep, ptrs, types, ws, hs, strides = [], [], [], [], [], []
    for x in imgs:
        if isinstance(x, DeviceImage):
            ptrs.append(x.ptr.value)
            types.append(x.type)
            h, w = x.shape
            strides.append(x.stride)
        else:
            a, typ = _image(x, op, "Image")
            keep.append(a)
            ptrs.append(a.ctypes.data)
            types.append(typ)
            h, w = a.shape
            strides.append(a.strides[0])
        hs.append(h)
        ws.append(w)
    dom_ptrs = None
    if domains is not None:
        ds = list(domains)
        if len(ds) != n_img:
            raise MvError(MV_STATUS_INVALID_ARGUMENT, "one domain (or None) per image required", op)
        dom_ptrs = (C.c_void_p * n_img)()
        for i, d in enumerate(ds):
            m = _domain(d, (hs[i], ws[i]), op)
            if m is not None:
                keep.append(m)
                dom_ptrs[i] = m.ctypes.data
    c_imgs = (C.c_void_p * n_img)(*ptrs)
    c_types = np.array(types, dtype=np.int32)
    c_w, c_h, c_s = (np.array(v, dtype=np.int64) for v in (ws, hs, strides))
    args = []
    for arr in arrs:
        args += [arr.ctypes.data, len(arr)]
    lib = load()
    per_image = max(16, int(quotas.sum()))
    cap = per_image * n_img
    offsets = np.zeros(n_img + 1, dtype=np.int64)
    statuses = np.zeros(n_img, dtype=np.int32)
    while True:
        out = [np.zeros(cap) for _ in range(4)] + [np.zeros(cap, dtype=np.int64)]
        cnt = C.c_int64()
        st = lib.mvg_find_ncc_models_batch(c_imgs, c_types.ctypes.data, c_w.ctypes.data, c_h.ctypes.data,
                                           c_s.ctypes.data, n_img, 1 if on_device[0] else 0, dom_ptrs, ids,
                                           len(ms), *args, int(workers),
                                           *[o.ctypes.data for o in out], cap, offsets.ctypes.data,
                                           statuses.ctypes.data, C.byref(cnt))
        if st != 0 and (raise_errors or not statuses.any()):
            _check(st, op)
        if cnt.value <= cap:
            break
        cap = int(cnt.value)
    results = []
    for i in range(n_img):
        if statuses[i] != 0:
            results.append(MvError(int(statuses[i]), f"image {i} failed", op))
            continue
        a, b = int(offsets[i]), int(offsets[i + 1])
        results.append(tuple(o[a:b].copy() for o in out))
    return results


def ncc_score_gradient(image, model: NccModel, poses, stream=None):
    """NCC of the model's unrotated level-0 raster under similarity poses and
    its gradient (scale degree of freedom; no counterpart in the reference).

    poses: (n, 4) float64 rows (row, column, angle, scale) in the matcher's
    pixel-centre image coordinates of the model origin.  Returns (score (n,),
    gradient (n, 4)): d score / d (row, column, angle, scale)."""
    op = "ncc_score_gradient"
    if not isinstance(model, NccModel) or not model.handle:
        raise MvError(MV_STATUS_TYPE_MISMATCH, "ModelID: NCC model handle required", op)
    p = np.ascontiguousarray(np.asarray(poses, dtype=np.float64).reshape(-1, 4))
    if isinstance(image, DeviceImage):
        ptr, typ, (h, w), stride, loc = image.ptr, image.type, image.shape, image.stride, 1
    else:
        a, typ = _image(image, op, "Image")
        ptr, (h, w), stride, loc = a.ctypes.data, a.shape, a.strides[0], 0
    n = p.shape[0]
    score = np.zeros(n)
    grad = np.zeros((n, 4))
    lib = load()
    lib.mvg_ncc_score_gradient.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                           C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mvg_ncc_score_gradient.restype = C.c_int32
    _check(lib.mvg_ncc_score_gradient(ptr, typ, w, h, stride, loc, model.handle, p.ctypes.data, n, score.ctypes.data,
                                      grad.ctypes.data, C.c_void_p(stream) if stream else None), op)
    return score, grad


def parabola_vertex_offsets(sm, s0, sp):
    """Vertex positions, in steps and clipped to [-1, 1], of the parabolas
    through (-1, sm), (0, s0), (1, sp); 0 where a value is not finite or the
    parabola does not open downwards."""
    sm, s0, sp = (np.asarray(v, dtype=np.float64) for v in (sm, s0, sp))
    den = sm - 2 * s0 + sp
    ok = np.isfinite(sm) & np.isfinite(sp) & np.isfinite(s0) & (den < 0)
    off = np.where(ok, 0.5 * (sm - sp) / np.where(ok, den, -1.0), 0.0)
    return np.clip(off, -1.0, 1.0)


def ncc_quadratic_peak_fit(image, model: NccModel, poses, steps, stream=None):
    """Quadratic peak fitting of similarity poses (row, column, angle, scale),
    the plain form of sub-sample pose estimation kept beside the Gauss-Newton
    refinements: per degree of freedom a parabola through the NCC at the pose
    and at pose -/+ step (the scores of ncc_score_gradient, on the GPU); the
    vertex offset, clipped to one step, moves that degree of freedom.  The
    four fits are separable (each from the unmoved pose).  steps: (row,
    column, angle, scale) sampling steps, e.g. (1, 1, the model's angle step,
    0.02).  Returns (fitted poses (n, 4), score at them (n,))."""
    p = np.array(np.asarray(poses, dtype=np.float64).reshape(-1, 4), copy=True)
    n = p.shape[0]
    if n == 0:
        return p, np.zeros(0)
    steps = np.asarray(steps, dtype=np.float64).reshape(4)
    probe = np.repeat(p[:, None, :], 9, axis=1)  # centre, then -/+ per DOF
    for d in range(4):
        probe[:, 1 + 2 * d, d] -= steps[d]
        probe[:, 2 + 2 * d, d] += steps[d]
    sc, _ = ncc_score_gradient(image, model, probe.reshape(-1, 4), stream=stream)
    sc = sc.reshape(n, 9)
    s0 = sc[:, 0]
    for d in range(4):
        p[:, d] += parabola_vertex_offsets(sc[:, 1 + 2 * d], s0, sc[:, 2 + 2 * d]) * steps[d]
    score, _ = ncc_score_gradient(image, model, p, stream=stream)
    return p, score


def ncc_refine_similarity(image, model: NccModel, poses, iterations: int = 20, stream=None):
    """Gauss-Newton refinement of similarity poses (row, column, angle,
    scale) on the NCC of ncc_score_gradient.  Returns (refined poses (n, 4),
    score (n,))."""
    op = "ncc_refine_similarity"
    if not isinstance(model, NccModel) or not model.handle:
        raise MvError(MV_STATUS_TYPE_MISMATCH, "ModelID: NCC model handle required", op)
    p = np.array(np.asarray(poses, dtype=np.float64).reshape(-1, 4), copy=True, order="C")
    if isinstance(image, DeviceImage):
        ptr, typ, (h, w), stride, loc = image.ptr, image.type, image.shape, image.stride, 1
    else:
        a, typ = _image(image, op, "Image")
        ptr, (h, w), stride, loc = a.ctypes.data, a.shape, a.strides[0], 0
    n = p.shape[0]
    score = np.zeros(n)
    lib = load()
    lib.mvg_ncc_refine_similarity.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                              C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]
    lib.mvg_ncc_refine_similarity.restype = C.c_int32
    _check(lib.mvg_ncc_refine_similarity(ptr, typ, w, h, stride, loc, model.handle, p.ctypes.data, n,
                                         int(iterations), score.ctypes.data, C.c_void_p(stream) if stream else None),
           op)
    return p, score


def find_ncc_model_stage(image, model: NccModel, angle_start, angle_extent, min_score, num_matches, max_overlap,
                         subpixel, num_levels, stage: int, domain=None) -> np.ndarray:
    """Candidate list of an internal stage (n x 4: row, column, angle, score;
    pixel-centre convention of mv::ncc_matching::find)."""
    op = "find_ncc_model"
    ctl = _find_controls(op, angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel, num_levels)
    a, typ = _image(image, op, "Image")
    cap = 20000
    dom = _domain(domain, a.shape, op)
    while True:
        out = np.zeros((cap, 4))
        cnt = C.c_int64()
        _check(load().mvg_find_ncc_model_stage(a.ctypes.data, typ, a.shape[1], a.shape[0], a.strides[0], 0,
                                               None if dom is None else dom.ctypes.data, model.handle, *ctl,
                                               int(stage), out.ctypes.data_as(_dp), cap, C.byref(cnt)), op)
        if cnt.value <= cap:
            return out[: cnt.value].copy()
        cap = int(cnt.value)


def pyramid_level(image, model: NccModel, highest_level: int, level: int):
    """Integer pyramid level (sums of 4^level pixels) and geometry."""
    a, typ = _image(image, "pyramid", "Image")
    out = np.zeros(a.size + 16, dtype=np.float32)
    geom = np.zeros(5)
    _check(load().mvg_ncc_pyramid_level(a.ctypes.data, typ, a.shape[1], a.shape[0], a.strides[0], model.handle,
                                        int(highest_level), int(level), out.ctypes.data_as(_fp), out.size,
                                        geom.ctypes.data_as(_dp)), "pyramid")
    w, h = int(geom[0]), int(geom[1])
    return out[: w * h].reshape(h, w).copy(), geom


class PinnedBuffer:
    """Page-locked host buffer (for host-to-device uploads at full DMA speed)."""

    def __init__(self, shape, dtype):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        _check(load().mvg_host_alloc(self.nbytes, C.byref(p)), "host_alloc")
        self.ptr = p
        self.array = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(self.nbytes,)).view(dtype).reshape(shape)

    def __del__(self):
        try:
            if self.ptr:
                load().mvg_host_free(self.ptr)
                self.ptr = None
        except Exception:
            pass


PROFILE_STAGES = 13


def ncc_model_raster(model: NccModel, level: int, index: int = 0) -> dict:
    """One FP64 raster of the model as its build made it (the Patch of
    src/ncc_matching/model.hpp:30-43): level >= 0 and index select the
    rotated raster of that level and trained angle, level < 0 the unrotated
    level-0 raster.  Returns angle, origin_row, origin_column, weight_sum
    and the rows, cols and weights arrays."""
    op = "ncc_model_raster"
    if not isinstance(model, NccModel) or not model.handle:
        raise MvError(MV_STATUS_TYPE_MISMATCH, "ModelID: NCC model handle required", op)
    lib = load()
    f = lib.mvg_ncc_model_raster
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                  _i64p]
    f.restype = C.c_int32
    meta = np.zeros(4)
    cnt = C.c_int64()
    _check(f(model.handle, int(level), int(index), None, None, None, 0, meta.ctypes.data, C.byref(cnt)), op)
    n = int(cnt.value)
    rows, cols, w = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n)
    _check(f(model.handle, int(level), int(index), rows.ctypes.data, cols.ctypes.data, w.ctypes.data, n,
             meta.ctypes.data, C.byref(cnt)), op)
    return dict(angle=meta[0], origin_row=meta[1], origin_column=meta[2], weight_sum=meta[3], rows=rows, cols=cols,
                weights=w)


def set_model_build(where: str) -> None:
    """'device' (default): models' rotated rasters are built on the GPU when
    one is present; 'host': in FP64 on the CPU.  Same weights bit for bit."""
    if where not in ("device", "host"):
        raise MvError(MV_STATUS_INVALID_ARGUMENT, "model build must be 'device' or 'host'", "set_model_build")
    lib = load()
    lib.mvg_set_model_build.argtypes = [C.c_int32]
    lib.mvg_set_model_build.restype = C.c_int32
    _check(lib.mvg_set_model_build(0 if where == "device" else 1), "set_model_build")


def model_tables_digest(model: NccModel) -> int:
    """FNV-1a 64 digest of the model's find tables (equal = bit-identical)."""
    lib = load()
    lib.mvg_ncc_model_tables_digest.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    lib.mvg_ncc_model_tables_digest.restype = C.c_int32
    d = C.c_uint64()
    _check(lib.mvg_ncc_model_tables_digest(model.handle, C.byref(d)), "model_tables_digest")
    return d.value


def set_correlation_path(path: str) -> None:
    """'tensor' (default) or 'plain' for this thread's finds."""
    lib = load()
    lib.mvg_set_correlation_path.argtypes = [C.c_int32]
    lib.mvg_set_correlation_path.restype = C.c_int32
    _check(lib.mvg_set_correlation_path(0 if path == "tensor" else 1), "set_correlation_path")


def set_tc_weight_lookahead(rows: int) -> None:
    """Grid rows of tensor-core weights this thread's finds keep in flight
    ahead of the MMAs (1..64); a launch-shape setting, results do not change."""
    lib = load()
    lib.mvg_set_tc_weight_lookahead.argtypes = [C.c_int32]
    lib.mvg_set_tc_weight_lookahead.restype = C.c_int32
    _check(lib.mvg_set_tc_weight_lookahead(int(rows)), "set_tc_weight_lookahead")


def set_budgets(samples: int = 0, pixels: int = 0, candidates: int = 0) -> None:
    """Extended mode: this thread's model-raster sample, search-image pixel and
    coarse-candidate budgets (0 = the reference's 16 000 000, 32 000 000 and
    10 000)."""
    lib = load()
    lib.mvg_set_budgets.argtypes = [C.c_int64, C.c_int64, C.c_int32]
    lib.mvg_set_budgets.restype = C.c_int32
    _check(lib.mvg_set_budgets(int(samples), int(pixels), int(candidates)), "set_budgets")


def get_budgets() -> dict:
    lib = load()
    a, b, c = C.c_int64(), C.c_int64(), C.c_int32()
    lib.mvg_get_budgets.argtypes = [_i64p, _i64p, _i32p]
    _check(lib.mvg_get_budgets(C.byref(a), C.byref(b), C.byref(c)), "get_budgets")
    return {"samples": a.value, "pixels": b.value, "candidates": c.value}


class extended_budgets:
    """Context manager: the budgets raised inside, restored on exit."""

    def __init__(self, samples: int = 0, pixels: int = 0, candidates: int = 0):
        self.want = (samples, pixels, candidates)

    def __enter__(self):
        self.old = get_budgets()
        set_budgets(*self.want)
        return self

    def __exit__(self, *exc):
        set_budgets(self.old["samples"], self.old["pixels"], self.old["candidates"])


def set_batch_merge(cohorts: int = 0) -> None:
    """Batched calls from this thread merge their finds' tensor-core launches
    within `cohorts` groups of workers; 0 (the library's default) launches
    them per find."""
    lib = load()
    lib.mvg_set_batch_merge.argtypes = [C.c_int32]
    lib.mvg_set_batch_merge.restype = C.c_int32
    _check(lib.mvg_set_batch_merge(int(cohorts)), "set_batch_merge")


def batch_profile_reset() -> None:
    _check(load().mvg_batch_profile_reset(), "batch_profile")


def batch_profile_read() -> dict:
    """Merged tensor-core launches of batched calls since the last reset:
    {ms, launches, jobs, macs, issued} (event time on the batcher's stream)."""
    lib = load()
    ms, macs, issued = C.c_double(), C.c_double(), C.c_double()
    launches, jobs = C.c_int64(), C.c_int64()
    lib.mvg_batch_profile_read.argtypes = [_dp, _i64p, _i64p, _dp, _dp]
    _check(lib.mvg_batch_profile_read(C.byref(ms), C.byref(launches), C.byref(jobs), C.byref(macs),
                                      C.byref(issued)), "batch_profile")
    return {"ms": ms.value, "launches": launches.value, "jobs": jobs.value, "macs": macs.value,
            "issued": issued.value}


def profile_enable(on: bool = True) -> None:
    """Per-thread stage timing of finds (CUDA events on the find's stream)."""
    _check(load().mvg_profile_enable(1 if on else 0), "profile")


def profile_reset() -> None:
    _check(load().mvg_profile_reset(), "profile")


def profile_read() -> dict:
    """{stage: {ms, launches, work}} plus 'finds' for this thread's finds since the last reset."""
    out = {}
    finds = 0
    for i in range(PROFILE_STAGES):
        name = C.c_char_p()
        ms, work = C.c_double(), C.c_double()
        launches, nf = C.c_int64(), C.c_int64()
        _check(load().mvg_profile_read(i, C.byref(name), C.byref(ms), C.byref(launches), C.byref(work), C.byref(nf)),
               "profile")
        out[name.value.decode()] = dict(ms=ms.value, launches=launches.value, work=work.value)
        finds = nf.value
    out["finds"] = finds
    issued = C.c_double()
    lib = load()
    lib.mvg_profile_tensor_issued.argtypes = [C.POINTER(C.c_double)]
    lib.mvg_profile_tensor_issued.restype = C.c_int32
    _check(lib.mvg_profile_tensor_issued(C.byref(issued)), "profile")
    out["tensor_issued_macs"] = issued.value
    return out
