"""ctypes access to the checkers: the FP64 oracle restatement (oracle/_ref/liboracle.so)
and, where it was built in this container, the reference compiled from its own
sources (oracle/_ref/libref_{scalar,avx2}.so).  Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
REF_DIR = ORACLE_DIR / "_ref"

_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)


def build_oracle() -> Path:
    lib = REF_DIR / "liboracle.so"
    src = ORACLE_DIR / "ncc_oracle.cpp"
    if not lib.exists() or lib.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return lib


class Checker:
    """One of the CPU implementations of find (prefix 'orc' or 'ref')."""

    def __init__(self, path: Path, prefix: str):
        self.path = path
        self.prefix = prefix
        lib = C.CDLL(str(path))
        self.lib = lib
        g = lambda n: getattr(lib, f"{prefix}_{n}")
        self._create = g("ncc_create" if prefix == "ref" else "create")
        self._create.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64, _u8p, C.c_int,
                                 C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_void_p),
                                 C.c_char_p, C.c_int]
        self._create.restype = C.c_int
        self._free = g("ncc_free" if prefix == "ref" else "free")
        self._free.argtypes = [C.c_void_p]
        self._info = g("ncc_model_info" if prefix == "ref" else "model_info")
        self._info.argtypes = [C.c_void_p, _dp]
        self._level = g("ncc_level" if prefix == "ref" else "level")
        self._level.argtypes = [C.c_void_p, C.c_int, _i64p, _dp]
        self._patch = g("ncc_patch" if prefix == "ref" else "patch")
        self._patch.argtypes = [C.c_void_p, C.c_int, C.c_int, _i32p, _i32p, _dp, C.c_int64, _dp]
        self._patch.restype = C.c_int64
        self._find = g("ncc_find" if prefix == "ref" else "find")
        if prefix == "ref":
            self._find.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64, _u8p,
                                   C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double, C.c_int,
                                   C.c_int, C.c_int, _dp, C.c_int64, _i64p, C.c_char_p, C.c_int]
        else:
            self._find.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64, _u8p,
                                   C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double, C.c_int,
                                   C.c_int, C.c_int, C.c_int, _dp, C.c_int64, _i64p, C.c_char_p, C.c_int]
            self._pyr = lib.orc_pyramid
            self._pyr.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_int,
                                  C.c_int, _dp, C.c_int64, _dp, C.c_char_p, C.c_int]
            self._many = lib.orc_find_many
            self._many.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_int, C.c_int64, C.c_int64, C.c_int64,
                                   C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int64,
                                   C.c_double, C.c_int, C.c_int, C.c_int]
            self._many.restype = C.c_int64
        self._find.restype = C.c_int
        if prefix == "ref":
            self._ser = lib.ref_ncc_serialize
            self._ser.argtypes = [C.c_void_p, C.c_char_p, C.c_int64, C.c_char_p, C.c_int]
            self._ser.restype = C.c_int64
            self._deser = lib.ref_ncc_deserialize
            self._deser.argtypes = [C.c_char_p, C.c_int64, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
            self._deser.restype = C.c_int

    # -- multi-model find (reference only: mv::ncc_matching::find_models)
    def find_models(self, models, image, opts, sel_num_matches, sel_max_overlap, capacity=4096):
        img = np.ascontiguousarray(image)
        typ = 1 if img.dtype == np.uint16 else 0
        n = len(models)
        f = self.lib.ref_ncc_find_models
        f.argtypes = [C.POINTER(C.c_void_p), C.c_int64, C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64,
                      _dp, _dp, _dp, _i64p, _dp, _i32p, _i32p, _i32p, C.c_int64, C.c_double, _dp, C.c_int64,
                      _i64p, C.c_char_p, C.c_int]
        f.restype = C.c_int
        hs = (C.c_void_p * n)(*[m.handle for m in models])
        col = lambda k, dt: np.ascontiguousarray([o[k] for o in opts], dtype=dt)
        a0, ae, ms, mo = col("angle_start", np.float64), col("angle_extent", np.float64), \
            col("min_score", np.float64), col("max_overlap", np.float64)
        nm = col("num_matches", np.int64)
        sp, hi, lo = col("subpixel", np.int32), col("highest", np.int32), col("lowest", np.int32)
        out = np.zeros((capacity, 5))
        cnt = C.c_int64()
        err = C.create_string_buffer(256)
        st = f(hs, n, img.ctypes.data, typ, img.shape[1], img.shape[0], img.strides[0],
               a0.ctypes.data_as(_dp), ae.ctypes.data_as(_dp), ms.ctypes.data_as(_dp), nm.ctypes.data_as(_i64p),
               mo.ctypes.data_as(_dp), sp.ctypes.data_as(_i32p), hi.ctypes.data_as(_i32p), lo.ctypes.data_as(_i32p),
               int(sel_num_matches), float(sel_max_overlap), out.ctypes.data_as(_dp), capacity, C.byref(cnt), err, 256)
        if st != 0:
            raise CheckerError(st, err.value.decode())
        return out[: min(cnt.value, capacity)].copy()

    # -- model files (reference only: mv::ncc_matching::serialize/deserialize)
    def serialize(self, model) -> bytes:
        err = C.create_string_buffer(256)
        n = self._ser(model.handle, None, 0, err, 256)
        if n < 0:
            raise CheckerError(-1000, err.value.decode())
        buf = C.create_string_buffer(max(1, n))
        self._ser(model.handle, buf, n, err, 256)
        return buf.raw[:n]

    def deserialize(self, data: bytes):
        h = C.c_void_p()
        err = C.create_string_buffer(256)
        st = self._deser(bytes(data), len(data), C.byref(h), err, 256)
        if st != 0:
            raise CheckerError(st, err.value.decode())
        return Model(self, h)

    # -- model
    def create(self, tmpl: np.ndarray, levels=0, angle_start=0.0, angle_extent=0.0, angle_step=0.0,
               ignore_polarity=False, mask: np.ndarray | None = None):
        t = np.ascontiguousarray(tmpl)
        typ = 1 if t.dtype == np.uint16 else 0
        m = None
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
        h = C.c_void_p()
        err = C.create_string_buffer(256)
        st = self._create(t.ctypes.data, typ, t.shape[1], t.shape[0], t.strides[0],
                          m.ctypes.data_as(_u8p) if m is not None else None, int(levels), angle_start,
                          angle_extent, angle_step, int(bool(ignore_polarity)), C.byref(h), err, 256)
        if st != 0:
            raise CheckerError(st, err.value.decode())
        return Model(self, h)

    def find(self, model, image: np.ndarray, angle_start, angle_extent, min_score, num_matches,
             max_overlap, subpixel=True, highest=0, lowest=1, stage=-1, domain=None, capacity=20000):
        img = np.ascontiguousarray(image)
        typ = 1 if img.dtype == np.uint16 else 0
        out = np.zeros((capacity, 4), dtype=np.float64)
        cnt = C.c_int64()
        err = C.create_string_buffer(256)
        d = None if domain is None else np.ascontiguousarray(domain, dtype=np.uint8)
        args = [model.handle, img.ctypes.data, typ, img.shape[1], img.shape[0], img.strides[0],
                d.ctypes.data_as(_u8p) if d is not None else None, angle_start, angle_extent, min_score,
                int(num_matches), max_overlap, int(bool(subpixel)), int(highest), int(lowest)]
        if self.prefix == "orc":
            args.append(int(stage))
        args += [out.ctypes.data_as(_dp), capacity, C.byref(cnt), err, 256]
        st = self._find(*args)
        if st != 0:
            raise CheckerError(st, err.value.decode())
        return out[: min(cnt.value, capacity)].copy()

    def pyramid(self, model, image: np.ndarray, highest: int, level: int):
        img = np.ascontiguousarray(image)
        typ = 1 if img.dtype == np.uint16 else 0
        out = np.zeros(img.size + 16, dtype=np.float64)
        geom = np.zeros(6)
        err = C.create_string_buffer(256)
        st = self._pyr(model.handle, img.ctypes.data, typ, img.shape[1], img.shape[0], img.strides[0],
                       int(highest), int(level), out.ctypes.data_as(_dp), out.size, geom.ctypes.data_as(_dp),
                       err, 256)
        if st != 0:
            raise CheckerError(st, err.value.decode())
        w, h = int(geom[0]), int(geom[1])
        return out[: w * h].reshape(h, w).copy(), geom

    def find_many(self, model, images, threads, angle_start, angle_extent, min_score, num_matches,
                  max_overlap, subpixel=True, highest=0, lowest=1) -> int:
        arr = (C.c_void_p * len(images))(*[im.ctypes.data for im in images])
        im0 = images[0]
        typ = 1 if im0.dtype == np.uint16 else 0
        return self._many(model.handle, arr, typ, im0.shape[1], im0.shape[0], im0.strides[0], len(images),
                          int(threads), angle_start, angle_extent, min_score, int(num_matches), max_overlap,
                          int(bool(subpixel)), int(highest), int(lowest))


class CheckerError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status
        self.message = message


class Model:
    def __init__(self, checker: Checker, handle):
        self.checker = checker
        self.handle = handle

    def __del__(self):
        try:
            if self.handle:
                self.checker._free(self.handle)
                self.handle = None
        except Exception:
            pass

    def info(self):
        a = np.zeros(6)
        self.checker._info(self.handle, a.ctypes.data_as(_dp))
        return dict(levels=int(a[0]), angle_step=a[1], origin_row=a[2], origin_column=a[3],
                    patches=int(a[4]), original_samples=int(a[5]))

    def level(self, level: int):
        dims = np.zeros(2, dtype=np.int64)
        org = np.zeros(2)
        self.checker._level(self.handle, level, dims.ctypes.data_as(_i64p), org.ctypes.data_as(_dp))
        return int(dims[0]), int(dims[1]), float(org[0]), float(org[1])

    def patch(self, level: int, index: int):
        meta = np.zeros(4)
        n = self.checker._patch(self.handle, level, index, None, None, None, 0, meta.ctypes.data_as(_dp))
        rows = np.zeros(n, dtype=np.int32)
        cols = np.zeros(n, dtype=np.int32)
        w = np.zeros(n)
        self.checker._patch(self.handle, level, index, rows.ctypes.data_as(_i32p), cols.ctypes.data_as(_i32p),
                            w.ctypes.data_as(_dp), n, meta.ctypes.data_as(_dp))
        return dict(angle=meta[0], origin_row=meta[1], origin_column=meta[2], weight_sum=meta[3],
                    rows=rows, cols=cols, weights=w)


def oracle() -> Checker:
    return Checker(build_oracle(), "orc")


def set_oracle_budgets(samples: int = 0, pixels: int = 0, candidates: int = 0) -> None:
    """The oracle's raster-sample, image-pixel and candidate budgets for the
    following calls (process-wide; 0 = the reference's)."""
    lib = oracle().lib
    lib.orc_set_budgets.argtypes = [C.c_int64, C.c_int64, C.c_int64]
    lib.orc_set_budgets.restype = None
    lib.orc_set_budgets(int(samples), int(pixels), int(candidates))


def reference(kind: str = "scalar") -> Checker | None:
    p = REF_DIR / f"libref_{kind}.so"
    if not p.exists():
        return None
    return Checker(p, "ref")


def to_halcon(rows_cols_angles_scores: np.ndarray) -> np.ndarray:
    """Pose convention of the C API: src/c_api/ncc_matching_api.cpp:171-176."""
    m = np.asarray(rows_cols_angles_scores, dtype=np.float64).reshape(-1, 4)
    c, s = np.cos(m[:, 2]), np.sin(m[:, 2])
    out = m.copy()
    out[:, 0] = m[:, 0] + 0.5 * (1 - c + s)
    out[:, 1] = m[:, 1] + 0.5 * (1 - c - s)
    return out
