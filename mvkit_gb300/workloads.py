"""Seeded synthetic search scenes for the NCC matching path.

The scenes follow the workload descriptions the matcher is benchmarked on:
a smoothed-noise background (std 20 around mid-grey), filled rectangles and
ellipses with intensities U[30, 220], a template cropped from a second scene
of the same kind and pasted at known sub-pixel poses by bilinear warping, then
additive Gaussian noise and clipping.

Every step is integer arithmetic or IEEE +,-,*,floor on float64 (the pose
rotation uses ``math.cos``/``math.sin`` once per pose), so the same seed gives
the same bytes on x86-64 and aarch64.  Gaussian noise is Irwin-Hall (sum of 12
uniform integers); smoothing is three passes of an integer box filter
(radius 3, equivalent Gaussian sigma ~3.5 px).

Poses use the matcher's internal convention: (row, column) is the template
origin (the centroid of its domain) in pixel-centre coordinates, a template
offset (dr, dc) from the origin lands at
``row + cos(a)*dr - sin(a)*dc, column + sin(a)*dr + cos(a)*dc``
(src/ncc_matching/matcher.cpp:144-148 in the reference).
"""
from __future__ import annotations

import hashlib
import math
from dataclasses import dataclass, field

import numpy as np

BOX_RADIUS = 3


def _box(a: np.ndarray, r: int, axis: int) -> np.ndarray:
    """Integer box sum of width 2r+1 along `axis` with edge replication."""
    pad = [(0, 0), (0, 0)]
    pad[axis] = (r + 1, r)
    p = np.pad(a, pad, mode="edge")
    c = np.cumsum(p, axis=axis, dtype=np.int64)
    n = a.shape[axis]
    hi = np.take(c, np.arange(2 * r + 1, 2 * r + 1 + n), axis=axis)
    lo = np.take(c, np.arange(0, n), axis=axis)
    return hi - lo


def _gauss_int(rng: np.random.Generator, shape, sigma_num: int, sigma_den: int = 1) -> np.ndarray:
    """Integer approximately-normal noise with std sigma_num/sigma_den (Irwin-Hall, 12 terms)."""
    s = np.zeros(shape, dtype=np.int64)
    for _ in range(12):
        s += rng.integers(0, 4096, size=shape, dtype=np.int64)
    s -= 12 * 4095 // 2  # centre (24570)
    # std of s is ~4096; scale with rounding toward -inf on a biased value
    num = s * sigma_num * 2 + 4096 * sigma_den
    return np.floor_divide(num, 2 * 4096 * sigma_den)


def scene(seed: int, height: int, width: int, shapes: int = 40, bg_std: int = 20,
          maxval: int = 255) -> np.ndarray:
    """Background + shapes (no additive noise) as int64, range [0, maxval] before noise."""
    rng = np.random.default_rng(seed)
    scale = (maxval + 1) // 256  # 1 for 8-bit scenes, 16 for 12-bit scenes
    n = rng.integers(-1024, 1024, size=(height, width), dtype=np.int64)
    for _ in range(3):
        n = _box(n, BOX_RADIUS, 0)
        n = _box(n, BOX_RADIUS, 1)
    n = np.floor_divide(n, 4096)  # keep squares well inside int64 for 8192^2 scenes
    n -= int(n.sum()) // n.size
    var = int((n * n).sum()) // n.size
    sd = max(1, math.isqrt(var))
    img = (128 * scale) + (n * (bg_std * scale)) // sd
    for _ in range(shapes):
        kind = int(rng.integers(0, 2))
        cy = int(rng.integers(0, height))
        cx = int(rng.integers(0, width))
        hy = int(rng.integers(max(2, height // 64), max(3, height // 8)))
        hx = int(rng.integers(max(2, width // 64), max(3, width // 8)))
        val = int(rng.integers(30, 221)) * scale
        r0, r1 = max(0, cy - hy), min(height, cy + hy + 1)
        c0, c1 = max(0, cx - hx), min(width, cx + hx + 1)
        if r0 >= r1 or c0 >= c1:
            continue
        if kind == 0:
            img[r0:r1, c0:c1] = val
        else:
            yy = (np.arange(r0, r1, dtype=np.int64) - cy)[:, None]
            xx = (np.arange(c0, c1, dtype=np.int64) - cx)[None, :]
            inside = yy * yy * hx * hx + xx * xx * hy * hy <= hy * hy * hx * hx
            sub = img[r0:r1, c0:c1]
            sub[inside] = val
    return img


@dataclass
class Pose:
    row: float
    column: float
    angle: float
    contrast: float = 1.0


def paste(img: np.ndarray, tmpl: np.ndarray, pose: Pose) -> None:
    """Bilinear-warp `tmpl` (float64 values) into `img` (int64) at `pose`, in place."""
    th, tw = tmpl.shape
    cy, cx = (th - 1) / 2.0, (tw - 1) / 2.0
    ca, sa = math.cos(pose.angle), math.sin(pose.angle)
    rad = math.hypot(th, tw) / 2.0 + 2
    r0 = max(0, int(math.floor(pose.row - rad)))
    r1 = min(img.shape[0], int(math.ceil(pose.row + rad)) + 1)
    c0 = max(0, int(math.floor(pose.column - rad)))
    c1 = min(img.shape[1], int(math.ceil(pose.column + rad)) + 1)
    if r0 >= r1 or c0 >= c1:
        return
    y = np.arange(r0, r1, dtype=np.float64)[:, None] - pose.row
    x = np.arange(c0, c1, dtype=np.float64)[None, :] - pose.column
    # inverse of y = ca*dr - sa*dc, x = sa*dr + ca*dc
    tr = (ca * y + sa * x) + cy
    tc = (ca * x - sa * y) + cx
    ok = (tr >= 0) & (tc >= 0) & (tr <= th - 1) & (tc <= tw - 1)
    rr = np.floor(np.where(ok, tr, 0.0))
    cc = np.floor(np.where(ok, tc, 0.0))
    fr = np.where(ok, tr, 0.0) - rr
    fc = np.where(ok, tc, 0.0) - cc
    ri = rr.astype(np.int64)
    ci = cc.astype(np.int64)
    ri1 = np.minimum(ri + 1, th - 1)
    ci1 = np.minimum(ci + 1, tw - 1)
    a = tmpl[ri, ci]
    b = tmpl[ri, ci1]
    d = tmpl[ri1, ci]
    e = tmpl[ri1, ci1]
    v = (1 - fr) * ((1 - fc) * a + fc * b) + fr * ((1 - fc) * d + fc * e)
    if pose.contrast != 1.0:
        mid = float(tmpl.mean())
        v = (v - mid) * pose.contrast + mid
    sub = img[r0:r1, c0:c1]
    sub[ok] = np.floor(v[ok] + 0.5).astype(np.int64)


@dataclass
class Workload:
    image: np.ndarray            # uint8 or uint16, (H, W)
    template: np.ndarray         # same dtype, (th, tw)
    poses: list = field(default_factory=list)   # ground-truth Pose list (internal convention)
    maxval: int = 255

    def digest(self) -> str:
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.image).tobytes())
        h.update(np.ascontiguousarray(self.template).tobytes())
        return h.hexdigest()[:16]


def _finish(img: np.ndarray, rng: np.random.Generator, noise_sigma: int, maxval: int, dtype) -> np.ndarray:
    img = img + _gauss_int(rng, img.shape, noise_sigma)
    return np.clip(img, 0, maxval).astype(dtype)


def make_workload(seed: int, height: int, width: int, tsize: int, n_poses: int,
                  angle_range: tuple = (0.0, 0.0), noise_sigma: int = 3, shapes: int = 40,
                  maxval: int = 255, contrast: float = 0.0, subpixel: bool = True,
                  invert_odd: bool = False, border: float | None = None,
                  template_seed: int | None = None) -> Workload:
    """One search scene with `n_poses` pastes of one square template of side `tsize`.

    angle_range is in radians; contrast > 0 scales each paste by U[1-c, 1+c];
    invert_odd pastes every second pose with inverted contrast.  Pastes are
    kept apart by at least the template diagonal, and `border` pixels (default
    half the diagonal + 8) away from the image edge.
    """
    dtype = np.uint8 if maxval <= 255 else np.uint16
    tseed = seed if template_seed is None else template_seed
    rng = np.random.default_rng([tseed, 1])
    src = scene(tseed * 7919 + 17, max(2 * tsize, 64), max(2 * tsize, 64), shapes=max(8, shapes // 4),
                maxval=maxval)
    ty = int(rng.integers(0, src.shape[0] - tsize + 1))
    tx = int(rng.integers(0, src.shape[1] - tsize + 1))
    tmpl_i = src[ty:ty + tsize, tx:tx + tsize]
    tmpl_i = np.clip(tmpl_i + _gauss_int(rng, tmpl_i.shape, noise_sigma), 0, maxval)
    if template_seed is not None:
        rng = np.random.default_rng([seed, 2])  # scene poses and noise of this scene
    img = scene(seed, height, width, shapes=shapes, maxval=maxval)
    diag = math.hypot(tsize, tsize)
    margin = diag / 2.0 + 8 if border is None else float(border)
    poses: list[Pose] = []
    tries = 0
    while len(poses) < n_poses:
        tries += 1
        if tries > 10000:
            raise ValueError("cannot place the requested poses without overlap")
        row = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (height - 1 - 2 * margin)
        col = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (width - 1 - 2 * margin)
        if not subpixel:
            row, col = float(round(row)), float(round(col))
        lo, hi = angle_range
        ang = lo + float(rng.integers(0, 1 << 20)) / (1 << 20) * (hi - lo)
        c = 1.0
        if contrast > 0:
            c = 1.0 - contrast + 2 * contrast * float(rng.integers(0, 1 << 20)) / (1 << 20)
        if invert_odd and len(poses) % 2 == 1:
            c = -c
        if all(math.hypot(row - p.row, col - p.column) > diag + 4 for p in poses):
            poses.append(Pose(row, col, ang, c))
    t_f = tmpl_i.astype(np.float64)
    for p in poses:
        paste(img, t_f, p)
    image = _finish(img, rng, noise_sigma, maxval, dtype)
    return Workload(image=image, template=tmpl_i.astype(dtype), poses=poses, maxval=maxval)


@dataclass
class MultiWorkload:
    image: np.ndarray
    templates: list              # one square template per model
    poses: list                  # per template, its ground-truth Pose list
    maxval: int = 255

    def digest(self) -> str:
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.image).tobytes())
        for t in self.templates:
            h.update(np.ascontiguousarray(t).tobytes())
        return h.hexdigest()[:16]


def make_multi_workload(seed: int, height: int, width: int, tsizes: tuple, n_poses: tuple,
                        angle_range: tuple = (0.0, 0.0), noise_sigma: int = 3, shapes: int = 40,
                        maxval: int = 255, contrast: float = 0.0,
                        template_seed: int | None = None, fit: bool = False) -> MultiWorkload:
    """One scene holding several different templates (FindNccModels): template
    k (side tsizes[k], cropped from its own source scene) is pasted n_poses[k]
    times; no two pastes overlap.  contrast > 0 scales each paste by
    U[1-c, 1+c]; template_seed (default: seed) makes the templates, so scenes
    of one batch can share them.  fit: a template gets fewer pastes (at least
    none) when no free place is found in 10000 tries, instead of an error."""
    dtype = np.uint8 if maxval <= 255 else np.uint16
    tseed = seed if template_seed is None else template_seed
    templates = []
    for k, ts in enumerate(tsizes):
        rng_t = np.random.default_rng([tseed, 100 + k])
        src = scene(tseed * 7919 + 31 * k + 5, max(2 * ts, 64), max(2 * ts, 64), shapes=max(8, shapes // 4),
                    maxval=maxval)
        ty = int(rng_t.integers(0, src.shape[0] - ts + 1))
        tx = int(rng_t.integers(0, src.shape[1] - ts + 1))
        t = src[ty:ty + ts, tx:tx + ts]
        templates.append(np.clip(t + _gauss_int(rng_t, t.shape, noise_sigma), 0, maxval))
    rng = np.random.default_rng([seed, 3])
    img = scene(seed, height, width, shapes=shapes, maxval=maxval)
    placed = []  # (row, col, diag)
    poses = [[] for _ in tsizes]
    for k, ts in enumerate(tsizes):
        diag = math.hypot(ts, ts)
        margin = diag / 2.0 + 8
        tries = 0
        while len(poses[k]) < n_poses[k]:
            tries += 1
            if tries > 10000:
                if fit:
                    break
                raise ValueError("cannot place the requested poses without overlap")
            row = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (height - 1 - 2 * margin)
            col = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (width - 1 - 2 * margin)
            lo, hi = angle_range
            ang = lo + float(rng.integers(0, 1 << 20)) / (1 << 20) * (hi - lo)
            if all(math.hypot(row - r, col - c) > (diag + d) / 2 + 4 for r, c, d in placed):
                gain = 1.0
                if contrast > 0:
                    gain = 1.0 - contrast + 2 * contrast * float(rng.integers(0, 1 << 20)) / (1 << 20)
                poses[k].append(Pose(row, col, ang, gain))
                placed.append((row, col, diag))
    for k, t in enumerate(templates):
        tf = t.astype(np.float64)
        for p in poses[k]:
            paste(img, tf, p)
    image = _finish(img, rng, noise_sigma, maxval, dtype)
    return MultiWorkload(image=image, templates=[t.astype(dtype) for t in templates], poses=poses, maxval=maxval)


@dataclass
class SimilarityPose:
    row: float
    column: float
    angle: float
    scale: float
    model: int


@dataclass
class SimilarityWorkload:
    image: np.ndarray
    templates: list              # square uint8 templates, one per model
    poses: list                  # SimilarityPose (template centre, angle, scale, template index)


def paste_similarity(img: np.ndarray, patch: np.ndarray, row: float, col: float, angle: float, scale: float) -> None:
    """Bilinear FP64 paste of a square patch at a similarity pose, in place:
    the patch offset (dr, dc) from its centre lands at row + s (cos dr -
    sin dc), col + s (sin dr + cos dc) (the matcher's pose convention with a
    scale factor)."""
    t = patch.shape[0]
    o = (t - 1) / 2.0
    ca, sa = math.cos(angle), math.sin(angle)
    reach = int(math.ceil(scale * t * 0.75)) + 2
    r0, c0 = max(0, int(row) - reach), max(0, int(col) - reach)
    r1, c1 = min(img.shape[0], int(row) + reach + 1), min(img.shape[1], int(col) + reach + 1)
    if r0 >= r1 or c0 >= c1:
        return
    dy = np.arange(r0, r1, dtype=np.float64)[:, None] - row
    dx = np.arange(c0, c1, dtype=np.float64)[None, :] - col
    tr = (ca * dy + sa * dx) / scale + o
    tc = (-sa * dy + ca * dx) / scale + o
    inside = (tr >= 0) & (tc >= 0) & (tr <= t - 1) & (tc <= t - 1)
    ir = np.clip(np.floor(tr).astype(np.int64), 0, t - 1)
    ic = np.clip(np.floor(tc).astype(np.int64), 0, t - 1)
    ir1, ic1 = np.minimum(ir + 1, t - 1), np.minimum(ic + 1, t - 1)
    fr, fc = tr - np.floor(tr), tc - np.floor(tc)
    f = patch.astype(np.float64)
    v = (1 - fr) * ((1 - fc) * f[ir, ic] + fc * f[ir, ic1]) + fr * ((1 - fc) * f[ir1, ic] + fc * f[ir1, ic1])
    sub = img[r0:r1, c0:c1]
    sub[inside] = np.floor(v[inside] + 0.5)


def _square(row: float, col: float, angle: float, half: float):
    """Corners (row, col) of a square of half side `half` rotated by `angle`
    about (row, col), in the matcher's pose convention."""
    ca, sa = math.cos(angle), math.sin(angle)
    return [(row + ca * dr - sa * dc, col + sa * dr + ca * dc) for dr, dc in
            ((-half, -half), (-half, half), (half, half), (half, -half))]


def _squares_apart(a, b, gap: float) -> bool:
    """True when two convex quadrilaterals are at least `gap` apart along
    some edge normal (separating axis test)."""
    for poly in (a, b):
        for i in range(4):
            (y0, x0), (y1, x1) = poly[i], poly[(i + 1) % 4]
            ny, nx = x1 - x0, -(y1 - y0)
            norm = math.hypot(ny, nx)
            ny, nx = ny / norm, nx / norm
            pa = [ny * y + nx * x for y, x in a]
            pb = [ny * y + nx * x for y, x in b]
            if max(pa) + gap <= min(pb) or max(pb) + gap <= min(pa):
                return True
    return False


def make_similarity_workload(seed: int, height: int, width: int, tsizes: tuple, n_poses: int,
                             scale_range: tuple = (0.95, 1.05), noise_sigma: int = 3) -> SimilarityWorkload:
    """One uint8 scene holding `n_poses` pastes of the templates (template
    n mod len(tsizes) for paste n) at similarity poses: subpixel row and
    column, angle U[0, 2 pi), scale U[scale_range]; the rotated template
    squares do not overlap (2 px apart).  Each paste first lays the texture
    around its template (a patch 1.5 x the template, cropped from the same
    source scene around the same centre), as an object in a real scene has;
    then every template square is pasted over it, so no surround covers
    another paste's template."""
    rng = np.random.default_rng([seed, 11])
    templates, patches = [], []
    for k, ts in enumerate(tsizes):
        src = scene(seed * 7919 + 31 * k + 7, 2 * ts + 16, 2 * ts + 16, shapes=10)
        ps = ts + 2 * (ts // 4)
        y0 = (src.shape[0] - ps) // 2
        patch = src[y0:y0 + ps, y0:y0 + ps]
        m = ts // 4
        patches.append(patch)
        templates.append(np.clip(patch[m:m + ts, m:m + ts], 0, 255).astype(np.uint8))
    img = scene(seed, height, width).astype(np.float64)
    # larger templates are placed first (the packing is dense)
    order = sorted(range(n_poses), key=lambda n: -tsizes[n % len(tsizes)])
    placed = {}
    squares = []  # (row, col, reach, corners)
    for n in order:
        k = n % len(tsizes)
        tries = 0
        while True:
            tries += 1
            if tries > 100000:
                raise ValueError("cannot place the requested poses without overlap")
            s = scale_range[0] + float(rng.integers(0, 1 << 20)) / (1 << 20) * (scale_range[1] - scale_range[0])
            half = s * tsizes[k] / 2
            margin = half * 1.5 * math.sqrt(2) + 4
            row = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (height - 1 - 2 * margin)
            col = margin + float(rng.integers(0, 1 << 20)) / (1 << 20) * (width - 1 - 2 * margin)
            ang = float(rng.integers(0, 1 << 20)) / (1 << 20) * 2 * math.pi - math.pi
            sq = _square(row, col, ang, half)
            reach = half * math.sqrt(2)
            if all(math.hypot(row - r, col - c) > reach + q + 2 or _squares_apart(sq, corners, 2.0)
                   for r, c, q, corners in squares):
                squares.append((row, col, reach, sq))
                placed[n] = SimilarityPose(row, col, ang, s, k)
                break
    poses = [placed[n] for n in range(n_poses)]
    for p in poses:
        paste_similarity(img, patches[p.model], p.row, p.column, p.angle, p.scale)
    for p in poses:
        paste_similarity(img, templates[p.model], p.row, p.column, p.angle, p.scale)
    if noise_sigma:
        img = img + _gauss_int(rng, img.shape, noise_sigma)
    image = np.clip(img, 0, 255).astype(np.uint8)
    return SimilarityWorkload(image=image, templates=templates, poses=poses)


# Named workloads.  "find_640x480_t64" is the CPU-runnable case; "find_2048_t128_5x"
# is the single-GPU throughput case.
CONFIGS = {
    "find_640x480_t64": dict(
        gen=dict(height=480, width=640, tsize=64, n_poses=1, angle_range=(0.0, 0.0)),
        create=dict(num_levels=3, angle_start=0.0, angle_extent=0.0, angle_step="auto",
                    metric="use_polarity"),
        find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.8, num_matches=1,
                  max_overlap=0.5, subpixel=True, num_levels=3),
    ),
    "find_2048_t128_5x": dict(
        gen=dict(height=2048, width=2048, tsize=128, n_poses=5,
                 angle_range=(-math.radians(30), math.radians(30))),
        create=dict(num_levels=4, angle_start=-math.radians(30), angle_extent=math.radians(60),
                    angle_step="auto", metric="use_polarity"),
        find=dict(angle_start=-math.radians(30), angle_extent=math.radians(60), min_score=0.7,
                  num_matches=5, max_overlap=0.5, subpixel=True, num_levels=4),
    ),
}


def config_workload(name: str, seed: int) -> Workload:
    return make_workload(seed, **CONFIGS[name]["gen"])


def _multi_args(a):
    return make_multi_workload(*a[0], **a[1])


def make_batch_workloads(seed: int, n_images: int, sizes: tuple, tsizes: tuple, max_pastes: int,
                         angle_range: tuple = (-math.pi, math.pi), contrast: float = 0.1, noise_sigma: int = 5,
                         maxval: int = 255, processes: int = 1, fit: bool = False) -> list:
    """A batch of scenes of uneven size sharing one template set (one model
    per template searches every scene): scene i has a size drawn from
    `sizes` ((height, width) pairs) and each template pasted 1..max_pastes
    times, with contrast U[1-c, 1+c] and noise `noise_sigma`.  processes > 1
    generates the scenes in that many spawned processes (same scenes); fit:
    a scene too small for its pastes gets as many as fit (its poses list
    them)."""
    rng = np.random.default_rng([seed, 7])
    jobs = []
    for i in range(n_images):
        h, w = sizes[int(rng.integers(0, len(sizes)))]
        n = tuple(int(rng.integers(1, max_pastes + 1)) for _ in tsizes)
        jobs.append(((seed * 1000 + i + 1, h, w, tsizes, n, angle_range, noise_sigma),
                     dict(maxval=maxval, contrast=contrast, template_seed=seed, fit=fit)))
    if processes <= 1:
        return [_multi_args(j) for j in jobs]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    with ProcessPoolExecutor(processes, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_multi_args, jobs))
