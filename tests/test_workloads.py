"""Host logic of the synthetic configuration workloads and of the quadratic
peak fit (no device): similarity scenes place their template squares apart
and reproducibly, a similarity paste at unit scale and zero angle copies the
template, and the parabola vertex of the quadratic fit."""
from __future__ import annotations

import hashlib
import math

import numpy as np
import pytest

from mvkit_gb300 import ncc
from mvkit_gb300 import workloads as W


def _seg_dist(p, a, b):
    (py, px), (ay, ax), (by, bx) = p, a, b
    dy, dx = by - ay, bx - ax
    t = max(0.0, min(1.0, ((py - ay) * dy + (px - ax) * dx) / (dy * dy + dx * dx)))
    return math.hypot(py - (ay + t * dy), px - (ax + t * dx))


def _poly_dist(a, b):
    """Euclidean distance of two disjoint convex quadrilaterals (corner to
    edge, both ways)."""
    return min(min(_seg_dist(p, q[i], q[(i + 1) % 4]) for p in pp for i in range(4)) for pp, q in ((a, b), (b, a)))


def test_squares_apart_separating_axis():
    a = W._square(0.0, 0.0, 0.0, 10.0)
    assert W._squares_apart(a, W._square(0.0, 25.0, 0.0, 10.0), 2.0)        # 5 px apart
    assert not W._squares_apart(a, W._square(0.0, 21.0, 0.0, 10.0), 2.0)    # 1 px apart
    assert not W._squares_apart(a, W._square(3.0, 3.0, 0.5, 10.0), 0.0)     # overlapping
    d = W._square(0.0, 10 + 10 * math.sqrt(2) + 3, math.pi / 4, 10.0)        # corner 3 px from an edge
    assert W._squares_apart(a, d, 2.0) and not W._squares_apart(a, d, 4.0)


def test_similarity_scene_places_squares_apart_and_reproducibly():
    wl = W.make_similarity_workload(5, 640, 640, (32, 48), 12)
    assert len(wl.poses) == 12 and [t.shape[0] for t in wl.templates] == [32, 48]
    sq = []
    for p in wl.poses:
        half = p.scale * wl.templates[p.model].shape[0] / 2
        assert 0.95 <= p.scale <= 1.05 and -math.pi <= p.angle < math.pi
        assert half < p.row < 639 - half and half < p.column < 639 - half
        sq.append(W._square(p.row, p.column, p.angle, half))
    for i in range(len(sq)):
        for j in range(i):
            assert _poly_dist(sq[i], sq[j]) >= 2.0 - 1e-9, (i, j)
    again = W.make_similarity_workload(5, 640, 640, (32, 48), 12)
    assert hashlib.sha256(wl.image.tobytes()).digest() == hashlib.sha256(again.image.tobytes()).digest()


def test_similarity_paste_copies_template_at_unit_scale():
    rng = np.random.default_rng(3)
    t = rng.integers(0, 256, size=(17, 17)).astype(np.uint8)
    img = np.zeros((64, 64))
    W.paste_similarity(img, t, 30.0, 20.0, 0.0, 1.0)   # centre (8, 8) of the patch at (30, 20)
    assert np.array_equal(img[22:39, 12:29], t.astype(np.float64))
    assert img[:22].sum() == 0 and img[39:].sum() == 0


@pytest.mark.parametrize("x0", [-0.7, -0.3, 0.0, 0.3, 0.9])
def test_parabola_vertex(x0):
    f = lambda x: 1.0 - 2.0 * (x - x0) ** 2
    off = ncc.parabola_vertex_offsets(f(-1.0), f(0.0), f(1.0))
    assert abs(float(off) - x0) < 1e-12


def test_parabola_vertex_edge_cases():
    off = ncc.parabola_vertex_offsets([0.0, 1.0, np.nan, 0.8], [1.0, 0.5, 1.0, 0.9], [0.9, 0.0, 0.5, 0.2])
    assert off[1] == 0.0                       # opens upwards: no move
    assert off[2] == 0.0                       # a score missing: no move
    assert 0.0 < off[0] <= 1.0 and -1.0 <= off[3] < 0.0
    far = ncc.parabola_vertex_offsets(0.0, 0.5, 0.9)   # vertex 4.5 steps out: clipped to one
    assert float(far) == 1.0
