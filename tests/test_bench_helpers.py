"""The bench's pose checks on the host (no device): the operator's and the
matcher's pose conventions invert each other, the nearest-pose error counts
and bounds, the bit-identity of two passes and the similarity pose errors."""
from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np

import bench
from mvkit_gb300 import workloads as W


def test_pose_conventions_invert():
    for r, c, a in ((10.0, 20.0, 0.0), (5.5, 7.25, 0.4), (100.0, 3.0, -2.9)):
        hr, hc = bench.halcon(r, c, a)
        mr, mc = bench.matcher_pose(hr, hc, a)
        assert abs(mr - r) < 1e-12 and abs(mc - c) < 1e-12
    assert bench.halcon(3.0, 4.0, 0.0) == (3.0, 4.0)


def _found(poses, drow=0.0, dcol=0.0, dang=0.0):
    hr = [bench.halcon(p.row, p.column, p.angle) for p in poses]
    return (np.array([h[0] + drow for h in hr]), np.array([h[1] + dcol for h in hr]),
            np.array([p.angle + dang for p in poses]), np.full(len(poses), 0.9))


def test_pose_error_nearest_match_and_unmatched():
    poses = [W.Pose(100.0, 200.0, 0.1), W.Pose(300.0, 50.0, -0.2)]
    wl = SimpleNamespace(poses=poses)
    out = bench.pose_error([_found(poses, 0.03, -0.02, math.radians(0.01))], [wl])["vs_truth"]
    assert out["unmatched"] == 0 and out["poses"] == 2
    assert abs(out["max_drow"] - 0.03) < 1e-9 and abs(out["max_dcol"] - 0.02) < 1e-9
    assert abs(out["max_dangle_deg"] - 0.01) < 1e-9
    far = bench.pose_error([_found(poses, 2.5)], [wl])["vs_truth"]      # beyond 2 px: not a match
    assert far["unmatched"] == 2
    none = bench.pose_error([(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))], [wl])["vs_truth"]
    assert none["unmatched"] == 2


def test_same_results_is_bit_identity():
    a = [(np.array([1.0, 2.0]), np.array([3.0, 4.0]), np.array([0.1, 0.2]), np.array([0.9, 0.8]))]
    b = [tuple(x.copy() for x in a[0])]
    assert bench.same_results(a, b)
    b[0][3][1] = np.nextafter(0.8, 1.0)
    assert not bench.same_results(a, b)
    assert not bench.same_results(a, a + a)


def test_similarity_errors():
    truth = [W.SimilarityPose(50.0, 60.0, 0.5, 1.02, 0), W.SimilarityPose(150.0, 160.0, -1.0, 0.97, 1),
             W.SimilarityPose(250.0, 260.0, 3.1, 1.0, 1)]
    poses = np.array([[50.01, 60.02, 0.5 + math.radians(0.01), 1.021],
                      [150.2, 160.0, -1.0, 0.97],
                      [250.0, 260.0, 3.1 - 2 * math.pi, 1.0]])
    model_of = np.array([0, 1, 0])          # the third pose was found with the wrong model
    out = bench.similarity_errors(poses, model_of, truth)
    assert out["found"] == 2 and out["missing"] == 1
    assert abs(out["max"]["row_px"] - 0.2) < 1e-9
    assert abs(out["within_0.05px_0.05deg"] - 0.5) < 1e-12
    wrapped = bench.similarity_errors(poses, np.array([0, 1, 1]), truth)
    # angles compared modulo 2 pi: the third pose adds no angle error
    assert wrapped["found"] == 3 and abs(wrapped["max"]["angle_deg"] - 0.01) < 1e-9
