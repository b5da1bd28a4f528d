"""Seeded parity cases shared by the golden-fixture generator and the tests.

Each case regenerates its image and template from mvkit_gb300.workloads
(platform-deterministic), builds a model and runs one find.  The fixture
file golden.json stores, per case, the input digest and the reference's
final matches (matcher-internal pixel-centre convention)."""
from __future__ import annotations

import math

from mvkit_gb300 import workloads as W

D = math.radians

# name: generator kwargs, create kwargs, find kwargs, optional template mask kind
CASES = {
    "cfg1_s1": dict(gen=dict(seed=1, height=480, width=640, tsize=64, n_poses=1),
                    create=dict(levels=3, angle_start=0.0, angle_extent=0.0),
                    find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.8, num_matches=1, max_overlap=0.5,
                              subpixel=True, highest=3, lowest=1)),
    "cfg1_s2": dict(gen=dict(seed=2, height=480, width=640, tsize=64, n_poses=1),
                    create=dict(levels=3, angle_start=0.0, angle_extent=0.0),
                    find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.8, num_matches=1, max_overlap=0.5,
                              subpixel=True, highest=3, lowest=1)),
    "cfg1_s3": dict(gen=dict(seed=3, height=480, width=640, tsize=64, n_poses=1),
                    create=dict(levels=3, angle_start=0.0, angle_extent=0.0),
                    find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.8, num_matches=1, max_overlap=0.5,
                              subpixel=True, highest=3, lowest=1)),
    "rot3_all": dict(gen=dict(seed=11, height=600, width=800, tsize=64, n_poses=3, angle_range=(-D(30), D(30))),
                     create=dict(levels=3, angle_start=-D(30), angle_extent=D(60)),
                     find=dict(angle_start=-D(30), angle_extent=D(60), min_score=0.7, num_matches=0,
                               max_overlap=0.5, subpixel=True, highest=3, lowest=1)),
    "rot_l4_2": dict(gen=dict(seed=12, height=768, width=1024, tsize=96, n_poses=2, angle_range=(-D(20), D(20))),
                     create=dict(levels=4, angle_start=-D(20), angle_extent=D(40)),
                     find=dict(angle_start=-D(20), angle_extent=D(40), min_score=0.7, num_matches=2,
                               max_overlap=0.5, subpixel=True, highest=4, lowest=1)),
    "u16_rot": dict(gen=dict(seed=13, height=480, width=640, tsize=64, n_poses=2, angle_range=(-D(20), D(20)),
                             maxval=4095, noise_sigma=20),
                    create=dict(levels=3, angle_start=-D(20), angle_extent=D(40)),
                    find=dict(angle_start=-D(20), angle_extent=D(40), min_score=0.7, num_matches=2,
                              max_overlap=0.5, subpixel=True, highest=3, lowest=1)),
    "polarity": dict(gen=dict(seed=14, height=480, width=640, tsize=64, n_poses=2, invert_odd=True),
                     create=dict(levels=3, angle_start=0.0, angle_extent=0.0, ignore_polarity=True),
                     find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.7, num_matches=0, max_overlap=0.5,
                               subpixel=True, highest=3, lowest=1)),
    "no_subpixel": dict(gen=dict(seed=15, height=480, width=640, tsize=48, n_poses=2, angle_range=(-D(10), D(10))),
                        create=dict(levels=3, angle_start=-D(10), angle_extent=D(20)),
                        find=dict(angle_start=-D(10), angle_extent=D(20), min_score=0.7, num_matches=2,
                                  max_overlap=0.5, subpixel=False, highest=3, lowest=1)),
    "lowest2": dict(gen=dict(seed=16, height=480, width=640, tsize=64, n_poses=2, angle_range=(-D(10), D(10))),
                    create=dict(levels=3, angle_start=-D(10), angle_extent=D(20)),
                    find=dict(angle_start=-D(10), angle_extent=D(20), min_score=0.6, num_matches=2,
                              max_overlap=0.5, subpixel=True, highest=3, lowest=2)),
    "endpoints": dict(gen=dict(seed=17, height=480, width=640, tsize=64, n_poses=2, angle_range=(-D(8), D(12))),
                      create=dict(levels=3, angle_start=-D(30), angle_extent=D(60)),
                      find=dict(angle_start=-0.2, angle_extent=0.45, min_score=0.7, num_matches=2, max_overlap=0.5,
                                subpixel=True, highest=3, lowest=1)),
    "border": dict(gen=dict(seed=18, height=400, width=500, tsize=64, n_poses=2, border=34.0),
                   create=dict(levels=3, angle_start=0.0, angle_extent=0.0),
                   find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.7, num_matches=2, max_overlap=0.5,
                             subpixel=True, highest=3, lowest=1)),
    "no_match": dict(gen=dict(seed=19, height=480, width=640, tsize=64, n_poses=1, noise_sigma=12),
                     create=dict(levels=3, angle_start=0.0, angle_extent=0.0),
                     find=dict(angle_start=0.0, angle_extent=0.0, min_score=0.99, num_matches=1, max_overlap=0.5,
                               subpixel=True, highest=3, lowest=1)),
    "mask_disc": dict(gen=dict(seed=20, height=480, width=640, tsize=64, n_poses=2, angle_range=(-D(15), D(15))),
                      create=dict(levels=3, angle_start=-D(15), angle_extent=D(30)),
                      find=dict(angle_start=-D(15), angle_extent=D(30), min_score=0.7, num_matches=2,
                                max_overlap=0.5, subpixel=True, highest=3, lowest=1),
                      mask="disc"),
    "overlap_tight": dict(gen=dict(seed=21, height=600, width=800, tsize=48, n_poses=4, angle_range=(-D(5), D(5))),
                          create=dict(levels=3, angle_start=-D(5), angle_extent=D(10)),
                          find=dict(angle_start=-D(5), angle_extent=D(10), min_score=0.5, num_matches=0,
                                    max_overlap=0.0, subpixel=True, highest=3, lowest=1)),
    # full-circle models: the angle list wraps, coarse stride and windows span it
    "full_circle": dict(gen=dict(seed=22, height=480, width=640, tsize=64, n_poses=3,
                                 angle_range=(-math.pi, math.pi)),
                        create=dict(levels=4, angle_start=-math.pi, angle_extent=2 * math.pi),
                        find=dict(angle_start=-math.pi, angle_extent=2 * math.pi, min_score=0.7, num_matches=3,
                                  max_overlap=0.5, subpixel=True, highest=4, lowest=1)),
    "full_circle_72": dict(gen=dict(seed=28, height=480, width=640, tsize=72, n_poses=3,
                                    angle_range=(-math.pi, math.pi)),
                           create=dict(levels=4, angle_start=-math.pi, angle_extent=2 * math.pi),
                           find=dict(angle_start=-math.pi, angle_extent=2 * math.pi, min_score=0.7, num_matches=0,
                                     max_overlap=0.5, subpixel=True, highest=4, lowest=1)),
    # automatic levels on a full circle: the reference exceeds its coarse
    # candidate budget and returns LimitExceeded (-103)
    "budget_360": dict(gen=dict(seed=22, height=480, width=640, tsize=48, n_poses=3,
                                angle_range=(-math.pi, math.pi)),
                       create=dict(levels=0, angle_start=-math.pi, angle_extent=2 * math.pi),
                       find=dict(angle_start=-math.pi, angle_extent=2 * math.pi, min_score=0.7, num_matches=3,
                                 max_overlap=0.5, subpixel=True, highest=0, lowest=1)),
    # query range wider than the trained range (clipped to it)
    "query_clip": dict(gen=dict(seed=24, height=480, width=640, tsize=56, n_poses=2, angle_range=(-D(18), D(18))),
                       create=dict(levels=3, angle_start=-D(20), angle_extent=D(40)),
                       find=dict(angle_start=-D(40), angle_extent=D(100), min_score=0.7, num_matches=2,
                                 max_overlap=0.5, subpixel=True, highest=3, lowest=1)),
    # 12-bit data in uint16 (the large-image configuration's format), wide angles
    "u16_12bit": dict(gen=dict(seed=25, height=480, width=640, tsize=64, n_poses=2, angle_range=(-D(45), D(45)),
                               maxval=4095, noise_sigma=20),
                      create=dict(levels=3, angle_start=-D(45), angle_extent=D(90)),
                      find=dict(angle_start=-D(45), angle_extent=D(90), min_score=0.6, num_matches=2,
                                max_overlap=0.5, subpixel=True, highest=3, lowest=1)),
    "tiny16": dict(gen=dict(seed=26, height=240, width=320, tsize=16, n_poses=2, angle_range=(-D(10), D(10))),
                   create=dict(levels=2, angle_start=-D(10), angle_extent=D(20)),
                   find=dict(angle_start=-D(10), angle_extent=D(20), min_score=0.7, num_matches=2, max_overlap=0.5,
                             subpixel=True, highest=2, lowest=1)),
    "big160": dict(gen=dict(seed=27, height=720, width=960, tsize=160, n_poses=2, angle_range=(-D(12), D(12))),
                   create=dict(levels=4, angle_start=-D(12), angle_extent=D(24)),
                   find=dict(angle_start=-D(12), angle_extent=D(24), min_score=0.7, num_matches=2, max_overlap=0.5,
                             subpixel=True, highest=4, lowest=1)),
    # shaped like the reference's demo (examples/ncc_matching.cpp:6-31):
    # automatic levels, an explicit angle step, NumLevels 0, one match
    "demo_like": dict(gen=dict(seed=30, height=320, width=480, tsize=56, n_poses=1, angle_range=(-0.3, 0.3)),
                      create=dict(levels=0, angle_start=-0.35, angle_extent=0.7, angle_step=0.025),
                      find=dict(angle_start=-0.35, angle_extent=0.7, min_score=0.75, num_matches=1,
                                max_overlap=0.5, subpixel=True, highest=0, lowest=1)),
}

# Reduced search domains (ROI, image.domain() in src/ncc_matching/matcher.cpp:
# 249-251, 375-393, 505-534, 633-643, 870-876, 954, 1034-1060) on one
# three-pose rotated scene.  "domain" lists shapes relative to the true poses
# (see search_domain); an empty list is an empty domain.
_ROI_GEN = dict(seed=11, height=600, width=800, tsize=64, n_poses=3, angle_range=(-D(30), D(30)))
_ROI_CREATE = dict(levels=3, angle_start=-D(30), angle_extent=D(60))
_ROI_FIND = dict(angle_start=-D(30), angle_extent=D(60), min_score=0.7, num_matches=0, max_overlap=0.5,
                 subpixel=True, highest=3, lowest=1)
for _name, _dom in {
        "roi_rect": [("around", 0, 40)],                      # one pose inside, dense domain
        "roi_two": [("around", 0, 20), ("around", 2, 20)],    # two far rectangles: sparse domain
        "roi_ring": [("ring", 1, 3, 30), ("around", 0, 2)],   # a hole at a pose centre, sparse
        "roi_strips": [("hline", 0, 0, 60), ("hline", 0, 6, 60)],  # two one-pixel rows
        "roi_point": [("around", 2, 0)],                      # one pixel at a pose
        "roi_border": [("left_of", 0, 5)],                    # full-height band cut through a pose
        "roi_empty": [],
}.items():
    CASES[_name] = dict(gen=_ROI_GEN, create=_ROI_CREATE, find=_ROI_FIND, domain=_dom)
CASES["roi_lowest2"] = dict(gen=_ROI_GEN, create=_ROI_CREATE, find=dict(_ROI_FIND, lowest=2),
                            domain=[("around", 0, 40), ("around", 1, 6)])
CASES["roi_no_subpixel"] = dict(gen=_ROI_GEN, create=_ROI_CREATE, find=dict(_ROI_FIND, subpixel=False),
                                domain=[("ring", 1, 2, 25), ("around", 2, 30)])


def search_domain(case: dict, wl):
    """The search-image domain mask of a case (None = the full image)."""
    import numpy as np
    if "domain" not in case:
        return None
    h, w = wl.image.shape
    m = np.zeros((h, w), np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    for shape in case["domain"]:
        p = wl.poses[shape[1]]
        r, c = int(math.floor(p.row + .5)), int(math.floor(p.column + .5))
        if shape[0] == "around":
            k = shape[2]
            m[max(0, r - k):r + k + 1, max(0, c - k):c + k + 1] = 1
        elif shape[0] == "ring":
            d2 = (yy - r) ** 2 + (xx - c) ** 2
            m[(d2 > shape[2] ** 2) & (d2 <= shape[3] ** 2)] = 1
        elif shape[0] == "hline":
            m[r + shape[2], max(0, c - shape[3]):c + shape[3] + 1] = 1
        elif shape[0] == "left_of":
            m[:, :c + shape[2] + 1] = 1
        else:
            raise ValueError(shape[0])
    return m


# The throughput configuration (2048^2 u8, one 128^2 template pasted 5 times
# at U[-30, 30] degrees), five seeds, checked against the reference at full size.
LARGE = {
    f"cfg2_s{k}": dict(gen=dict(seed=k, height=2048, width=2048, tsize=128, n_poses=5, angle_range=(-D(30), D(30))),
                       create=dict(levels=4, angle_start=-D(30), angle_extent=D(60)),
                       find=dict(angle_start=-D(30), angle_extent=D(60), min_score=0.7, num_matches=5,
                                 max_overlap=0.5, subpixel=True, highest=4, lowest=1))
    for k in range(1, 6)
}


def make_inputs(case: dict):
    wl = W.make_workload(**case["gen"])
    mask = None
    if case.get("mask") == "disc":
        import numpy as np
        t = wl.template.shape[0]
        yy, xx = np.mgrid[0:t, 0:t]
        c = (t - 1) / 2.0
        mask = ((yy - c) ** 2 + (xx - c) ** 2 <= (t / 2.0) ** 2).astype(np.uint8)
    return wl, mask
