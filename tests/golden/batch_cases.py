"""Batched FindNccModels parity cases: batches of scenes of uneven size that
share one template set, each scene searched for every model with the same
control tuples (mv_find_ncc_models per image,
src/c_api/ncc_matching_api.cpp:191-201 over find_models,
src/ncc_matching/matcher.cpp:1077-1124).

The scenes come from mvkit_gb300.workloads.make_batch_workloads.  Sizes are
the batched benchmark configuration's (512x512 ... 4096x3000) scaled down so
the reference finishes each batch in about a minute; templates, 360 degree
rotation, +-10 % contrast and noise sigma 5 follow it.  make_batch.py
records the reference's per-image status and matches into batch.json."""
from __future__ import annotations

import math

from mvkit_gb300 import workloads as W

FULL = (-math.pi, 2 * math.pi)

BATCH_CASES = {
    # full circle: the smaller scenes give matches, the larger ones exceed the
    # reference's coarse candidate budget (LimitExceeded, per image)
    "batch_360": dict(
        gen=dict(seed=3, n_images=4, sizes=((384, 512), (480, 640), (768, 1024)), tsizes=(64, 96), max_pastes=2,
                 angle_range=(-math.pi, math.pi)),
        create=dict(levels=4, angle_start=FULL[0], angle_extent=FULL[1]),
        find=dict(angle_start=[FULL[0]], angle_extent=[FULL[1]], min_score=[0.7], num_matches=[0],
                  max_overlap=[0.5], subpixel=["true"], num_levels=[4])),
    # three templates over +-30 degrees on six scenes of three sizes,
    # per-model match quotas
    "batch_uneven": dict(
        gen=dict(seed=5, n_images=6, sizes=((320, 400), (480, 640), (600, 800)), tsizes=(40, 56, 72),
                 max_pastes=2, angle_range=(-math.radians(30), math.radians(30))),
        create=dict(levels=3, angle_start=-math.radians(30), angle_extent=math.radians(60)),
        find=dict(angle_start=[-math.radians(30)], angle_extent=[math.radians(60)], min_score=[0.7],
                  num_matches=[2, 1, 2], max_overlap=[0.5], subpixel=["true"], num_levels=[3])),
    # the batched configuration's own controls (automatic levels, full
    # circle, MinScore 0.6) with four of its template sizes: the reference
    # returns LimitExceeded for every scene
    "batch_auto_controls": dict(
        gen=dict(seed=9, n_images=3, sizes=((512, 512), (1024, 1280)), tsizes=(32, 48, 64, 96), max_pastes=1,
                 angle_range=(-math.pi, math.pi)),
        create=dict(levels=0, angle_start=FULL[0], angle_extent=FULL[1]),
        find=dict(angle_start=[FULL[0]], angle_extent=[FULL[1]], min_score=[0.6], num_matches=[0],
                  max_overlap=[0.5], subpixel=["true"], num_levels=[0])),
}


def make_batch_inputs(case: dict) -> list:
    return W.make_batch_workloads(**case["gen"])
