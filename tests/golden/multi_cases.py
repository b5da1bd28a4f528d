"""FindNccModels parity cases (mv_find_ncc_models,
src/c_api/ncc_matching_api.cpp:191-201 over find_models,
src/ncc_matching/matcher.cpp:1077-1124).

Each case builds one multi-template scene (mvkit_gb300.workloads.
make_multi_workload), one model per entry of "models" (a template index and
create options; "same": k reuses model k's handle), and passes the control
tuples as the operator receives them.  make_multi.py records the reference's
matches into multi.json; the GPU tests call find_ncc_models with the same
tuples."""
from __future__ import annotations

import math

from mvkit_gb300 import workloads as W

D = math.radians
R3 = dict(levels=3, angle_start=-0.3, angle_extent=0.6)

MULTI_CASES = {
    # three different templates, everything shared: all matches, one overlap rule
    "three_shared": dict(
        gen=dict(seed=41, height=480, width=640, tsizes=(64, 48, 56), n_poses=(2, 2, 1), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=1, create=R3), dict(t=2, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.7], num_matches=[0], max_overlap=[0.5],
                  subpixel=["true"], num_levels=[3])),
    # per-model quotas with a shared overlap: quotas first, then cross-model
    # suppression (HALCON's rule)
    "per_model_quota": dict(
        gen=dict(seed=42, height=480, width=640, tsizes=(64, 48, 56), n_poses=(2, 2, 2), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=1, create=R3), dict(t=2, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.7], num_matches=[1, 2, 1],
                  max_overlap=[0.5], subpixel=["true"], num_levels=[3])),
    # per-model overlap thresholds with a shared limit of 3 matches
    "per_model_overlap": dict(
        gen=dict(seed=43, height=480, width=640, tsizes=(64, 48), n_poses=(3, 2), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=1, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.7], num_matches=[3],
                  max_overlap=[0.5, 0.2], subpixel=["true"], num_levels=[3])),
    # the same template as two models and one model handle given twice:
    # cross-model suppression removes the copies
    "duplicates_shared": dict(
        gen=dict(seed=44, height=480, width=640, tsizes=(64, 48), n_poses=(2, 1), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=0, create=R3), dict(same=0), dict(t=1, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.7], num_matches=[0], max_overlap=[0.5],
                  subpixel=["true"], num_levels=[3])),
    # ... and with per-model overlap each copy keeps its matches
    "duplicates_per_model": dict(
        gen=dict(seed=44, height=480, width=640, tsizes=(64, 48), n_poses=(2, 1), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=0, create=R3), dict(same=0), dict(t=1, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.7], num_matches=[0],
                  max_overlap=[0.5, 0.5, 0.5, 0.5], subpixel=["true"], num_levels=[3])),
    # different level pairs and angle ranges per model; one model without
    # subpixel refinement
    "mixed_levels": dict(
        gen=dict(seed=45, height=480, width=640, tsizes=(64, 56), n_poses=(2, 2), angle_range=(-0.2, 0.2)),
        models=[dict(t=0, create=dict(levels=3, angle_start=-0.3, angle_extent=0.6)),
                dict(t=1, create=dict(levels=3, angle_start=-0.25, angle_extent=0.5))],
        find=dict(angle_start=[-0.3, -0.25], angle_extent=[0.6, 0.5], min_score=[0.7, 0.6], num_matches=[2],
                  max_overlap=[0.5], subpixel=["true", "false"], num_levels=[3, 1, 3, 2])),
    # a shared match limit smaller than the matches present
    "shared_limit": dict(
        gen=dict(seed=46, height=600, width=800, tsizes=(48, 48, 40), n_poses=(2, 2, 2), angle_range=(-0.3, 0.3)),
        models=[dict(t=0, create=R3), dict(t=1, create=R3), dict(t=2, create=R3)],
        find=dict(angle_start=[-0.3], angle_extent=[0.6], min_score=[0.6], num_matches=[3], max_overlap=[0.5],
                  subpixel=["true"], num_levels=[3])),
    # 12-bit data in uint16
    "u16_two": dict(
        gen=dict(seed=47, height=480, width=640, tsizes=(64, 48), n_poses=(2, 2), angle_range=(-D(15), D(15)),
                 maxval=4095, noise_sigma=20),
        models=[dict(t=0, create=dict(levels=3, angle_start=-D(15), angle_extent=D(30))),
                dict(t=1, create=dict(levels=3, angle_start=-D(15), angle_extent=D(30)))],
        find=dict(angle_start=[-D(15)], angle_extent=[D(30)], min_score=[0.6], num_matches=[0], max_overlap=[0.5],
                  subpixel=["true"], num_levels=[3])),
}


def make_multi_inputs(case: dict):
    return W.make_multi_workload(**case["gen"])


def expand(find: dict, n: int):
    """Per-model FindOptions and the shared selection from the control tuples
    (NccControls, src/c_api/ncc_matching_api.cpp:126-162).  Returns (list of
    option dicts, selection num_matches, selection max_overlap)."""
    def pick(v, i):
        return v[0] if len(v) == 1 else v[i]
    lv = find["num_levels"]
    opts = []
    for i in range(n):
        hi, lo, pair = 0, 0, False
        if len(lv) == n and n > 1:
            hi = i
        elif len(lv) == 2 * n:
            hi, lo, pair = 2 * i, 2 * i + 1, True
        elif len(lv) == 2:
            lo, pair = 1, True
        opts.append(dict(angle_start=pick(find["angle_start"], i), angle_extent=pick(find["angle_extent"], i),
                         min_score=pick(find["min_score"], i), num_matches=pick(find["num_matches"], i),
                         max_overlap=pick(find["max_overlap"], i), subpixel=pick(find["subpixel"], i) == "true",
                         highest=lv[hi], lowest=max(1, lv[lo] if pair else 1)))
    sel_n = find["num_matches"][0] if len(find["num_matches"]) == 1 else -1
    sel_o = find["max_overlap"][0] if len(find["max_overlap"]) == 1 else -1.0
    return opts, sel_n, sel_o
