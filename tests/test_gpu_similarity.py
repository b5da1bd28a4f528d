"""Differentiable sub-pixel refinement on the configuration's task, scaled
down: templates pasted at similarity poses (subpixel row and column, angle
over a full circle, scale 0.95-1.05) in a 1536^2 scene.  A full-circle
FindNccModels finds every paste; then, per degree of freedom, the pose error
against the pasted pose of

- the reference's rigid Gauss-Newton (the find's SubPixel "true" poses,
  scale 1),
- quadratic peak fitting (ncc_quadratic_peak_fit around the find's discrete
  SubPixel "false" poses),
- the adjoint-driven Gauss-Newton on (row, column, angle, scale)
  (ncc_refine_similarity from the rigid poses).

The adjoint form must be within 0.05 px, 0.05 deg and 2e-3 in scale on every
paste, and its median error below the other two forms' in every degree of
freedom."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    mvkit_gb300.load()
    return mvkit_gb300


def to_matcher(r, c, a):
    """The matcher's pixel-centre pose of the operator's edge-centred one."""
    ca, sa = np.cos(a), np.sin(a)
    return r - .5 * (1 - ca + sa), c - .5 * (1 - ca - sa)


def pose_errors(poses, model_of, truth):
    """|drow|, |dcol|, |dangle| (deg), |dscale| of the nearest pose of the
    paste's model for every paste (None: none within 3 px)."""
    out = []
    for t in truth:
        sel = np.nonzero(model_of == t.model)[0]
        d = np.hypot(poses[sel, 0] - t.row, poses[sel, 1] - t.column) if len(sel) else np.zeros(0)
        if not len(sel) or d.min() > 3:
            out.append(None)
            continue
        p = poses[sel[int(np.argmin(d))]]
        out.append((abs(p[0] - t.row), abs(p[1] - t.column),
                    abs(math.degrees(math.remainder(p[2] - t.angle, 2 * math.pi))), abs(p[3] - t.scale)))
    return out


def refine_all(mg, image, models, ctl):
    """(rigid, quadratic, adjoint) poses (n, 4) and model indices of the
    rigid and discrete finds."""
    found = {}
    for sp in ("true", "false"):
        r, c, a, _, m = mg.find_ncc_models(image, models, *ctl[:5], sp, ctl[6])
        mr, mc = to_matcher(r, c, a)
        found[sp] = (np.stack([mr, mc, a, np.ones_like(a)], axis=1), m)
    rigid, mr_ = found["true"]
    discrete, md = found["false"]
    adjoint, quad = rigid.copy(), discrete.copy()
    for k, model in enumerate(models):
        if (mr_ == k).any():
            adjoint[mr_ == k], _ = mg.ncc_refine_similarity(image, model, rigid[mr_ == k], iterations=40)
        if (md == k).any():
            step = mg.get_ncc_model_params(model)[3]
            quad[md == k], _ = mg.ncc_quadratic_peak_fit(image, model, discrete[md == k], (1.0, 1.0, step, 0.02))
    return rigid, mr_, quad, md, adjoint


def test_adjoint_refinement_beats_rigid_and_quadratic_fit(mg):
    from mvkit_gb300 import workloads as W
    wl = W.make_similarity_workload(4, 1536, 1536, (128, 160), 8)
    with mg.extended_budgets(samples=200_000_000, candidates=1 << 20):
        models = [mg.create_ncc_model(t, 4, -math.pi, 2 * math.pi, "auto", "use_polarity") for t in wl.templates]
        rigid, mr_, quad, md, adjoint = refine_all(mg, wl.image, models,
                                                   (-math.pi, 2 * math.pi, 0.4, [4, 4], 0.5, None, 4))
    e = {name: pose_errors(p, m, wl.poses) for name, p, m in
         (("rigid", rigid, mr_), ("quadratic", quad, md), ("adjoint", adjoint, mr_))}
    for name, v in e.items():
        assert all(x is not None for x in v), f"{name}: a paste was not found"
    adj = np.array(e["adjoint"])
    assert adj[:, :2].max() <= 0.05 and adj[:, 2].max() <= 0.05 and adj[:, 3].max() <= 2e-3, adj
    med = {k: np.median(np.array(v), axis=0) for k, v in e.items()}
    assert np.all(med["adjoint"] < med["rigid"][[0, 1, 2, 3]]), med
    assert np.all(med["adjoint"] < med["quadratic"]), med
