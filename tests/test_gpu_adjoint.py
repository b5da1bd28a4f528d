"""The NCC adjoint with a scale degree of freedom (mvg_ncc_score_gradient; the
reference is rigid and has no counterpart).

Checked three ways on seeded scenes:
- against an FP64 NumPy restatement of the same warp, bilinear sampling and
  NCC algebra (scores within 2e-6, gradients within 1e-4 + 1e-3 relative:
  the device sums in FP32 with pair totals);
- against central finite differences (h = 1e-3 in pixels, radians and
  scale units) of the device score, with the bilinear cell crossings of a
  step accounted for (see test_adjoint_central_differences);
- through a torch.autograd.Function defined here, in the test harness only,
  whose backward is the device gradient.
"""
import math

import numpy as np
import pytest

import oracle_lib
from golden.cases import CASES, make_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    mvkit_gb300.load()
    return mvkit_gb300


def original_raster(case, wl, mask):
    """(dr, dc, w) of the model's unrotated level-0 raster, from the oracle."""
    orc = oracle_lib.oracle()
    c = case["create"]
    om = orc.create(wl.template, levels=c["levels"], angle_start=c["angle_start"], angle_extent=c["angle_extent"],
                    ignore_polarity=c.get("ignore_polarity", False), mask=mask)
    p = om.patch(-1, 0)
    return p["rows"] - p["origin_row"], p["cols"] - p["origin_column"], p["weights"]


def ncc64(img, dr, dc, w, pose, absolute=False):
    """FP64 score and gradient of one similarity pose (the kernel's algebra)."""
    row, col, ang, s = pose
    ca, sa = math.cos(ang), math.sin(ang)
    u, v = ca * dr - sa * dc, sa * dr + ca * dc
    y, x = row + s * u, col + s * v
    h, W = img.shape
    if y.min() < 0 or x.min() < 0 or y.max() > h - 1 or x.max() > W - 1:
        return -math.inf, np.zeros(4)
    iy, ix = np.floor(y).astype(np.int64), np.floor(x).astype(np.int64)
    fy, fx = y - iy, x - ix
    iy1, ix1 = np.minimum(iy + 1, h - 1), np.minimum(ix + 1, W - 1)
    f = img.astype(np.float64)
    a, b, d, e = f[iy, ix], f[iy, ix1], f[iy1, ix], f[iy1, ix1]
    q = (1 - fy) * ((1 - fx) * a + fx * b) + fy * ((1 - fx) * d + fx * e)
    gy = (1 - fx) * (d - a) + fx * (e - b)
    gx = (1 - fy) * (b - a) + fy * (e - d)
    dq = [gy, gx, s * (gx * u - gy * v), gy * u + gx * v]
    n = len(q)
    D = (w * q).sum() - q.sum() / n * w.sum()
    E = (q * q).sum() - q.sum() ** 2 / n
    ncc = D / math.sqrt(E)
    sign = -1.0 if absolute and ncc < 0 else 1.0
    g = np.zeros(4)
    for j in range(4):
        dD = (w * dq[j]).sum() - dq[j].sum() / n * w.sum()
        dE = 2 * ((q * dq[j]).sum() - q.sum() * dq[j].sum() / n)
        g[j] = sign * (dD / math.sqrt(E) - D * dE / (2 * E ** 1.5))
    return sign * ncc, g


def poses_near_truth(wl, seed, per=4):
    rng = np.random.default_rng(seed)
    out = []
    for p in wl.poses:
        for _ in range(per):
            out.append([p.row + rng.uniform(-0.6, 0.6), p.column + rng.uniform(-0.6, 0.6),
                        p.angle + rng.uniform(-0.03, 0.03), 1 + rng.uniform(-0.04, 0.04)])
    return np.array(out)


@pytest.mark.parametrize("name", ["rot3_all", "u16_rot", "polarity"])
def test_adjoint_matches_fp64_restatement(mg, name):
    case = CASES[name]
    wl, mask = make_inputs(case)
    c = case["create"]
    model = mg.create_ncc_model(wl.template, c["levels"], c["angle_start"], c["angle_extent"], "auto",
                                "ignore_global_polarity" if c.get("ignore_polarity") else "use_polarity")
    dr, dc, w = original_raster(case, wl, mask)
    poses = poses_near_truth(wl, 7)
    score, grad = mg.ncc_score_gradient(wl.image, model, poses)
    for k, pose in enumerate(poses):
        s64, g64 = ncc64(wl.image, dr, dc, w, pose, c.get("ignore_polarity", False))
        assert abs(score[k] - s64) <= 2e-6, (k, score[k], s64)
        assert np.all(np.abs(grad[k] - g64) <= 1e-4 + 1e-3 * np.abs(g64)), (k, grad[k], g64)


def test_adjoint_central_differences(mg):
    """The gradient against central differences.  A step moves samples across
    bilinear cell boundaries (an angle or scale step of h moves a sample at
    radius r by about h r pixels), where the one-sided cell derivative that
    the gradient uses jumps.  So: FP64 differences at h = 1e-7 equal the FP64
    analytic gradient (the algebra), device differences at h = 1e-3 equal
    FP64 differences at the same h (the kernel), and for row and column
    (h r = 1e-3 px) the device differences equal the device gradient."""
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    c = case["create"]
    model = mg.create_ncc_model(wl.template, c["levels"], c["angle_start"], c["angle_extent"], "auto",
                                "use_polarity")
    dr, dc, w = original_raster(case, wl, mask)
    poses = poses_near_truth(wl, 11, per=3)
    score, grad = mg.ncc_score_gradient(wl.image, model, poses)
    for k in range(0, len(poses), 3):
        _, g64 = ncc64(wl.image, dr, dc, w, poses[k])
        for j in range(4):
            e = np.zeros(4)
            e[j] = 1e-7
            fd = (ncc64(wl.image, dr, dc, w, poses[k] + e)[0] - ncc64(wl.image, dr, dc, w, poses[k] - e)[0]) / 2e-7
            assert abs(fd - g64[j]) <= 1e-5 + 1e-4 * abs(g64[j]), (k, j, fd, g64[j])
    h = 1e-3
    for j in range(4):
        e = np.zeros(4)
        e[j] = h
        sp, _ = mg.ncc_score_gradient(wl.image, model, poses + e)
        sm, _ = mg.ncc_score_gradient(wl.image, model, poses - e)
        fd = (sp - sm) / (2 * h)
        fd64 = np.array([(ncc64(wl.image, dr, dc, w, p + e)[0] - ncc64(wl.image, dr, dc, w, p - e)[0]) / (2 * h)
                         for p in poses])
        assert np.all(np.abs(fd - fd64) <= 2e-4 + 1e-3 * np.abs(fd64)), (j, fd, fd64)
        if j < 2:
            assert np.all(np.abs(fd - grad[:, j]) <= 1e-3 + 2e-2 * np.abs(grad[:, j])), (j, fd, grad[:, j])


def test_adjoint_edges(mg):
    """Outside the image: -inf and a zero gradient; no poses: no work."""
    case = CASES["cfg1_s1"]
    wl, mask = make_inputs(case)
    model = mg.create_ncc_model(wl.template, 3, 0.0, 0.0, "auto", "use_polarity")
    s, g = mg.ncc_score_gradient(wl.image, model, [[5.0, 5.0, 0.0, 1.0], [240.0, 320.0, 0.0, 1.0]])
    assert s[0] == -math.inf and np.all(g[0] == 0)
    assert np.isfinite(s[1])
    s, g = mg.ncc_score_gradient(wl.image, model, np.zeros((0, 4)))
    assert s.shape == (0,) and g.shape == (0, 4)


def test_adjoint_torch_autograd(mg):
    """A torch.autograd.Function over the C ABI: backward returns the
    device gradient; finite differences of its forward agree with it."""
    torch = pytest.importorskip("torch")
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    c = case["create"]
    model = mg.create_ncc_model(wl.template, c["levels"], c["angle_start"], c["angle_extent"], "auto",
                                "use_polarity")

    class NccScore(torch.autograd.Function):
        @staticmethod
        def forward(ctx, poses):
            s, g = mg.ncc_score_gradient(wl.image, model, poses.detach().cpu().numpy())
            ctx.save_for_backward(torch.from_numpy(g))
            return torch.from_numpy(s)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout[:, None] * g

    poses = torch.tensor(poses_near_truth(wl, 5, per=2), dtype=torch.float64, requires_grad=True)
    wts = torch.linspace(0.5, 1.5, poses.shape[0], dtype=torch.float64)
    (NccScore.apply(poses) * wts).sum().backward()
    _, g = mg.ncc_score_gradient(wl.image, model, poses.detach().numpy())
    np.testing.assert_allclose(poses.grad.numpy(), wts.numpy()[:, None] * g, rtol=0, atol=0)
    h = 1e-3
    with torch.no_grad():
        # row and column (angle and scale steps cross bilinear cells; they
        # are checked against FP64 differences above)
        for j in range(2):
            e = torch.zeros(4, dtype=torch.float64)
            e[j] = h
            fd = (NccScore.apply(poses + e) - NccScore.apply(poses - e)) / (2 * h)
            tol = 1e-3 + 2e-2 * torch.from_numpy(g[:, j]).abs()
            assert torch.all((fd - torch.from_numpy(g[:, j])).abs() <= tol)


def paste_similarity(img, tmpl, row, col, angle, scale):
    """FP64 paste of a square template at a similarity pose: the template
    offset (dr, dc) from its centre lands at row + s (cos dr - sin dc),
    col + s (sin dr + cos dc); each covered image pixel takes the template's
    bilinear value at the inverse-mapped offset."""
    t = tmpl.shape[0]
    o = (t - 1) / 2
    ca, sa = math.cos(angle), math.sin(angle)
    reach = int(math.ceil(scale * t * 0.75)) + 2
    r0, c0 = int(row) - reach, int(col) - reach
    yy, xx = np.mgrid[r0:r0 + 2 * reach + 1, c0:c0 + 2 * reach + 1].astype(np.float64)
    dy, dx = yy - row, xx - col
    tr = (ca * dy + sa * dx) / scale + o
    tc = (-sa * dy + ca * dx) / scale + o
    inside = (tr >= 0) & (tc >= 0) & (tr <= t - 1) & (tc <= t - 1)
    ir, ic = np.clip(np.floor(tr).astype(int), 0, t - 1), np.clip(np.floor(tc).astype(int), 0, t - 1)
    ir1, ic1 = np.minimum(ir + 1, t - 1), np.minimum(ic + 1, t - 1)
    fr, fc = tr - np.floor(tr), tc - np.floor(tc)
    f = tmpl.astype(np.float64)
    v = (1 - fr) * ((1 - fc) * f[ir, ic] + fc * f[ir, ic1]) + fr * ((1 - fc) * f[ir1, ic] + fc * f[ir1, ic1])
    region = img[r0:r0 + 2 * reach + 1, c0:c0 + 2 * reach + 1]
    region[inside] = v[inside]


def test_similarity_refinement_recovers_scale(mg):
    """Templates pasted at scales 0.96-1.04: Gauss-Newton on (row, column,
    angle, scale) from the unit-scale pose nearby recovers the pose within
    0.05 px, 0.1 deg and 3e-3 in scale, and raises the score.  The pasted
    patch is larger than the model's template (the same texture continues
    around it), as in a real scene: a template pasted with hard edges would
    let the edge samples mix in background and bias the scale."""
    from mvkit_gb300 import workloads as W
    src = W.scene(63, 240, 240)
    big = np.clip(src[50:146, 60:156], 0, 255).astype(np.uint8)   # 96 x 96, centre 47.5
    tmpl = np.ascontiguousarray(big[16:80, 16:80])                 # 64 x 64, centre 31.5
    img = W.scene(62, 480, 640).astype(np.float64)
    truth = [(120.3, 150.7, 0.12, 0.96), (130.6, 470.2, -0.2, 0.98), (340.1, 160.4, 0.05, 1.02),
             (350.8, 480.9, -0.08, 1.04)]
    for p in truth:
        paste_similarity(img, big, *p)
    image = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    model = mg.create_ncc_model(tmpl, 3, -0.3, 0.6, "auto", "use_polarity")
    rng = np.random.default_rng(3)
    start = np.array([[r + rng.uniform(-0.4, 0.4), c + rng.uniform(-0.4, 0.4), a + rng.uniform(-0.01, 0.01), 1.0]
                      for r, c, a, s in truth])
    s0, _ = mg.ncc_score_gradient(image, model, start)
    refined, score = mg.ncc_refine_similarity(image, model, start, iterations=40)
    err = np.abs(refined - np.array(truth))
    assert np.all(err[:, :2] <= 0.05), err
    assert np.all(err[:, 2] <= math.radians(0.1)), err
    assert np.all(err[:, 3] <= 3e-3), err
    assert np.all(score > s0) and np.all(score > 0.95), (s0, score)
    # the reported score is the score at the refined pose
    s1, _ = mg.ncc_score_gradient(image, model, refined)
    np.testing.assert_allclose(score, s1, atol=1e-6)
    # iterations = 0 leaves the poses and reports their scores
    same, s2 = mg.ncc_refine_similarity(image, model, start, iterations=0)
    np.testing.assert_array_equal(same, start)
    np.testing.assert_allclose(s2, s0, atol=1e-6)
