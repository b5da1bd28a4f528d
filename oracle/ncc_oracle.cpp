// Test infrastructure only (the checker, never the product).
//
// FP64 CPU restatement of the reference mvkit NCC matching path as the
// reference's scalar build runs it (MVKIT_NCC_HAS_AVX2=0, single model, no
// query caches).  Every function cites the reference lines it follows.
// Floating-point expressions keep the reference's evaluation order and are
// compiled with -ffp-contract=off so the results are bit-identical to the
// reference built the same way (checked by tests/test_oracle.py against
// libref_scalar.so and against tests/golden/).
#include "ncc_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace orc {
namespace {

constexpr double kTau = 6.283185307179586476925286766559;
constexpr std::size_t kMaxPixels = 1048576, kMaxAngles = 4096;
// Budgets (model.cpp:15, matcher.cpp:373-374, model.hpp:21): the reference's
// by default; orc_set_budgets lifts them for checking the library's extended
// mode (process-wide, set before the calls it applies to).
std::size_t g_max_samples = 16000000;
long long g_max_image_pixels = 32000000;
std::size_t g_max_candidates = 10000;
const double kMissing = -std::numeric_limits<double>::infinity();

enum Status : int {
  kOk = 0, kInvalidArgument = -1, kInvalidState = -7, kLimitExceeded = -103, kInternal = -1000,
  kOutOfMemory = -5
};
struct Failure {
  int status;
  std::string message;
};
[[noreturn]] void fail(int status, const char* message) { throw Failure{status, message}; }

struct Sample { std::int32_t row, col; double w; };
struct Run { std::int32_t row, begin, end; };
struct Patch {
  double angle = 0, orow = 0, ocol = 0;
  std::int32_t rmin = 0, rmax = 0, cmin = 0, cmax = 0;
  std::vector<Sample> s;
  std::vector<double> relr, relc;
  double wsum = 0;
  std::vector<Run> runs;
};
struct Level {
  std::size_t w = 0, h = 0;
  double orow = 0, ocol = 0;
  std::vector<double> gray;
  std::vector<std::uint8_t> mask;
  std::vector<Patch> patches;
};
struct CreateOpts { int levels = 0; bool ignore = false; double start = 0, extent = 0, step = 0; };
struct Model {
  CreateOpts opt;
  std::size_t sample_count = 0;
  double orow = 0, ocol = 0;
  Patch original;
  std::vector<Level> levels;
};
struct Pose { double row = 0, col = 0, angle = 0, score = 0; };
struct FindOpts {
  double start = 0, extent = 0, min_score = .8, max_overlap = .5;
  std::size_t num_matches = 1, max_candidates = g_max_candidates;
  bool subpixel = true;
  int highest = 0, lowest = 1;
};

// Search-image domain as sorted runs (row, begin, end); `full` marks the
// image's own rectangle (no reduced domain).
struct Domain {
  bool full = true;
  std::int64_t height = 0, width = 0;
  std::vector<Run> runs;
  std::int64_t rmin = 0, rmax = -1, cmin = 0, cmax = -1;
  std::int64_t area = 0;
  bool contains(std::int64_t r, std::int64_t c) const {
    if (full) return r >= 0 && c >= 0 && r < height && c < width;
    auto it = std::lower_bound(runs.begin(), runs.end(), r,
                               [](const Run& a, std::int64_t row) { return a.row < row; });
    for (; it != runs.end() && it->row == r; ++it)
      if (c >= it->begin && c <= it->end) return true;
    return false;
  }
};

Domain make_domain(std::int64_t w, std::int64_t h, const std::uint8_t* mask) {
  Domain d;
  d.width = w;
  d.height = h;
  if (!mask) {
    d.full = true;
    for (std::int64_t r = 0; r < h; ++r) d.runs.push_back({std::int32_t(r), 0, std::int32_t(w - 1)});
    d.rmin = 0; d.rmax = h - 1; d.cmin = 0; d.cmax = w - 1; d.area = w * h;
    return d;
  }
  d.full = false;
  d.rmin = h; d.cmin = w;
  for (std::int64_t r = 0; r < h; ++r) {
    std::int64_t c = 0;
    while (c < w) {
      while (c < w && !mask[r * w + c]) ++c;
      if (c >= w) break;
      const auto b = c;
      while (c < w && mask[r * w + c]) ++c;
      d.runs.push_back({std::int32_t(r), std::int32_t(b), std::int32_t(c - 1)});
      d.area += c - b;
      d.rmin = std::min(d.rmin, r); d.rmax = std::max(d.rmax, r);
      d.cmin = std::min(d.cmin, b); d.cmax = std::max(d.cmax, c - 1);
    }
  }
  return d;
}

// ---------------------------------------------------------------- model build
// src/ncc_matching/model.cpp:38-65 (normalize)
struct Normalization { double mean, energy; };
bool normalize(Patch& p, const Normalization* prepared) {
  if (p.s.size() < 4) return false;
  double mean = prepared ? prepared->mean : 0;
  if (!prepared)
    for (std::size_t i = 0; i < p.s.size(); ++i) mean += (p.s[i].w - mean) / double(i + 1);
  double energy = prepared ? prepared->energy : 0;
  if (prepared) {
    for (auto& x : p.s) x.w -= mean;
  } else {
    for (auto& x : p.s) { x.w -= mean; energy += x.w * x.w; }
  }
  if (!(energy > 0) || !std::isfinite(energy)) return false;
  const double scale = 1 / std::sqrt(energy);
  p.rmin = p.rmax = p.s.front().row;
  p.cmin = p.cmax = p.s.front().col;
  for (auto& x : p.s) {
    x.w *= scale;
    p.wsum += x.w;
    p.rmin = std::min(p.rmin, x.row); p.rmax = std::max(p.rmax, x.row);
    p.cmin = std::min(p.cmin, x.col); p.cmax = std::max(p.cmax, x.col);
    if (!p.runs.empty() && p.runs.back().row == x.row && p.runs.back().end + 1 == x.col) p.runs.back().end = x.col;
    else p.runs.push_back({x.row, x.col, x.col});
  }
  return true;
}

// src/ncc_matching/model.cpp:66-98 (rotate): bilinear resample of the level
// about its origin; a sample survives only when its four neighbours are masked.
Patch rotate(const Level& L, double angle, const Normalization* prepared) {
  Patch p;
  p.angle = angle;
  if (std::abs(std::remainder(angle, kTau)) < 1e-12) {
    p.orow = L.orow; p.ocol = L.ocol;
    for (std::size_t r = 0; r < L.h; ++r)
      for (std::size_t c = 0; c < L.w; ++c)
        if (L.mask[r * L.w + c]) p.s.push_back({int(r), int(c), L.gray[r * L.w + c]});
    if (!normalize(p, prepared)) p.s.clear();
    return p;
  }
  const double ca = std::cos(angle), sa = std::sin(angle);
  double rmin = 0, rmax = 0, cmin = 0, cmax = 0;
  for (double r : {0., double(L.h - 1)})
    for (double c : {0., double(L.w - 1)}) {
      const double dr = r - L.orow, dc = c - L.ocol;
      const double rr = ca * dr - sa * dc, cc = sa * dr + ca * dc;
      rmin = std::min(rmin, rr); rmax = std::max(rmax, rr);
      cmin = std::min(cmin, cc); cmax = std::max(cmax, cc);
    }
  const double rw = std::ceil(rmax) - std::floor(rmin) + 1, cw = std::ceil(cmax) - std::floor(cmin) + 1;
  if (rw > 4 * kMaxPixels / cw) fail(kLimitExceeded, "rotated bounding box exceeds budget");
  for (int r = int(std::floor(rmin)); r <= int(std::ceil(rmax)); ++r)
    for (int c = int(std::floor(cmin)); c <= int(std::ceil(cmax)); ++c) {
      const double rr = ca * r + sa * c + L.orow, cc = -sa * r + ca * c + L.ocol;
      if (rr < 0 || cc < 0 || rr > L.h - 1 || cc > L.w - 1) continue;
      const std::size_t r0 = std::size_t(rr), c0 = std::size_t(cc);
      const std::size_t r1 = std::min(r0 + 1, L.h - 1), c1 = std::min(c0 + 1, L.w - 1);
      const std::size_t a = r0 * L.w + c0, b = r0 * L.w + c1, d = r1 * L.w + c0, e = r1 * L.w + c1;
      if (!L.mask[a] || !L.mask[b] || !L.mask[d] || !L.mask[e]) continue;
      const double fr = rr - r0, fc = cc - c0;
      p.s.push_back({r, c, (1 - fr) * ((1 - fc) * L.gray[a] + fc * L.gray[b]) +
                               fr * ((1 - fc) * L.gray[d] + fc * L.gray[e])});
    }
  if (!normalize(p, nullptr)) p.s.clear();
  return p;
}

// src/ncc_matching/model.cpp:20-36 (validate_zero)
bool level_ok(const Level& L, std::size_t* count) {
  std::size_t n = 0;
  double mean = 0;
  for (std::size_t i = 0; i < L.w * L.h; ++i)
    if (L.mask[i]) mean += (L.gray[i] - mean) / double(++n);
  *count = 0;
  if (n < 4) return false;
  double energy = 0;
  for (std::size_t i = 0; i < L.w * L.h; ++i)
    if (L.mask[i]) { const double v = L.gray[i] - mean; energy += v * v; }
  if (!(energy > 0) || !std::isfinite(energy)) return false;
  *count = n;
  return true;
}

// src/ncc_matching/model.cpp:173-242 (rebuild)
Model rebuild(Level first, const CreateOpts& opt, double orow, double ocol) {
  Model m;
  m.opt = opt;
  m.orow = orow; m.ocol = ocol;
  m.sample_count = std::size_t(std::count(first.mask.begin(), first.mask.end(), std::uint8_t{1}));
  m.levels.push_back(std::move(first));
  Normalization first_norm{};
  {
    const Level& L = m.levels.front();
    Patch& p = m.original;
    p.orow = L.orow; p.ocol = L.ocol;
    double mean = 0;
    std::size_t count = 0;
    for (std::size_t i = 0; i < L.gray.size(); ++i)
      if (L.mask[i]) mean += (L.gray[i] - mean) / double(++count);
    double energy = 0;
    for (std::size_t r = 0; r < L.h; ++r)
      for (std::size_t c = 0; c < L.w; ++c)
        if (L.mask[r * L.w + c]) {
          const double v = L.gray[r * L.w + c] - mean;
          energy += v * v;
          p.s.push_back({int(r), int(c), v});
        }
    if (count < 4 || !(energy > 0) || !std::isfinite(energy))
      fail(kInvalidArgument, "constant template cannot define an NCC model");
    first_norm = {mean, energy};
    const double norm = std::sqrt(energy);
    p.rmin = p.rmax = p.s.front().row;
    p.cmin = p.cmax = p.s.front().col;
    for (auto& x : p.s) {
      x.w /= norm;
      p.rmin = std::min(p.rmin, x.row); p.rmax = std::max(p.rmax, x.row);
      p.cmin = std::min(p.cmin, x.col); p.cmax = std::max(p.cmax, x.col);
      p.relr.push_back(x.row - L.orow);
      p.relc.push_back(x.col - L.ocol);
    }
  }
  const int wanted = opt.levels ? opt.levels : 16;
  while (m.levels.size() < std::size_t(wanted)) {
    const Level& prev = m.levels.back();
    if (prev.w < 8 || prev.h < 8) break;
    Level next;
    next.w = prev.w / 2; next.h = prev.h / 2;
    next.orow = (prev.orow - .5) * .5; next.ocol = (prev.ocol - .5) * .5;
    next.gray.resize(next.w * next.h);
    next.mask.resize(next.gray.size());
    for (std::size_t r = 0; r < next.h; ++r)
      for (std::size_t c = 0; c < next.w; ++c) {
        const std::size_t i = 2 * r * prev.w + 2 * c;
        next.mask[r * next.w + c] = prev.mask[i] && prev.mask[i + 1] && prev.mask[i + prev.w] && prev.mask[i + prev.w + 1];
        // src/imageproc/gray_pyramid.hpp:9-13 (box2_gray)
        const double* r0 = prev.gray.data() + 2 * r * prev.w;
        const double* r1 = prev.gray.data() + (2 * r + 1) * prev.w;
        const std::size_t c0 = 2 * c, c1 = c0 + 1 < prev.w ? c0 + 1 : c0;
        next.gray[r * next.w + c] = .25 * (r0[c0] + r0[c1] + r1[c0] + r1[c1]);
      }
    std::size_t count = 0;
    const bool ok = level_ok(next, &count);
    if (!ok || count < 8 || (m.levels.size() >= 2 && count < 64)) break;
    m.levels.push_back(std::move(next));
  }
  if (opt.levels && m.levels.size() != std::size_t(opt.levels))
    fail(kInvalidArgument, "requested pyramid level is degenerate or too small");
  const double radius = std::hypot(double(m.levels.front().w), double(m.levels.front().h)) * .5;
  m.opt.step = opt.step > 0 ? opt.step : std::max(.01, std::min(.15, 1 / std::max(1., radius)));
  const double intervals = std::ceil(opt.extent / m.opt.step);
  if (!std::isfinite(intervals) || intervals >= kMaxAngles) fail(kLimitExceeded, "angle grid exceeds limit");
  const std::size_t angles = std::size_t(intervals) + 1;
  std::size_t total = 0;
  for (auto& L : m.levels) {
    L.patches.reserve(angles);
    for (std::size_t i = 0; i < angles; ++i) {
      const double angle = opt.start + std::min(opt.extent, i * m.opt.step);
      Patch p = rotate(L, angle, &L == &m.levels.front() ? &first_norm : nullptr);
      if (p.s.empty()) fail(kInvalidArgument, "rotation produces a degenerate template");
      if (p.s.size() > g_max_samples - total) fail(kLimitExceeded, "model raster budget exceeded");
      total += p.s.size();
      L.patches.push_back(std::move(p));
    }
  }
  return m;
}

// src/ncc_matching/model.cpp:120-171 (create), byte/uint16 templates.
template <class T>
Model create(const T* px, std::int64_t w, std::int64_t h, std::int64_t stride_elems,
             const std::uint8_t* mask, const CreateOpts& opt) {
  if (!std::isfinite(opt.start) || !std::isfinite(opt.extent) || !std::isfinite(opt.step) || opt.extent < 0 ||
      opt.extent > kTau || !std::isfinite(opt.start + opt.extent) || opt.step < 0 || opt.levels < 0 || opt.levels > 16)
    fail(kInvalidArgument, "invalid levels or angle range");
  const Domain dom = make_domain(w, h, mask);
  if (dom.area < 4) fail(kInvalidArgument, "template domain requires at least four pixels");
  Level first;
  first.w = std::size_t(dom.cmax - dom.cmin + 1);
  first.h = std::size_t(dom.rmax - dom.rmin + 1);
  if (first.h > kMaxPixels / first.w) fail(kLimitExceeded, "template bounding box exceeds one million pixels");
  first.gray.assign(first.w * first.h, 0.);
  first.mask.assign(first.gray.size(), 0);
  long double sum_row = 0, sum_col = 0;
  std::int64_t isum = 0;
  for (const Run& run : dom.runs) {
    const std::int64_t count = std::int64_t(run.end) - run.begin + 1;
    sum_row += static_cast<long double>(run.row) * count;
    sum_col += (static_cast<long double>(run.begin) + run.end) * count / 2;
    const std::size_t off = std::size_t(run.row - dom.rmin) * first.w;
    for (std::int64_t c = run.begin; c <= run.end; ++c) {
      const T v = px[run.row * stride_elems + c];
      const std::size_t idx = off + std::size_t(c - dom.cmin);
      first.gray[idx] = double(v);
      first.mask[idx] = 1;
      isum += v;
    }
  }
  const std::uint64_t area = std::uint64_t(dom.area);
  const double orow = double(sum_row / area), ocol = double(sum_col / area);
  first.orow = double((sum_row - static_cast<long double>(dom.rmin) * area) / area);
  first.ocol = double((sum_col - static_cast<long double>(dom.cmin) * area) / area);
  const double mean = double(isum) / double(area);
  for (std::size_t i = 0; i < first.gray.size(); ++i)
    if (first.mask[i]) first.gray[i] -= mean;
  return rebuild(std::move(first), opt, orow, ocol);
}

// ----------------------------------------------------------------- find path
// src/ncc_matching/matcher.cpp:28-40 (Gray): one pyramid level; level 0 of a
// byte image may hold only a window of the crop (storage_*).
struct Gray {
  std::size_t w = 0, h = 0;
  std::vector<double> v;
  std::size_t srow = 0, scol = 0, sw = 0, sh = 0;
  double at(std::size_t r, std::size_t c) const { return v[(r - srow) * sw + c - scol]; }
};

// src/ncc_matching/matcher.cpp:87-106 (discrete)
double discrete(const Gray& g, const Patch& p, int row, int col, bool absolute) {
  if (row + p.rmin < 0 || col + p.cmin < 0 || row + p.rmax >= std::int64_t(g.h) || col + p.cmax >= std::int64_t(g.w))
    return kMissing;
  if (row + p.rmin < std::int64_t(g.srow) || col + p.cmin < std::int64_t(g.scol) ||
      row + p.rmax >= std::int64_t(g.srow + g.sh) || col + p.cmax >= std::int64_t(g.scol + g.sw))
    return kMissing;
  const Sample& f = p.s.front();
  const double offset = g.at(std::size_t(row + f.row), std::size_t(col + f.col));
  double sum = 0, sq = 0, dot = 0;
  for (const Sample& x : p.s) {
    const double v = g.at(std::size_t(row + x.row), std::size_t(col + x.col)) - offset;
    sum += v; sq += v * v; dot += x.w * v;
  }
  const double var = sq - sum * sum / double(p.s.size());
  if (!(var > 0)) return kMissing;
  const double r = std::clamp(dot / std::sqrt(var), -1., 1.);
  return absolute ? std::abs(r) : r;
}

// src/ncc_matching/matcher.cpp:107-114 (sample)
double sample(const Gray& g, double row, double col) {
  if (row < 0 || col < 0 || row > g.h - 1 || col > g.w - 1) return kMissing;
  if (row < g.srow || col < g.scol || row > g.srow + g.sh - 1 || col > g.scol + g.sw - 1) return kMissing;
  const std::size_t r = std::size_t(row), c = std::size_t(col);
  const std::size_t r1 = std::min(r + 1, g.h - 1), c1 = std::min(c + 1, g.w - 1);
  const double fr = row - r, fc = col - c;
  return (1 - fr) * ((1 - fc) * g.at(r, c) + fc * g.at(r, c1)) + fr * ((1 - fc) * g.at(r1, c) + fc * g.at(r1, c1));
}

// src/ncc_matching/matcher.cpp:144-156 (continuous, scalar branch)
double continuous(const Gray& g, const Level& L, const Patch& orig, const Pose& pose, bool absolute) {
  const double ca = std::cos(pose.angle), sa = std::sin(pose.angle);
  double sum = 0, sq = 0, dot = 0, offset = 0;
  bool first = true;
  for (const Sample& p : orig.s) {
    const double r = p.row - L.orow, c = p.col - L.ocol;
    double v = sample(g, pose.row + ca * r - sa * c, pose.col + sa * r + ca * c);
    if (!std::isfinite(v)) return kMissing;
    if (first) { offset = v; first = false; }
    v -= offset;
    sum += v; sq += v * v; dot += p.w * v;
  }
  const double var = sq - sum * sum / double(orig.s.size());
  if (!(var > 0)) return kMissing;
  const double s = std::clamp(dot / std::sqrt(var), -1., 1.);
  return absolute ? std::abs(s) : s;
}

// src/ncc_matching/matcher.cpp:170-240 (refinement_step, scalar branch):
// analytic NCC gradient w.r.t. (row, column, angle) and one Gauss-Newton step.
bool gn_step(const Gray& g, const Level& L, const Patch& orig, const Pose& pose, bool absolute, bool rotate,
             double* delta, double* out_score, const double* minimum) {
  const double ca = std::cos(pose.angle), sa = std::sin(pose.angle);
  double sum = 0, energy = 0, dot = 0, gs[3]{}, qg[3]{}, wg[3]{}, gg[3][3]{}, offset = 0;
  bool first = true;
  for (const Sample& p : orig.s) {
    const double dr = p.row - L.orow, dc = p.col - L.ocol;
    const double y = pose.row + ca * dr - sa * dc, x = pose.col + sa * dr + ca * dc;
    if (y < g.srow || x < g.scol || y >= g.srow + g.sh - 1 || x >= g.scol + g.sw - 1) return false;
    const std::size_t r = std::size_t(y), c = std::size_t(x);
    const double fy = y - r, fx = x - c;
    const double a = g.at(r, c), b = g.at(r, c + 1), d = g.at(r + 1, c), e = g.at(r + 1, c + 1);
    double q = (1 - fy) * ((1 - fx) * a + fx * b) + fy * ((1 - fx) * d + fx * e);
    if (first) { offset = q; first = false; }
    q -= offset;
    const double gy = (1 - fx) * (d - a) + fx * (e - b), gx = (1 - fy) * (b - a) + fy * (e - d);
    const double gv[3] = {gy, gx, gy * (-sa * dr - ca * dc) + gx * (ca * dr - sa * dc)};
    sum += q; energy += q * q; dot += q * p.w;
    for (int i = 0; i < (rotate ? 3 : 2); ++i) {
      gs[i] += gv[i]; qg[i] += q * gv[i]; wg[i] += p.w * gv[i];
      for (int j = 0; j <= i; ++j) gg[i][j] += gv[i] * gv[j];
    }
  }
  const double n = double(orig.s.size());
  energy -= sum * sum / n;
  if (!(energy > 0)) return false;
  const double sign = absolute && dot < 0 ? -1 : 1, score = sign * dot / std::sqrt(energy);
  if (out_score) *out_score = std::clamp(score, -1., 1.);
  if (minimum && std::clamp(score, -1., 1.) <= *minimum) return false;
  const int axes = rotate ? 3 : 2;
  double m[3][4]{};
  for (int i = 0; i < axes; ++i) qg[i] -= sum * gs[i] / n;
  for (int i = 0; i < axes; ++i) {
    for (int j = 0; j < axes; ++j)
      m[i][j] = (gg[std::max(i, j)][std::min(i, j)] - gs[i] * gs[j] / n - qg[i] * qg[j] / energy) / energy;
    m[i][axes] = sign * wg[i] / std::sqrt(energy) - score * qg[i] / energy;
  }
  for (int i = 0; i < axes; ++i) {
    int pivot = i;
    for (int j = i + 1; j < axes; ++j)
      if (std::abs(m[j][i]) > std::abs(m[pivot][i])) pivot = j;
    if (std::abs(m[pivot][i]) < 1e-14) return false;
    for (int k = i; k <= axes; ++k) std::swap(m[i][k], m[pivot][k]);
    const double div = m[i][i];
    for (int k = i; k <= axes; ++k) m[i][k] /= div;
    for (int j = 0; j < axes; ++j)
      if (j != i) {
        const double f = m[j][i];
        for (int k = i; k <= axes; ++k) m[j][k] -= f * m[i][k];
      }
  }
  for (int i = 0; i < axes; ++i) delta[i] = m[i][axes];
  if (!rotate) delta[2] = 0;
  return std::isfinite(delta[0]) && std::isfinite(delta[1]) && std::isfinite(delta[2]);
}

// src/ncc_matching/matcher.cpp:241-248 (merge_identical)
void merge_identical(std::vector<Pose>& c) {
  std::sort(c.begin(), c.end(), [](const Pose& a, const Pose& b) {
    if (a.row != b.row) return a.row < b.row;
    if (a.col != b.col) return a.col < b.col;
    return a.angle < b.angle;
  });
  c.erase(std::unique(c.begin(), c.end(), [](const Pose& a, const Pose& b) {
            return a.row == b.row && a.col == b.col && a.angle == b.angle;
          }), c.end());
}

bool domain_contains(const Domain& d, const Pose& m) {
  return d.contains(std::int64_t(std::floor(m.row + .5)), std::int64_t(std::floor(m.col + .5)));
}

// src/ncc_matching/matcher.cpp:252-277 (overlap): area of the intersection of
// the two rotated template rectangles over the template area.
double overlap(const Pose& a, const Pose& b, const Level& L) {
  struct Pt { double x, y; };
  auto corners = [&](const Pose& m) {
    Pt out[4];
    const double ca = std::cos(m.angle), sa = std::sin(m.angle);
    const double left = -L.ocol - .5, right = L.w - L.ocol - .5;
    const double top = -L.orow - .5, bottom = L.h - L.orow - .5;
    const Pt in[4] = {{left, top}, {right, top}, {right, bottom}, {left, bottom}};
    for (int i = 0; i < 4; ++i)
      out[i] = {m.col - a.col + ca * in[i].x + sa * in[i].y, m.row - a.row - sa * in[i].x + ca * in[i].y};
    return std::vector<Pt>(out, out + 4);
  };
  const auto clip = corners(b);
  std::vector<Pt> poly = corners(a), next;
  auto cross = [](Pt p, Pt q, Pt u) { return (q.x - p.x) * (u.y - p.y) - (q.y - p.y) * (u.x - p.x); };
  for (int edge = 0; edge < 4 && !poly.empty(); ++edge) {
    const Pt p = clip[edge], q = clip[(edge + 1) % 4];
    next.clear();
    for (std::size_t i = 0; i < poly.size(); ++i) {
      const Pt u = poly[i], v = poly[(i + 1) % poly.size()];
      const double du = cross(p, q, u), dv = cross(p, q, v);
      if (du >= 0) next.push_back(u);
      if ((du >= 0) != (dv >= 0)) {
        const double t = du / (du - dv);
        next.push_back({u.x + t * (v.x - u.x), u.y + t * (v.y - u.y)});
      }
    }
    poly = next;
  }
  double area = 0;
  for (std::size_t i = 0; i < poly.size(); ++i)
    area += poly[i].x * poly[(i + 1) % poly.size()].y - poly[(i + 1) % poly.size()].x * poly[i].y;
  return std::abs(area) * .5 / (double(L.w) * L.h);
}

// State of one query: src/ncc_matching/matcher.cpp:304-341 (PreparedQuery)
struct Query {
  const Model* model = nullptr;
  FindOpts opt;
  Domain dom;
  std::int64_t crop_row = 0, crop_col = 0;
  std::size_t level_count = 0, finest = 0;
  std::vector<Gray> pyr;
  std::vector<std::vector<const Patch*>> qpatches;
  std::vector<std::vector<Patch>> endpoints;
  std::unique_ptr<Patch> coarse_original;
  std::vector<Pose> cand;
  std::vector<std::vector<Pose>> stages;  // stage dumps (coarse, per tracking step)
  double dc = 0;
};

template <class T>
void build_pyramid(Query& q, const T* px, std::int64_t stride_elems, std::int64_t crop_bottom, std::int64_t crop_right) {
  // src/ncc_matching/matcher.cpp:407-454: level 0 is the crop minus its first
  // pixel; level k+1 is the 2x2 mean of level k (floor dimensions).
  Gray first;
  first.w = std::size_t(crop_right - q.crop_col);
  first.h = std::size_t(crop_bottom - q.crop_row);
  first.sw = first.w; first.sh = first.h;
  const double offset = double(px[q.crop_row * stride_elems + q.crop_col]);
  q.dc = offset;
  first.v.resize(first.w * first.h);
  for (std::size_t r = 0; r < first.h; ++r)
    for (std::size_t c = 0; c < first.w; ++c)
      first.v[r * first.w + c] = double(px[(std::int64_t(r) + q.crop_row) * stride_elems + std::int64_t(c) + q.crop_col]) - offset;
  q.pyr.push_back(std::move(first));
  for (std::size_t l = 1; l < q.level_count; ++l) {
    const Gray& prev = q.pyr.back();
    Gray next;
    next.w = std::max<std::size_t>(1, prev.w / 2);
    next.h = std::max<std::size_t>(1, prev.h / 2);
    next.sw = next.w; next.sh = next.h;
    next.v.resize(next.w * next.h);
    for (std::size_t r = 0; r < next.h; ++r)
      for (std::size_t c = 0; c < next.w; ++c) {
        const std::size_t r0 = 2 * r, r1 = std::min(r0 + 1, prev.h - 1), c0 = 2 * c, c1 = std::min(c0 + 1, prev.w - 1);
        next.v[r * next.w + c] = .25 * (prev.at(r0, c0) + prev.at(r0, c1) + prev.at(r1, c0) + prev.at(r1, c1));
      }
    q.pyr.push_back(std::move(next));
  }
}

// src/ncc_matching/matcher.cpp:343-851 (prepare), scalar branch.
template <class T>
std::unique_ptr<Query> prepare(const T* px, std::int64_t W, std::int64_t H, std::int64_t stride_elems,
                               const std::uint8_t* dmask, const Model& model, const FindOpts& requested,
                               bool is_byte, int stop_stage, int* pyramid_only = nullptr) {
  auto q = std::make_unique<Query>();
  q->model = &model;
  FindOpts opt = requested;
  q->opt = opt;
  if (model.levels.empty()) fail(kInvalidState, "model is empty");
  if (opt.highest < 0 || opt.lowest < 1) fail(kInvalidArgument, "invalid pyramid levels");
  const std::size_t level_count = opt.highest ? std::min(model.levels.size(), std::size_t(opt.highest)) : model.levels.size();
  opt.lowest = int(std::min(std::size_t(opt.lowest), level_count));
  const std::size_t finest = std::size_t(opt.lowest - 1);
  q->level_count = level_count;
  q->finest = finest;
  if (finest) {
    Patch o = rotate(model.levels[finest], 0, nullptr);
    for (const Sample& s : o.s) {
      o.relr.push_back(s.row - model.levels[finest].orow);
      o.relc.push_back(s.col - model.levels[finest].ocol);
    }
    q->coarse_original = std::make_unique<Patch>(std::move(o));
  }
  if (!std::isfinite(opt.start) || !std::isfinite(opt.extent) || opt.extent < 0 || !std::isfinite(opt.min_score) ||
      opt.min_score < 0 || opt.min_score > 1 || !std::isfinite(opt.max_overlap) || opt.max_overlap < 0 ||
      opt.max_overlap > 1 || !opt.max_candidates)
    fail(kInvalidArgument, "invalid query range, score, overlap or candidate budget");
  const double angle_end = opt.start + opt.extent;  // unclipped end, as in the reference
  if (!std::isfinite(angle_end)) fail(kInvalidArgument, "query angle range must be finite");
  const double cs = std::max(opt.start, model.opt.start);
  const double ce = std::min(angle_end, model.opt.start + model.opt.extent);
  if (cs > ce + 1e-12) return q;
  opt.start = cs;
  opt.extent = std::max(0., ce - cs);
  q->opt = opt;
  if (!W || !H || W > std::numeric_limits<int>::max() || H > std::numeric_limits<int>::max() || H > g_max_image_pixels / (long long)W)
    fail(kLimitExceeded, "search image exceeds pixel budget");
  q->dom = make_domain(W, H, dmask);
  const Domain& dom = q->dom;
  if (dom.area == 0) return q;
  const Level& base = model.levels.front();
  const double radius = std::hypot(std::max(base.orow, double(base.h - 1) - base.orow),
                                   std::max(base.ocol, double(base.w - 1) - base.ocol));
  const std::int64_t lattice = std::int64_t(std::size_t{1} << (level_count - 1));
  const std::int64_t halo = std::int64_t(std::ceil(radius)) + 4 * lattice;
  const std::int64_t crop_row = std::max<std::int64_t>(0, dom.rmin - halo) / lattice * lattice;
  const std::int64_t crop_col = std::max<std::int64_t>(0, dom.cmin - halo) / lattice * lattice;
  const std::int64_t crop_bottom = std::min<std::int64_t>(H, ((dom.rmax + halo) / lattice + 1) * lattice);
  const std::int64_t crop_right = std::min<std::int64_t>(W, ((dom.cmax + halo) / lattice + 1) * lattice);
  q->crop_row = crop_row;
  q->crop_col = crop_col;
  build_pyramid(*q, px, stride_elems, crop_bottom, crop_right);
  if (pyramid_only) { *pyramid_only = 1; return q; }
  auto& pyr = q->pyr;
  // query patches per level: src/ncc_matching/matcher.cpp:463-475
  q->qpatches.resize(level_count);
  q->endpoints.resize(level_count);
  for (std::size_t li = 0; li < level_count; ++li) {
    const Level& L = model.levels[li];
    auto& list = q->qpatches[li];
    auto& ends = q->endpoints[li];
    ends.reserve(2);
    for (const Patch& p : L.patches)
      if (p.angle >= opt.start - 1e-12 && p.angle <= angle_end + 1e-12) list.push_back(&p);
    for (const double a : {opt.start, angle_end}) {
      bool found = false;
      for (const Patch* p : list)
        if (std::abs(p->angle - a) < 1e-12) found = true;
      if (found) continue;
      ends.push_back(rotate(L, a, nullptr));
      if (!ends.back().s.empty()) list.push_back(&ends.back());
    }
  }
  const std::size_t top = level_count - 1;
  const Gray& coarse = pyr[top];
  const double coarse_radius = .5 * std::hypot(double(model.levels[top].w), double(model.levels[top].h));
  const std::size_t stride = std::max<std::size_t>(1, std::size_t(std::min(double(q->qpatches[top].size()),
      std::ceil(.5 / std::max(1e-20, coarse_radius * model.opt.step)))));
  auto& coarse_angles = q->qpatches[top];
  std::sort(coarse_angles.begin(), coarse_angles.end(), [](const Patch* a, const Patch* b) { return a->angle < b->angle; });
  {
    std::size_t kept = 0;
    for (std::size_t i = 0; i < coarse_angles.size(); ++i)
      if (i % stride == 0 || i + 1 == coarse_angles.size()) coarse_angles[kept++] = coarse_angles[i];
    coarse_angles.resize(kept);
  }
  // support integral: src/ncc_matching/matcher.cpp:496-503
  std::vector<std::uint32_t> support((coarse.w + 1) * (coarse.h + 1), 0);
  for (std::size_t r = 0; r < coarse.h; ++r) {
    std::uint32_t row_sum = 0;
    for (std::size_t c = 0; c < coarse.w; ++c) {
      row_sum += coarse.at(r, c) != 0;
      support[(r + 1) * (coarse.w + 1) + c + 1] = support[r * (coarse.w + 1) + c + 1] + row_sum;
    }
  }
  auto has_support = [&](const Patch& p, int r, int c) {
    const std::size_t pitch = coarse.w + 1;
    const std::size_t r0 = std::size_t(r + p.rmin), r1 = std::size_t(r + p.rmax + 1);
    const std::size_t c0 = std::size_t(c + p.cmin), c1 = std::size_t(c + p.cmax + 1);
    return support[r1 * pitch + c1] - support[r1 * pitch + c0] - support[r0 * pitch + c1] + support[r0 * pitch + c0] != 0;
  };
  const double scale = std::ldexp(1., int(top)), phase = (scale - 1) * .5;
  const bool sparse = !dom.full && double(dom.area) < .7 * double(dom.rmax - dom.rmin + 1) * double(dom.cmax - dom.cmin + 1);
  // src/ncc_matching/matcher.cpp:507-534 (may_contain), uncached branch
  auto may_contain = [&](const Pose& pose, double spacing) {
    if (spacing == 1) return domain_contains(dom, pose);
    const double margin = 2 * spacing;
    if (pose.row < dom.rmin - margin || pose.row > dom.rmax + margin || pose.col < dom.cmin - margin ||
        pose.col > dom.cmax + margin)
      return false;
    if (!sparse) return true;
    auto it = std::lower_bound(dom.runs.begin(), dom.runs.end(), pose.row - margin,
                               [](const Run& run, double row) { return run.row < row; });
    for (; it != dom.runs.end() && it->row <= pose.row + margin; ++it)
      if (it->begin <= pose.col + margin && it->end >= pose.col - margin) return true;
    return false;
  };
  auto& cand = q->cand;
  std::vector<double> scores(coarse.w * coarse.h, kMissing);
  const bool ignore = model.opt.ignore;
  // coarse scan + NMS: src/ncc_matching/matcher.cpp:542-594
  for (const Patch* pp : coarse_angles) {
    const Patch& p = *pp;
    std::fill(scores.begin(), scores.end(), kMissing);
    const double margin = scale == 1 ? .5 : 2 * scale;
    const int r_begin = std::max({0, -p.rmin, int(std::ceil((dom.rmin - margin - crop_row - phase) / scale - p.orow))});
    const int r_end = std::min(int(coarse.h) - p.rmax, int(std::floor((dom.rmax + margin - crop_row - phase) / scale - p.orow)) + 1);
    const int c_begin = std::max({0, -p.cmin, int(std::ceil((dom.cmin - margin - crop_col - phase) / scale - p.ocol))});
    const int c_end = std::min(int(coarse.w) - p.cmax, int(std::floor((dom.cmax + margin - crop_col - phase) / scale - p.ocol)) + 1);
    for (int r = r_begin; r < r_end; ++r)
      for (int c = c_begin; c < c_end; ++c) {
        const Pose pose{crop_row + scale * (r + p.orow) + phase, crop_col + scale * (c + p.ocol) + phase, p.angle, 0};
        if (may_contain(pose, scale) && has_support(p, r, c)) scores[std::size_t(r) * coarse.w + c] = discrete(coarse, p, r, c, ignore);
      }
    for (int r = r_begin; r < r_end; ++r)
      for (int c = c_begin; c < c_end; ++c) {
        const double v = scores[std::size_t(r) * coarse.w + c];
        if (v < opt.min_score * .4 || !std::isfinite(v)) continue;
        bool maximum = true;
        for (int dr = -1; dr <= 1; ++dr)
          for (int dc = -1; dc <= 1; ++dc) {
            const std::int64_t rr = std::int64_t(r) + dr, cc = std::int64_t(c) + dc;
            if (rr < 0 || cc < 0 || rr >= std::int64_t(coarse.h) || cc >= std::int64_t(coarse.w) || (!dr && !dc)) continue;
            const double o = scores[std::size_t(rr) * coarse.w + std::size_t(cc)];
            if (o > v || (o == v && (dr < 0 || (!dr && dc < 0)))) maximum = false;
          }
        if (!maximum) continue;
        if (cand.size() == opt.max_candidates) fail(kLimitExceeded, "coarse candidate budget exceeded");
        cand.push_back({crop_row + scale * (r + p.orow) + phase, crop_col + scale * (c + p.ocol) + phase, p.angle, v});
      }
  }
  q->stages.push_back(cand);
  if (stop_stage == 0) return q;
  // level-0 window of a byte image: src/ncc_matching/matcher.cpp:612-629
  if (!finest && is_byte && !cand.empty()) {
    Gray& fine = pyr.front();
    double rmin = double(fine.h), cmin = double(fine.w), rmax = 0, cmax = 0;
    for (const Pose& p : cand) {
      rmin = std::min(rmin, p.row - crop_row); rmax = std::max(rmax, p.row - crop_row);
      cmin = std::min(cmin, p.col - crop_col); cmax = std::max(cmax, p.col - crop_col);
    }
    const double margin = radius + 4 * scale + 8;
    const std::size_t srow = std::size_t(std::max(0., std::floor(rmin - margin)));
    const std::size_t scol = std::size_t(std::max(0., std::floor(cmin - margin)));
    const std::size_t sh = std::size_t(std::min(double(fine.h), std::ceil(rmax + margin) + 1)) - srow;
    const std::size_t sw = std::size_t(std::min(double(fine.w), std::ceil(cmax + margin) + 1)) - scol;
    std::vector<double> win(sw * sh);
    for (std::size_t r = 0; r < sh; ++r)
      for (std::size_t c = 0; c < sw; ++c) win[r * sw + c] = fine.v[(r + srow) * fine.w + c + scol];
    fine.v.swap(win);
    fine.srow = srow; fine.scol = scol; fine.sw = sw; fine.sh = sh;
  }
  // coarse-to-fine tracking: src/ncc_matching/matcher.cpp:630-761
  int stage = 0;
  for (std::size_t l = top; l > finest; --l) {
    if (l == 1 && opt.subpixel) {
      for (Pose& p : cand)
        if (!domain_contains(dom, p)) {
          double best = std::numeric_limits<double>::infinity();
          Pose nearest = p;
          auto it = std::lower_bound(dom.runs.begin(), dom.runs.end(), p.row - 4,
                                     [](const Run& run, double row) { return run.row < row; });
          for (; it != dom.runs.end() && it->row <= p.row + 4; ++it) {
            const double c = std::clamp(std::round(p.col), double(it->begin), double(it->end));
            if (std::abs(c - p.col) > 4) continue;
            const double dist = std::hypot(double(it->row) - p.row, c - p.col);
            if (dist < best) { best = dist; nearest.row = double(it->row); nearest.col = c; }
          }
          if (std::isfinite(best)) p = nearest;
          else p.score = kMissing;
        }
      merge_identical(cand);
      q->stages.push_back(cand);
      ++stage;
      if (stop_stage == stage) return q;
      break;
    }
    const Level& L = model.levels[l - 1];
    const Gray& target = pyr[l - 1];
    const double step = std::ldexp(1., int(l - 1)), offset = (step - 1) * .5;
    (void)L;
    for (Pose& cd : cand) {
      Pose best = cd;
      best.score = kMissing;
      for (const Patch* pp : q->qpatches[l - 1]) {
        const Patch& p = *pp;
        if (std::abs(p.angle - cd.angle) > model.opt.step * (l == top ? double(stride) : 1.) * 1.01) continue;
        const int row = int(std::round((cd.row - crop_row - offset) / step - p.orow));
        const int col = int(std::round((cd.col - crop_col - offset) / step - p.ocol));
        for (int dr = -2; dr <= 2; ++dr)
          for (int dc = -2; dc <= 2; ++dc) {
            Pose pose{crop_row + step * (row + dr + p.orow) + offset, crop_col + step * (col + dc + p.ocol) + offset, p.angle, 0};
            if (!may_contain(pose, step)) continue;
            pose.score = discrete(target, p, row + dr, col + dc, ignore);
            if (pose.score > best.score) best = pose;
          }
      }
      cd = best;
    }
    merge_identical(cand);
    cand.erase(std::remove_if(cand.begin(), cand.end(),
                              [&](const Pose& p) { return !std::isfinite(p.score) || p.score < opt.min_score * .4; }),
               cand.end());
    q->stages.push_back(cand);
    ++stage;
    if (stop_stage == stage) return q;
  }
  // full-resolution score and sort: src/ncc_matching/matcher.cpp:813-827
  const Patch& original = finest ? *q->coarse_original : model.original;
  {
    const double sc = std::ldexp(1., int(finest)), ph = (sc - 1) * .5;
    for (Pose& c : cand)
      if (std::isfinite(c.score)) {
        Pose local = c;
        local.row = (local.row - crop_row - ph) / sc;
        local.col = (local.col - crop_col - ph) / sc;
        c.score = continuous(pyr[finest], model.levels[finest], original, local, ignore);
      }
  }
  std::sort(cand.begin(), cand.end(), [](const Pose& a, const Pose& b) {
    if (a.score != b.score) return a.score > b.score;
    if (a.row != b.row) return a.row < b.row;
    if (a.col != b.col) return a.col < b.col;
    return a.angle < b.angle;
  });
  return q;
}

// src/ncc_matching/matcher.cpp:853-877 (refine_coarse_candidate)
bool refine_coarse(Query& q, Pose& cand) {
  const Model& model = *q.model;
  const FindOpts& opt = q.opt;
  const Level& L = model.levels[q.finest];
  const Patch& orig = *q.coarse_original;
  const double scale = std::ldexp(1., int(q.finest)), phase = (scale - 1) * .5;
  const Gray& fine = q.pyr[q.finest];
  auto local = [&](Pose p) {
    p.row = (p.row - q.crop_row - phase) / scale;
    p.col = (p.col - q.crop_col - phase) / scale;
    return p;
  };
  auto score = [&](const Pose& p) { return continuous(fine, L, orig, local(p), model.opt.ignore); };
  if (opt.subpixel)
    for (int it = 0; it < 6; ++it) {
      double delta[3]{};
      if (!gn_step(fine, L, orig, local(cand), model.opt.ignore, opt.extent > 0, delta, nullptr, nullptr)) break;
      const double factor = std::min({1., .75 / std::max(1e-20, std::abs(delta[0])), .75 / std::max(1e-20, std::abs(delta[1])),
                                      opt.extent > 0 ? model.opt.step / std::max(1e-20, std::abs(delta[2])) : 1.});
      bool accepted = false;
      for (int bt = 0; bt < 4; ++bt) {
        const double st = std::ldexp(factor, -bt);
        Pose next = cand;
        next.row += scale * st * delta[0];
        next.col += scale * st * delta[1];
        next.angle = std::clamp(next.angle + st * delta[2], opt.start, opt.start + opt.extent);
        if (!domain_contains(q.dom, next)) continue;
        next.score = score(next);
        if (next.score > cand.score) { cand = next; accepted = true; break; }
      }
      if (!accepted) break;
    }
  return cand.score >= opt.min_score && domain_contains(q.dom, cand);
}

// src/ncc_matching/matcher.cpp:878-1061 (refine_candidate), single-model
// query: no memo, no background guard, no derivative cache.
bool refine(Query& q, Pose& cand) {
  if (q.finest) return refine_coarse(q, cand);
  const Model& model = *q.model;
  const FindOpts& opt = q.opt;
  const Domain& dom = q.dom;
  const double crop_row = double(q.crop_row), crop_col = double(q.crop_col);
  const std::size_t top = q.level_count - 1;
  const double angle_end = opt.start + opt.extent;
  const Patch& orig = model.original;
  const Gray& fine = q.pyr.front();
  const Level& L0 = model.levels.front();
  const bool ignore = model.opt.ignore;
  const bool rotate = opt.extent > 0;
  auto full_score = [&](Pose p) {
    p.row -= crop_row;
    p.col -= crop_col;
    return continuous(fine, L0, orig, p, ignore);
  };
  auto fit = [&](Pose& c) {
    bool cached = false;
    double next_delta[3]{};
    if (!opt.subpixel) return;
    for (int it = 0; it < 6; ++it) {
      Pose local = c;
      local.row -= crop_row;
      local.col -= crop_col;
      double delta[3]{};
      if (cached) std::copy(next_delta, next_delta + 3, delta);
      else if (!gn_step(fine, L0, orig, local, ignore, rotate, delta, nullptr, nullptr)) break;
      cached = false;
      const double factor = std::min({1., .75 / std::max(1e-20, std::abs(delta[0])), .75 / std::max(1e-20, std::abs(delta[1])),
                                      rotate ? model.opt.step / std::max(1e-20, std::abs(delta[2])) : 1.});
      bool accepted = false;
      for (int bt = 0; bt < 4; ++bt) {
        const double st = std::ldexp(factor, -bt);
        Pose imp = c;
        imp.row += st * delta[0];
        imp.col += st * delta[1];
        imp.angle = std::clamp(imp.angle + st * delta[2], opt.start, angle_end);
        if (!domain_contains(dom, imp)) continue;
        bool next_valid = false;
        if (bt == 0 && it + 1 < 6) {
          Pose nl = imp;
          nl.row -= crop_row;
          nl.col -= crop_col;
          imp.score = kMissing;
          next_valid = gn_step(fine, L0, orig, nl, ignore, rotate, next_delta, &imp.score, &c.score);
          if (!std::isfinite(imp.score)) imp.score = full_score(imp);
        } else {
          imp.score = full_score(imp);
        }
        if (imp.score > c.score) { c = imp; accepted = true; cached = next_valid; break; }
      }
      if (!accepted || (std::hypot(delta[0], delta[1]) < 1e-4 && std::abs(delta[2]) < 1e-5)) break;
    }
  };
  const Pose seed = cand;
  fit(cand);
  if (opt.subpixel && top > 0 && cand.score < opt.min_score) {
    // discrete recovery around the seed at full resolution
    Pose best = cand;
    for (const Patch* p : q.qpatches.front()) {
      if (std::abs(p->angle - seed.angle) > model.opt.step * 1.01) continue;
      const int r = int(std::round(seed.row - crop_row - p->orow)), c = int(std::round(seed.col - crop_col - p->ocol));
      for (int dr = -2; dr <= 2; ++dr)
        for (int dc = -2; dc <= 2; ++dc) {
          Pose pp{double(q.crop_row + r + dr) + p->orow, double(q.crop_col + c + dc) + p->ocol, p->angle, 0};
          if (!domain_contains(dom, pp)) continue;
          pp.score = discrete(fine, *p, r + dr, c + dc, ignore);
          if (pp.score > best.score) best = pp;
        }
    }
    if (best.row != cand.row || best.col != cand.col || best.angle != cand.angle) {
      best.score = full_score(best);
      fit(best);
      if (best.score > cand.score) cand = best;
    }
  }
  return cand.score >= opt.min_score && domain_contains(dom, cand);
}

// src/ncc_matching/matcher.cpp:1063-1076 (find)
std::vector<Pose> select(Query& q) {
  std::vector<Pose> result;
  const Level& L0 = q.model->levels.front();
  for (Pose c : q.cand) {
    if (!std::isfinite(c.score)) continue;
    bool dup = false;
    for (const Pose& p : result)
      if (overlap(c, p, L0) > q.opt.max_overlap + 1e-12) { dup = true; break; }
    if (dup || !refine(q, c)) continue;
    dup = false;
    for (const Pose& p : result)
      if (overlap(c, p, L0) > q.opt.max_overlap + 1e-12) { dup = true; break; }
    if (dup) continue;
    result.push_back(c);
    if (q.opt.num_matches && result.size() == q.opt.num_matches) break;
  }
  std::sort(result.begin(), result.end(), [](const Pose& a, const Pose& b) {
    if (a.score != b.score) return a.score > b.score;
    if (a.row != b.row) return a.row < b.row;
    if (a.col != b.col) return a.col < b.col;
    return a.angle < b.angle;
  });
  return result;
}

void set_err(char* err, int len, const std::string& s) {
  if (!err || len <= 0) return;
  std::strncpy(err, s.c_str(), std::size_t(len - 1));
  err[len - 1] = 0;
}

template <class Fn> int guarded(char* err, int len, Fn&& fn) {
  try {
    fn();
    return 0;
  } catch (const Failure& f) {
    set_err(err, len, f.message);
    return f.status;
  } catch (const std::bad_alloc&) {
    set_err(err, len, "out of memory");
    return kOutOfMemory;
  } catch (const std::exception& e) {
    set_err(err, len, e.what());
    return kInternal;
  }
}

FindOpts find_opts(double start, double extent, double min_score, std::int64_t num_matches, double max_overlap,
                   int subpixel, int highest, int lowest) {
  FindOpts o;
  o.start = start; o.extent = extent; o.min_score = min_score;
  o.num_matches = std::size_t(num_matches); o.max_overlap = max_overlap;
  o.subpixel = subpixel != 0; o.highest = highest; o.lowest = lowest < 1 ? 1 : lowest;
  return o;
}

std::vector<Pose> run_find(const Model& m, const void* img, int type, std::int64_t w, std::int64_t h, std::int64_t stride,
                           const std::uint8_t* dom, const FindOpts& o, int stage) {
  std::unique_ptr<Query> q;
  if (type == 1)
    q = prepare(static_cast<const std::uint16_t*>(img), w, h, stride / 2, dom, m, o, false, stage);
  else
    q = prepare(static_cast<const std::uint8_t*>(img), w, h, stride, dom, m, o, true, stage);
  if (stage >= 0 && stage < 100) {
    if (std::size_t(stage) < q->stages.size()) return q->stages[std::size_t(stage)];
    return {};
  }
  if (stage == 100) return q->cand;
  return select(*q);
}

}  // namespace
}  // namespace orc

using namespace orc;

extern "C" {

void orc_set_budgets(int64_t samples, int64_t pixels, int64_t candidates) {
  orc::g_max_samples = samples > 0 ? std::size_t(samples) : 16000000;
  orc::g_max_image_pixels = pixels > 0 ? pixels : 32000000;
  orc::g_max_candidates = candidates > 0 ? std::size_t(candidates) : 10000;
}

int orc_create(const void* pixels, int type, int64_t width, int64_t height, int64_t stride, const uint8_t* mask,
               int levels, double angle_start, double angle_extent, double angle_step, int ignore_polarity,
               void** model, char* err, int errlen) {
  *model = nullptr;
  return guarded(err, errlen, [&] {
    CreateOpts o;
    o.levels = levels; o.start = angle_start; o.extent = angle_extent; o.step = angle_step;
    o.ignore = ignore_polarity != 0;
    Model m = type == 1 ? create(static_cast<const std::uint16_t*>(pixels), width, height, stride / 2, mask, o)
                        : create(static_cast<const std::uint8_t*>(pixels), width, height, stride, mask, o);
    *model = new Model(std::move(m));
  });
}

void orc_free(void* model) { delete static_cast<Model*>(model); }

void orc_model_info(void* model, double* info) {
  const Model& m = *static_cast<Model*>(model);
  info[0] = double(m.levels.size());
  info[1] = m.opt.step;
  info[2] = m.orow;
  info[3] = m.ocol;
  info[4] = double(m.levels.front().patches.size());
  info[5] = double(m.original.s.size());
}

void orc_level(void* model, int level, int64_t* dims, double* origin) {
  const Level& L = static_cast<Model*>(model)->levels[std::size_t(level)];
  dims[0] = int64_t(L.w);
  dims[1] = int64_t(L.h);
  origin[0] = L.orow;
  origin[1] = L.ocol;
}

int64_t orc_patch(void* model, int level, int index, int32_t* rows, int32_t* cols, double* weights, int64_t capacity,
                  double* meta) {
  const Model& m = *static_cast<Model*>(model);
  const Patch& p = level < 0 ? m.original : m.levels[std::size_t(level)].patches[std::size_t(index)];
  meta[0] = p.angle;
  meta[1] = p.orow;
  meta[2] = p.ocol;
  meta[3] = p.wsum;
  const int64_t n = int64_t(p.s.size());
  if (rows && n <= capacity)
    for (int64_t i = 0; i < n; ++i) {
      rows[i] = p.s[std::size_t(i)].row;
      cols[i] = p.s[std::size_t(i)].col;
      weights[i] = p.s[std::size_t(i)].w;
    }
  return n;
}

int orc_find(void* model, const void* image, int type, int64_t width, int64_t height, int64_t stride,
             const uint8_t* domain, double angle_start, double angle_extent, double min_score, int64_t num_matches,
             double max_overlap, int subpixel, int highest, int lowest, int stage, double* out, int64_t capacity,
             int64_t* count, char* err, int errlen) {
  *count = 0;
  return guarded(err, errlen, [&] {
    const auto o = find_opts(angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel, highest, lowest);
    const auto res = run_find(*static_cast<Model*>(model), image, type, width, height, stride, domain, o, stage);
    *count = int64_t(res.size());
    for (std::size_t i = 0; i < res.size() && int64_t(i) < capacity; ++i) {
      out[4 * i + 0] = res[i].row;
      out[4 * i + 1] = res[i].col;
      out[4 * i + 2] = res[i].angle;
      out[4 * i + 3] = res[i].score;
    }
  });
}

int orc_pyramid(void* model, const void* image, int type, int64_t width, int64_t height, int64_t stride, int highest,
                int level, double* out, int64_t capacity, double* geom, char* err, int errlen) {
  return guarded(err, errlen, [&] {
    FindOpts o;
    o.highest = highest;
    o.start = -1e300; o.extent = 0;  // range irrelevant for the pyramid
    const Model& m = *static_cast<Model*>(model);
    o.start = m.opt.start;
    o.extent = m.opt.extent;
    int only = 0;
    std::unique_ptr<Query> q;
    if (type == 1)
      q = prepare(static_cast<const std::uint16_t*>(image), width, height, stride / 2, nullptr, m, o, false, 0, &only);
    else
      q = prepare(static_cast<const std::uint8_t*>(image), width, height, stride, nullptr, m, o, true, 0, &only);
    if (level < 0 || std::size_t(level) >= q->pyr.size()) fail(kInvalidArgument, "level out of range");
    const Gray& g = q->pyr[std::size_t(level)];
    geom[0] = double(g.w); geom[1] = double(g.h);
    geom[2] = double(q->crop_row); geom[3] = double(q->crop_col);
    geom[4] = q->dc; geom[5] = double(q->level_count);
    if (int64_t(g.v.size()) <= capacity) std::copy(g.v.begin(), g.v.end(), out);
  });
}

int64_t orc_find_many(void* model, const void* const* images, int type, int64_t width, int64_t height, int64_t stride,
                      int n, int threads, double angle_start, double angle_extent, double min_score, int64_t num_matches,
                      double max_overlap, int subpixel, int highest, int lowest) {
  const auto o = find_opts(angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel, highest, lowest);
  std::atomic<int> next{0};
  std::atomic<int64_t> total{0};
  auto worker = [&] {
    for (int i = next++; i < n; i = next++) {
      try {
        total += int64_t(run_find(*static_cast<Model*>(model), images[i], type, width, height, stride, nullptr, o, -1).size());
      } catch (...) {
        total += 0;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < std::max(1, threads); ++t) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  return total.load();
}

}  // extern "C"
