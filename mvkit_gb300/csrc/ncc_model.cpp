// CreateNccModel on the host in FP64.  The weights must equal the reference's
// bit for bit (they feed every score), so each expression keeps the
// reference's operation order; this file is compiled with -ffp-contract=off.
//   create   src/ncc_matching/model.cpp:120-171
//   rebuild  src/ncc_matching/model.cpp:173-242
//   rotate   src/ncc_matching/model.cpp:66-98
//   normalize src/ncc_matching/model.cpp:38-65
#include "ncc_model.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace mvg {
Budgets& thread_budgets() {
  thread_local Budgets b;
  return b;
}

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr size_t kTemplatePixels = kModelTemplatePixels, kAngles = kModelAngles;

// Pending raster before normalisation: FP64 gray values at integer offsets.
struct RawSample { int32_t row, col; double value; };

struct Moments { double mean, energy; };

// Zero-mean, unit-energy weights; bounds, runs.  Returns false when the raster
// has fewer than four samples or no finite positive energy.
bool finish_raster(std::vector<RawSample>& s, Raster& out, const Moments* known) {
  if (s.size() < 4) return false;
  double mean = 0;
  if (known) mean = known->mean;
  else
    for (size_t i = 0; i < s.size(); ++i) mean += (s[i].value - mean) / double(i + 1);
  double energy = 0;
  if (known) {
    energy = known->energy;
    for (auto& x : s) x.value -= mean;
  } else {
    for (auto& x : s) {
      x.value -= mean;
      energy += x.value * x.value;
    }
  }
  if (!(energy > 0) || !std::isfinite(energy)) return false;
  const double k = 1 / std::sqrt(energy);
  out.rows.reserve(s.size());
  out.cols.reserve(s.size());
  out.w.reserve(s.size());
  out.rmin = out.rmax = s.front().row;
  out.cmin = out.cmax = s.front().col;
  for (auto& x : s) {
    x.value *= k;
    out.rows.push_back(x.row);
    out.cols.push_back(x.col);
    out.w.push_back(x.value);
    out.wsum += x.value;
    out.rmin = std::min(out.rmin, x.row);
    out.rmax = std::max(out.rmax, x.row);
    out.cmin = std::min(out.cmin, x.col);
    out.cmax = std::max(out.cmax, x.col);
    if (!out.run_row.empty() && out.run_row.back() == x.row && out.run_end.back() + 1 == x.col) {
      out.run_end.back() = x.col;
    } else {
      out.run_row.push_back(x.row);
      out.run_begin.push_back(x.col);
      out.run_end.push_back(x.col);
    }
  }
  return true;
}

}  // namespace

RasterBox raster_box(const ModelLevel& L, double angle) {
  RasterBox b;
  b.angle = angle;
  b.unrotated = std::abs(std::remainder(angle, kTwoPi)) < 1e-12;
  if (b.unrotated) {
    b.r0 = 0;
    b.r1 = int(L.height) - 1;
    b.c0 = 0;
    b.c1 = int(L.width) - 1;
    return b;
  }
  const double ca = std::cos(angle), sa = std::sin(angle);
  b.ca = ca;
  b.sa = sa;
  // Bounding box of the rotated level corners about the origin (origin
  // included, so the box always contains 0).
  double lo_r = 0, hi_r = 0, lo_c = 0, hi_c = 0;
  const double corner_r[2] = {0., double(L.height - 1)}, corner_c[2] = {0., double(L.width - 1)};
  for (double r : corner_r)
    for (double c : corner_c) {
      const double dr = r - L.orow, dc = c - L.ocol;
      const double rr = ca * dr - sa * dc, cc = sa * dr + ca * dc;
      lo_r = std::min(lo_r, rr);
      hi_r = std::max(hi_r, rr);
      lo_c = std::min(lo_c, cc);
      hi_c = std::max(hi_c, cc);
    }
  const double span_r = std::ceil(hi_r) - std::floor(lo_r) + 1, span_c = std::ceil(hi_c) - std::floor(lo_c) + 1;
  b.too_large = span_r > 4 * kTemplatePixels / span_c;
  b.r0 = int(std::floor(lo_r));
  b.r1 = int(std::ceil(hi_r));
  b.c0 = int(std::floor(lo_c));
  b.c1 = int(std::ceil(hi_c));
  return b;
}

namespace {

Raster rotate_impl(const ModelLevel& L, double angle, const Moments* known) {
  Raster out;
  out.angle = angle;
  std::vector<RawSample> s;
  s.reserve(size_t(std::count(L.mask.begin(), L.mask.end(), uint8_t{1})));
  const RasterBox box = raster_box(L, angle);
  if (box.unrotated) {
    // Unrotated raster keeps absolute level coordinates.
    out.orow = L.orow;
    out.ocol = L.ocol;
    for (size_t r = 0; r < L.height; ++r)
      for (size_t c = 0; c < L.width; ++c)
        if (L.mask[r * L.width + c]) s.push_back({int32_t(r), int32_t(c), L.gray[r * L.width + c]});
    if (!finish_raster(s, out, known)) return Raster{};
    return out;
  }
  const double ca = box.ca, sa = box.sa;
  if (box.too_large) raise(kLimitExceeded, "rotated bounding box exceeds budget");
  for (int r = box.r0; r <= box.r1; ++r)
    for (int c = box.c0; c <= box.c1; ++c) {
      // source position of the rotated offset (r, c) in the level raster
      const double y = ca * r + sa * c + L.orow, x = -sa * r + ca * c + L.ocol;
      if (y < 0 || x < 0 || y > L.height - 1 || x > L.width - 1) continue;
      const size_t y0 = size_t(y), x0 = size_t(x);
      const size_t y1 = std::min(y0 + 1, L.height - 1), x1 = std::min(x0 + 1, L.width - 1);
      const size_t i00 = y0 * L.width + x0, i01 = y0 * L.width + x1, i10 = y1 * L.width + x0, i11 = y1 * L.width + x1;
      if (!L.mask[i00] || !L.mask[i01] || !L.mask[i10] || !L.mask[i11]) continue;
      const double fy = y - y0, fx = x - x0;
      const double v = (1 - fy) * ((1 - fx) * L.gray[i00] + fx * L.gray[i01]) +
                       fy * ((1 - fx) * L.gray[i10] + fx * L.gray[i11]);
      s.push_back({r, c, v});
    }
  if (!finish_raster(s, out, nullptr)) return Raster{};
  return out;
}

// Degeneracy test of a candidate pyramid level (model.cpp:20-36).
bool level_usable(const ModelLevel& L, size_t* count) {
  size_t n = 0;
  double mean = 0;
  const size_t px = L.width * L.height;
  for (size_t i = 0; i < px; ++i)
    if (L.mask[i]) mean += (L.gray[i] - mean) / double(++n);
  *count = n;
  if (n < 4) return false;
  double energy = 0;
  for (size_t i = 0; i < px; ++i)
    if (L.mask[i]) {
      const double v = L.gray[i] - mean;
      energy += v * v;
    }
  return energy > 0 && std::isfinite(energy);
}

}  // namespace

// rebuild() of src/ncc_matching/model.cpp:173-242: the original raster, the
// pyramid, the resolved angle step and every level's rotated rasters from the
// mean-free level-0 raster.
HostModel rebuild_model(ModelLevel first, const CreateParams& params, double origin_row, double origin_col,
                        bool rasters) {
  HostModel m;
  m.params = params;
  m.origin_row = origin_row;
  m.origin_col = origin_col;
  m.sample_count = size_t(std::count(first.mask.begin(), first.mask.end(), uint8_t{1}));
  m.levels.push_back(std::move(first));
  Moments level0{};
  {
    const ModelLevel& L = m.levels.front();
    Raster& o = m.original;
    o.orow = L.orow;
    o.ocol = L.ocol;
    double mean = 0;
    size_t n = 0;
    for (size_t i = 0; i < L.gray.size(); ++i)
      if (L.mask[i]) mean += (L.gray[i] - mean) / double(++n);
    double energy = 0;
    std::vector<RawSample> s;
    s.reserve(m.sample_count);
    for (size_t r = 0; r < L.height; ++r)
      for (size_t c = 0; c < L.width; ++c)
        if (L.mask[r * L.width + c]) {
          const double v = L.gray[r * L.width + c] - mean;
          energy += v * v;
          s.push_back({int32_t(r), int32_t(c), v});
        }
    if (n < 4 || !(energy > 0) || !std::isfinite(energy))
      raise(kInvalidArgument, "constant template cannot define an NCC model");
    level0 = {mean, energy};
    const double norm = std::sqrt(energy);
    o.rmin = o.rmax = s.front().row;
    o.cmin = o.cmax = s.front().col;
    for (auto& x : s) {
      x.value /= norm;  // division (not multiplication by 1/norm), as the reference does for this raster
      o.rows.push_back(x.row);
      o.cols.push_back(x.col);
      o.w.push_back(x.value);
      o.rmin = std::min(o.rmin, x.row);
      o.rmax = std::max(o.rmax, x.row);
      o.cmin = std::min(o.cmin, x.col);
      o.cmax = std::max(o.cmax, x.col);
    }
  }
  const int wanted = params.levels ? params.levels : 16;
  while (m.levels.size() < size_t(wanted)) {
    const ModelLevel& prev = m.levels.back();
    if (prev.width < 8 || prev.height < 8) break;
    ModelLevel next;
    next.width = prev.width / 2;
    next.height = prev.height / 2;
    next.orow = (prev.orow - .5) * .5;
    next.ocol = (prev.ocol - .5) * .5;
    next.gray.resize(next.width * next.height);
    next.mask.resize(next.gray.size());
    for (size_t r = 0; r < next.height; ++r)
      for (size_t c = 0; c < next.width; ++c) {
        const size_t i = 2 * r * prev.width + 2 * c;
        next.mask[r * next.width + c] =
            prev.mask[i] && prev.mask[i + 1] && prev.mask[i + prev.width] && prev.mask[i + prev.width + 1];
        // 2x2 mean, left-to-right (src/imageproc/gray_pyramid.hpp:9-13)
        const double* top = prev.gray.data() + 2 * r * prev.width;
        const double* bot = prev.gray.data() + (2 * r + 1) * prev.width;
        const size_t c0 = 2 * c, c1 = c0 + 1 < prev.width ? c0 + 1 : c0;
        next.gray[r * next.width + c] = .25 * (top[c0] + top[c1] + bot[c0] + bot[c1]);
      }
    size_t count = 0;
    if (!level_usable(next, &count) || count < 8 || (m.levels.size() >= 2 && count < 64)) break;
    m.levels.push_back(std::move(next));
  }
  if (params.levels && m.levels.size() != size_t(params.levels))
    raise(kInvalidArgument, "requested pyramid level is degenerate or too small");
  const double radius = std::hypot(double(m.levels.front().width), double(m.levels.front().height)) * .5;
  m.params.angle_step =
      params.angle_step > 0 ? params.angle_step : std::max(.01, std::min(.15, 1 / std::max(1., radius)));
  const double intervals = std::ceil(params.angle_extent / m.params.angle_step);
  if (!std::isfinite(intervals) || intervals >= kAngles) raise(kLimitExceeded, "angle grid exceeds limit");
  const size_t angles = size_t(intervals) + 1;
  for (size_t i = 0; i < angles; ++i)
    m.angles.push_back(params.angle_start + std::min(params.angle_extent, i * m.params.angle_step));
  m.level0_mean = level0.mean;
  m.level0_energy = level0.energy;
  m.rasters = false;
  m.sample_budget = thread_budgets().samples;
  if (rasters) build_rasters(m);
  return m;
}

void build_rasters(HostModel& m) {
  const Moments level0{m.level0_mean, m.level0_energy};
  size_t total = 0;
  for (size_t li = 0; li < m.levels.size(); ++li) {
    ModelLevel& L = m.levels[li];
    L.patches.clear();
    L.patches.reserve(m.angles.size());
    for (const double angle : m.angles) {
      Raster p = rotate_impl(L, angle, li == 0 ? &level0 : nullptr);
      if (p.w.empty()) raise(kInvalidArgument, "rotation produces a degenerate template");
      if (p.size() > m.sample_budget - total) raise(kLimitExceeded, "model raster budget exceeded");
      total += p.size();
      L.patches.push_back(std::move(p));
    }
  }
  m.rasters = true;
}

namespace {

template <class T>
HostModel create_typed(const T* px, int64_t width, int64_t height, int64_t stride_elems, const uint8_t* mask,
                       const CreateParams& params, bool rasters) {
  // Template domain as runs: mask or the full rectangle.
  int64_t rmin = height, rmax = -1, cmin = width, cmax = -1, area = 0;
  struct Span { int64_t row, begin, end; };
  std::vector<Span> spans;
  for (int64_t r = 0; r < height; ++r) {
    if (!mask) {
      spans.push_back({r, 0, width - 1});
      continue;
    }
    int64_t c = 0;
    while (c < width) {
      while (c < width && !mask[r * width + c]) ++c;
      if (c >= width) break;
      const int64_t b = c;
      while (c < width && mask[r * width + c]) ++c;
      spans.push_back({r, b, c - 1});
    }
  }
  for (const Span& s : spans) {
    area += s.end - s.begin + 1;
    rmin = std::min(rmin, s.row);
    rmax = std::max(rmax, s.row);
    cmin = std::min(cmin, s.begin);
    cmax = std::max(cmax, s.end);
  }
  if (area < 4) raise(kInvalidArgument, "template domain requires at least four pixels");
  ModelLevel first;
  first.width = size_t(cmax - cmin + 1);
  first.height = size_t(rmax - rmin + 1);
  if (first.height > kTemplatePixels / first.width)
    raise(kLimitExceeded, "template bounding box exceeds one million pixels");
  first.gray.assign(first.width * first.height, 0.);
  first.mask.assign(first.gray.size(), 0);
  // Centroid in long double, integer sum for the mean (model.cpp:134-168).
  long double sum_row = 0, sum_col = 0;
  int64_t isum = 0;
  for (const Span& s : spans) {
    const int64_t count = s.end - s.begin + 1;
    sum_row += static_cast<long double>(s.row) * count;
    sum_col += (static_cast<long double>(s.begin) + s.end) * count / 2;
    const size_t base = size_t(s.row - rmin) * first.width;
    for (int64_t c = s.begin; c <= s.end; ++c) {
      const T v = px[s.row * stride_elems + c];
      first.gray[base + size_t(c - cmin)] = double(v);
      first.mask[base + size_t(c - cmin)] = 1;
      isum += v;
    }
  }
  const uint64_t a = uint64_t(area);
  const double origin_row = double(sum_row / a), origin_col = double(sum_col / a);
  first.orow = double((sum_row - static_cast<long double>(rmin) * a) / a);
  first.ocol = double((sum_col - static_cast<long double>(cmin) * a) / a);
  const double mean = double(isum) / double(a);
  for (size_t i = 0; i < first.gray.size(); ++i)
    if (first.mask[i]) first.gray[i] -= mean;
  return rebuild_model(std::move(first), params, origin_row, origin_col, rasters);
}

}  // namespace

HostModel create_model(const void* pixels, int type, int64_t width, int64_t height, int64_t stride_bytes,
                       const uint8_t* mask, const CreateParams& p, bool rasters) {
  if (!pixels) raise(kInvalidArgument, "template pixels must not be null");
  if (type != 0 && type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
  if (width <= 0 || height <= 0) raise(kInvalidArgument, "one nonempty single-channel image required");
  const int64_t bpp = type == 1 ? 2 : 1;
  if (stride_bytes < width * bpp || stride_bytes % bpp) raise(kInvalidArgument, "invalid row stride");
  if (!std::isfinite(p.angle_start) || !std::isfinite(p.angle_extent) || !std::isfinite(p.angle_step) ||
      p.angle_extent < 0 || p.angle_extent > kTwoPi || !std::isfinite(p.angle_start + p.angle_extent) ||
      p.angle_step < 0 || p.levels < 0 || p.levels > 16)
    raise(kInvalidArgument, "invalid levels or angle range");
  if (type == 1)
    return create_typed(static_cast<const uint16_t*>(pixels), width, height, stride_bytes / 2, mask, p, rasters);
  return create_typed(static_cast<const uint8_t*>(pixels), width, height, stride_bytes, mask, p, rasters);
}

Raster rotate_level(const ModelLevel& level, double angle) { return rotate_impl(level, angle, nullptr); }

}  // namespace mvg
