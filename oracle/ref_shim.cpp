// Test-only C shim over the reference mvkit NCC matcher, compiled from the
// reference's own sources (see oracle/Makefile).  It is the parity pin for the
// oracle restatement in ncc_oracle.cpp and the generator of tests/golden/.
// Nothing in the product links or loads this file.
//
// Entry points mirror the reference internal API:
//   mv::ncc_matching::create  src/ncc_matching/model.cpp:120
//   mv::ncc_matching::find    src/ncc_matching/matcher.cpp:1063
//   normalized_correlation    src/ncc_matching/model.cpp:105
#include <ncc_matching/model.hpp>
#include <core/exception.hpp>
#include <core/image.hpp>
#include <core/region.hpp>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

namespace {
namespace ncc = mv::ncc_matching;

void set_error(char* err, int len, const char* text) {
  if (!err || len <= 0) return;
  std::strncpy(err, text, std::size_t(len - 1));
  err[len - 1] = 0;
}

template <class Fn> int guarded(char* err, int len, Fn&& fn) {
  try {
    fn();
    return 0;
  } catch (const mv::core::Exception& e) {
    set_error(err, len, std::string(e.message()).c_str());
    return int(e.status());
  } catch (const std::bad_alloc&) {
    set_error(err, len, "out of memory");
    return -5;
  } catch (const std::exception& e) {
    set_error(err, len, e.what());
    return -1000;
  }
}

// Builds a reference Image from a dense pixel buffer; `mask` (w*h bytes,
// nullable) becomes the image domain through Region::from_runs.
mv::core::Image make_image(const void* pixels, int type, std::int64_t w, std::int64_t h,
                           std::int64_t stride, const std::uint8_t* mask) {
  const auto pt = type == 1 ? mv::core::PixelType::UInt16 : mv::core::PixelType::UInt8;
  const std::size_t bpp = type == 1 ? 2 : 1;
  auto image = mv::core::Image::create(std::size_t(w), std::size_t(h), pt);
  auto* dst = static_cast<std::byte*>(image.mutable_data());
  const auto* src = static_cast<const std::byte*>(pixels);
  for (std::int64_t r = 0; r < h; ++r)
    std::memcpy(dst + r * image.stride(), src + r * stride, std::size_t(w) * bpp);
  if (!mask) return image;
  std::vector<mv::core::RegionRun> runs;
  for (std::int64_t r = 0; r < h; ++r) {
    std::int64_t c = 0;
    while (c < w) {
      while (c < w && !mask[r * w + c]) ++c;
      if (c >= w) break;
      const auto begin = c;
      while (c < w && mask[r * w + c]) ++c;
      runs.emplace_back(r, begin, c - 1);
    }
  }
  return image.reduce_domain(mv::core::Region::from_runs(runs));
}
}  // namespace

extern "C" {

int ref_ncc_create(const void* tmpl, int type, std::int64_t w, std::int64_t h, std::int64_t stride,
                   const std::uint8_t* mask, int levels, double angle_start, double angle_extent,
                   double angle_step, int ignore_polarity, void** out, char* err, int errlen) {
  *out = nullptr;
  return guarded(err, errlen, [&] {
    ncc::CreateOptions o;
    o.levels = levels;
    o.angle_start = angle_start;
    o.angle_extent = angle_extent;
    o.angle_step = angle_step;
    o.ignore_global_polarity = ignore_polarity != 0;
    auto model = new ncc::Model(ncc::create(make_image(tmpl, type, w, h, stride, mask), o));
    *out = model;
  });
}

void ref_ncc_free(void* model) { delete static_cast<ncc::Model*>(model); }

// Model file bytes (mv::ncc_matching::serialize, src/ncc_matching/persist.cpp:33).
// Returns the size; copies min(size, cap) bytes into buf.  -1 on error.
std::int64_t ref_ncc_serialize(void* model, char* buf, std::int64_t cap, char* err, int errlen) {
  std::int64_t size = -1;
  const int status = guarded(err, errlen, [&] {
    const std::string bytes = ncc::serialize(*static_cast<ncc::Model*>(model));
    size = std::int64_t(bytes.size());
    if (buf && cap > 0) std::memcpy(buf, bytes.data(), std::size_t(std::min<std::int64_t>(cap, size)));
  });
  return status ? -1 : size;
}

// mv::ncc_matching::deserialize (src/ncc_matching/persist.cpp:44); returns
// the reference status.
int ref_ncc_deserialize(const char* bytes, std::int64_t size, void** out, char* err, int errlen) {
  *out = nullptr;
  return guarded(err, errlen, [&] {
    *out = new ncc::Model(ncc::deserialize(std::string_view(bytes, std::size_t(size))));
  });
}

// info[0]=levels info[1]=angle_step info[2]=origin_row info[3]=origin_column
// info[4]=patches per level (level 0)  info[5]=original sample count
void ref_ncc_model_info(void* model, double* info) {
  const auto& m = *static_cast<ncc::Model*>(model);
  info[0] = double(m.levels.size());
  info[1] = m.options.angle_step;
  info[2] = m.origin_row;
  info[3] = m.origin_column;
  info[4] = double(m.levels.front().patches.size());
  info[5] = double(m.original.samples.size());
}

// Level geometry: dims[0]=width dims[1]=height; origin[0..1]=origin row/col.
void ref_ncc_level(void* model, int level, std::int64_t* dims, double* origin) {
  const auto& l = static_cast<ncc::Model*>(model)->levels[std::size_t(level)];
  dims[0] = std::int64_t(l.width);
  dims[1] = std::int64_t(l.height);
  origin[0] = l.origin_row;
  origin[1] = l.origin_column;
}

// Copies one patch: returns sample count; rows/cols/weights are filled when
// non-null and capacity allows.  meta = {angle, origin_row, origin_column, weight_sum}.
std::int64_t ref_ncc_patch(void* model, int level, int index, std::int32_t* rows,
                           std::int32_t* cols, double* weights, std::int64_t capacity, double* meta) {
  const auto& m = *static_cast<ncc::Model*>(model);
  const auto& p = level < 0 ? m.original : m.levels[std::size_t(level)].patches[std::size_t(index)];
  meta[0] = p.angle;
  meta[1] = p.origin_row;
  meta[2] = p.origin_column;
  meta[3] = p.weight_sum;
  const auto n = std::int64_t(p.samples.size());
  if (rows && n <= capacity)
    for (std::int64_t i = 0; i < n; ++i) {
      rows[i] = p.samples[std::size_t(i)].row;
      cols[i] = p.samples[std::size_t(i)].column;
      weights[i] = p.samples[std::size_t(i)].weight;
    }
  return n;
}

// Runs the reference find; out is capacity x 4 doubles (row, column, angle,
// score) in the matcher's internal pixel-centre convention.
int ref_ncc_find(void* model, const void* img, int type, std::int64_t w, std::int64_t h,
                 std::int64_t stride, const std::uint8_t* domain, double angle_start,
                 double angle_extent, double min_score, std::int64_t num_matches, double max_overlap,
                 int subpixel, int highest, int lowest, double* out, std::int64_t capacity,
                 std::int64_t* count, char* err, int errlen) {
  *count = 0;
  return guarded(err, errlen, [&] {
    ncc::FindOptions o;
    o.angle_start = angle_start;
    o.angle_extent = angle_extent;
    o.min_score = min_score;
    o.num_matches = std::size_t(num_matches);
    o.max_overlap = max_overlap;
    o.subpixel = subpixel != 0;
    o.highest_level = highest;
    o.lowest_level = lowest < 1 ? 1 : lowest;
    const auto found = ncc::find(make_image(img, type, w, h, stride, domain),
                                 *static_cast<ncc::Model*>(model), o);
    *count = std::int64_t(found.size());
    for (std::size_t i = 0; i < found.size() && std::int64_t(i) < capacity; ++i) {
      out[4 * i + 0] = found[i].row;
      out[4 * i + 1] = found[i].column;
      out[4 * i + 2] = found[i].angle;
      out[4 * i + 3] = found[i].score;
    }
  });
}

// Runs the reference multi-model find (mv::ncc_matching::find_models,
// src/ncc_matching/matcher.cpp:1077) as mv_find_ncc_models calls it
// (src/c_api/ncc_matching_api.cpp:191-201): per-model options (arrays of
// `count`), the shared selection (num_matches / max_overlap, -1 = per model)
// and HALCON's quota-before-overlap rule.  out is capacity x 5 doubles (row,
// column, angle, score, model index) in the matcher's pixel-centre convention.
int ref_ncc_find_models(void* const* models, std::int64_t count, const void* img, int type, std::int64_t w,
                        std::int64_t h, std::int64_t stride, const double* angle_start,
                        const double* angle_extent, const double* min_score, const std::int64_t* num_matches,
                        const double* max_overlap, const int* subpixel, const int* highest, const int* lowest,
                        std::int64_t sel_num_matches, double sel_max_overlap, double* out, std::int64_t capacity,
                        std::int64_t* found_count, char* err, int errlen) {
  *found_count = 0;
  return guarded(err, errlen, [&] {
    std::vector<const ncc::Model*> ms;
    std::vector<ncc::FindOptions> opts;
    for (std::int64_t i = 0; i < count; ++i) {
      ms.push_back(static_cast<const ncc::Model*>(models[i]));
      ncc::FindOptions o;
      o.angle_start = angle_start[i];
      o.angle_extent = angle_extent[i];
      o.min_score = min_score[i];
      o.num_matches = std::size_t(num_matches[i]);
      o.max_overlap = max_overlap[i];
      o.subpixel = subpixel[i] != 0;
      o.highest_level = highest[i];
      o.lowest_level = lowest[i] < 1 ? 1 : lowest[i];
      opts.push_back(o);
    }
    mv::matching::Selection sel;
    sel.num_matches = sel_num_matches;
    sel.max_overlap = sel_max_overlap;
    const auto found = ncc::find_models(make_image(img, type, w, h, stride, nullptr), ms, opts, sel, true);
    *found_count = std::int64_t(found.size());
    for (std::size_t i = 0; i < found.size() && std::int64_t(i) < capacity; ++i) {
      out[5 * i + 0] = found[i].pose.row;
      out[5 * i + 1] = found[i].pose.column;
      out[5 * i + 2] = found[i].pose.angle;
      out[5 * i + 3] = found[i].pose.score;
      out[5 * i + 4] = double(found[i].model_index);
    }
  });
}

double ref_normalized_correlation(const double* a, const double* b, std::int64_t n, int absolute) {
  return ncc::normalized_correlation({a, std::size_t(n)}, {b, std::size_t(n)}, absolute != 0);
}

}  // extern "C"
