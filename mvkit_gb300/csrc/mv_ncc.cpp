// The reference's NCC operators with their own C signatures
// (include/mvkit_gb300_mv.h) over the GPU library (include/mvkit_gb300_ncc.h).
// Inputs are read through the public tuple / iconic calls only; control
// checks, their order, statuses and messages follow
// src/c_api/ncc_matching_api.cpp:
//   mv_create_ncc_model      :29-66
//   control_model, filename  :69-86
//   mv_get_ncc_model_params  :87-98
//   mv_write/read_ncc_model  :99-111
//   ncc_models, NccControls  :112-162
//   ncc_image, ncc_columns   :163-176 (the pose convention is applied by the
//                                      GPU library's find calls)
//   mv_find_ncc_model(s)     :178-203
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/mvkit_gb300_ncc.h"
#include "mv_objects.h"

namespace mvg::mv {
namespace {

// core::default_error_code (src/core/exception.hpp:26-43)
MvErrorCode default_code(int32_t status) {
  switch (status) {
    case MV_STATUS_INVALID_ARGUMENT: return MV_ERROR_INVALID_VALUE;
    case MV_STATUS_OUT_OF_RANGE: return MV_ERROR_INDEX_OUT_OF_RANGE;
    case MV_STATUS_TYPE_MISMATCH: return MV_ERROR_INVALID_TYPE;
    case MV_STATUS_NOT_FOUND: return MV_ERROR_MISSING_ITEM;
    case MV_STATUS_UNSUPPORTED: return MV_ERROR_UNSUPPORTED_VALUE;
    case MV_STATUS_INVALID_STATE: return MV_ERROR_INVALID_OBJECT_STATE;
    case MV_STATUS_IO_ERROR:
    case MV_STATUS_DECODE_ERROR:
    case MV_STATUS_ENCODE_ERROR: return MV_ERROR_IO_FAILURE;
    default: return MV_ERROR_INTERNAL_FAILURE;
  }
}

constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kPi = 3.14159265358979323846;

// A failed public call of the object layer, reported as this operator's.
[[noreturn]] void forward() {
  MvErrorInfo e{};
  mv_get_last_error_info(&e);
  fail(e.status, e.code, std::string(e.parameter.data, e.parameter.size), e.parameter_index,
       std::string(e.message.data, e.message.size));
}
void ok(MvStatus s) {
  if (s != MV_STATUS_OK) forward();
}

// The parameter the reference names for an error of its model build, search
// or model files (src/ncc_matching/model.cpp:86-237, matcher.cpp:349-591,
// persist.cpp:16), by message; nullptr where it names none.
const char* algorithm_parameter(const std::string& m) {
  static const struct {
    const char* message;
    const char* parameter;
  } table[] = {
      {"rotated bounding box exceeds budget", "domain"},
      {"one nonempty single-channel image required", "image"},
      {"invalid levels or angle range", "options"},
      {"template domain requires at least four pixels", "domain"},
      {"template domain must be inside", "domain"},
      {"template bounding box exceeds one million pixels", "domain"},
      {"template samples must be finite", "image"},
      {"constant template cannot define an NCC model", "image"},
      {"requested pyramid level is degenerate or too small", "levels"},
      {"angle grid exceeds limit", "angle_step"},
      {"rotation produces a degenerate template", "domain"},
      {"model raster budget exceeded", "angle_extent"},
      {"model is empty", "model"},
      {"invalid pyramid levels", "NumLevels"},
      {"invalid query range, score, overlap or candidate budget", "options"},
      {"query angle range must be finite", "angle_extent"},
      {"search image exceeds pixel budget", "image"},
      {"search samples must be finite", "image"},
      {"coarse candidate budget exceeded", "max_candidates"},
  };
  for (const auto& t : table)
    if (m.find(t.message) == 0) return t.parameter;
  return nullptr;
}

// Error code and parameter of an error the GPU library reports: the
// reference's parameter where it names one, else inferred from status and
// message as the reference's C layer infers them (src/c_api/structured_error.hpp:14-51,
// core/exception.hpp:26-43).  `files`: a model read or write, whose own
// format errors name the path (persist.cpp:16).
bool has(const std::string& s, const char* t) { return s.find(t) != std::string::npos; }
[[noreturn]] void library_failure(int32_t status, bool files = false) {
  const std::string m = mvg_last_error();
  if (const char* p = algorithm_parameter(m)) fail(status, default_code(status), p, -1, m);
  const bool io_layer = m == "cannot open model for reading" || m == "model file exceeds size limit" ||
                        m == "cannot read model file";
  if (files && !io_layer) fail(status, default_code(status), "path", -1, m);
  MvErrorCode code;
  if (has(m, "must not be null") || has(m, "null")) code = MV_ERROR_NULL_ARGUMENT;
  else if (status == MV_STATUS_OUT_OF_RANGE || has(m, "out of range") || has(m, "capacity is too small"))
    code = MV_ERROR_INDEX_OUT_OF_RANGE;
  else if (status == MV_STATUS_UNSUPPORTED || has(m, "unsupported")) code = MV_ERROR_UNSUPPORTED_VALUE;
  else if (status == MV_STATUS_INVALID_ARGUMENT) code = MV_ERROR_INVALID_VALUE;
  else if (status == MV_STATUS_TYPE_MISMATCH) code = MV_ERROR_INVALID_TYPE;
  else if (status == MV_STATUS_INVALID_STATE) code = MV_ERROR_INVALID_OBJECT_STATE;
  else if (status == MV_STATUS_IO_ERROR || status == MV_STATUS_DECODE_ERROR) code = MV_ERROR_IO_FAILURE;
  else code = MV_ERROR_INTERNAL_FAILURE;
  const char* parameter = has(m, "index")      ? "index"
                          : has(m, "capacity") ? "capacity"
                          : has(m, "output")   ? "output"
                          : has(m, "image")    ? "image"
                          : has(m, "region")   ? "regions"
                          : has(m, "tuple")    ? "tuple"
                          : has(m, "model")    ? "model"
                          : has(m, "string")   ? "value"
                          : has(m, "parameter") ? "parameter"
                                                : "argument";
  fail(status, code, parameter, -1, m);
}

// An owned tuple of the object layer, destroyed on scope exit.
struct Owned {
  MvTuple t = nullptr;
  ~Owned() {
    if (t) mv_destroy_tuple(t);
  }
};
struct OwnedObj {
  MvObject o = nullptr;
  ~OwnedObj() {
    if (o) mv_clear_obj(o);
  }
};

// The search or template image of an operator (ncc_image,
// ncc_matching_api.cpp:163-170): nullptr pixels for an empty object.  The
// domain becomes a byte mask unless it is the whole image.
struct ImageIn {
  const void* pixels = nullptr;
  int32_t type = 0;
  int64_t width = 0, height = 0, stride = 0;
  std::vector<uint8_t> mask;
  const uint8_t* domain() const { return mask.empty() ? nullptr : mask.data(); }
};

ImageIn read_image(MvObject obj, const char* parameter, bool allow_empty) {
  if (!obj)
    fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, parameter, -1,
         allow_empty ? "iconic handle must not be null" : "image handle must not be null");
  Owned ptr, type, w, h, count;
  ok(mv_get_image_pointer1(obj, &ptr.t, &type.t, &w.t, &h.t));  // checks the object kind
  ok(mv_count_obj(obj, &count.t));
  int64_t n = 0;
  ok(mv_get_i(count.t, 0, &n));
  ImageIn im;
  if (n == 0 && allow_empty) return im;
  if (n != 1)
    fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_INVALID_CARDINALITY, parameter, -1,
         "operator requires exactly one image object");
  MvStringView tv{nullptr, 0};
  ok(mv_get_s(type.t, 0, &tv));
  const std::string tn(tv.data, tv.size);
  if (tn != "byte" && tn != "uint2")
    fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, parameter, -1, "one byte or uint2 channel required");
  int64_t p = 0;
  ok(mv_get_i(ptr.t, 0, &p));
  ok(mv_get_i(w.t, 0, &im.width));
  ok(mv_get_i(h.t, 0, &im.height));
  im.pixels = reinterpret_cast<const void*>(uintptr_t(p));
  im.type = tn == "uint2" ? MVG_PIXEL_UINT2 : MVG_PIXEL_BYTE;
  im.stride = im.width * (tn == "uint2" ? 2 : 1);
  // domain: runs of mv_get_domain, as a mask unless they cover the image
  OwnedObj dom;
  ok(mv_get_domain(obj, &dom.o));
  Owned rr, rb, re;
  ok(mv_get_region_runs(dom.o, &rr.t, &rb.t, &re.t));
  size_t runs = 0;
  ok(mv_length_tuple(rr.t, &runs));
  int64_t area = 0;
  std::vector<int64_t> row(runs), b(runs), e(runs);
  for (size_t i = 0; i < runs; ++i) {
    ok(mv_get_i(rr.t, i, &row[i]));
    ok(mv_get_i(rb.t, i, &b[i]));
    ok(mv_get_i(re.t, i, &e[i]));
    area += e[i] - b[i] + 1;
  }
  if (area != im.width * im.height) {
    im.mask.assign(size_t(im.width) * size_t(im.height), 0);
    for (size_t i = 0; i < runs; ++i)
      std::memset(im.mask.data() + size_t(row[i]) * size_t(im.width) + size_t(b[i]), 1, size_t(e[i] - b[i] + 1));
  }
  return im;
}

void release_model(void* p) { mvg_clear_ncc_model(static_cast<mvg_ncc_model>(p)); }

// control_model (ncc_matching_api.cpp:69-77)
mvg_ncc_model control_model(MvTuple input) {
  const Control view(input, "ModelID");
  if (view.size() != 1) view.fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one NCC model required");
  const MvHandle h = view.handle(0);
  void* m = handle_object(h, MV_OBJECT_TYPE_NCC_MODEL);
  if (!m) view.fail(MV_ERROR_INVALID_TYPE, 0, "control handle is not an NCC model");
  return static_cast<mvg_ncc_model>(m);
}

// filename (ncc_matching_api.cpp:78-85)
std::string filename(MvTuple input) {
  const Control view(input, "FileName");
  if (view.size() != 1) view.fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one file name required");
  const std::string name = view.string(0);
  if (name.empty() || name.find('\0') != std::string::npos)
    view.fail(MV_ERROR_INVALID_VALUE, 0, "nonempty file name without NUL required");
  return name;
}

// ncc_models (ncc_matching_api.cpp:112-125)
std::vector<mvg_ncc_model> ncc_models(MvTuple input, bool multiple) {
  const Control ids(input, multiple ? "ModelIDs" : "ModelID");
  if (!ids.size() || ids.size() > 4096 || (!multiple && ids.size() != 1))
    ids.fail(MV_ERROR_INVALID_CARDINALITY, -1, "one model or a nonempty model array (maximum 4096) required");
  std::vector<mvg_ncc_model> out;
  for (size_t i = 0; i < ids.size(); ++i) {
    if (ids.kind(i) != MV_VALUE_HANDLE) ids.fail(MV_ERROR_INVALID_TYPE, int64_t(i), "NCC model handle required");
    void* m = handle_object(ids.handle(i), MV_OBJECT_TYPE_NCC_MODEL);
    if (!m) ids.fail(MV_ERROR_INVALID_TYPE, int64_t(i), "control handle is not an NCC model");
    out.push_back(static_cast<mvg_ncc_model>(m));
  }
  return out;
}

// NccControls (ncc_matching_api.cpp:126-162): per model, the checked
// controls as the GPU library's arrays.
struct Controls {
  std::vector<double> start, extent, score, overlap;
  std::vector<int64_t> matches;
  std::vector<int32_t> subpixel, levels;  // levels: (highest, lowest) per model
  int64_t n_matches = 0, n_overlap = 0;   // 1 = shared (selection), else per model
};

Controls controls(size_t count, MvTuple a, MvTuple e, MvTuple s, MvTuple n, MvTuple o, MvTuple p, MvTuple l) {
  const Control start(a, "AngleStart"), extent(e, "AngleExtent"), score(s, "MinScore"), matches(n, "NumMatches"),
      overlap(o, "MaxOverlap"), subpixel(p, "SubPixel"), levels(l, "NumLevels");
  for (const Control* c : {&start, &extent, &score, &matches, &overlap, &subpixel})
    if (c->size() != 1 && c->size() != count)
      c->fail(MV_ERROR_INVALID_CARDINALITY, -1, "one value or one value per model required");
  if (levels.size() != 1 && levels.size() != 2 && levels.size() != count && levels.size() != 2 * count)
    levels.fail(MV_ERROR_INVALID_CARDINALITY, -1, "highest level or shared/per-model level pairs required");
  auto number = [](const Control& v, size_t i, double lo, double hi) {
    const size_t at = v.size() == 1 ? 0 : i;
    const double x = v.number(at);
    if (!std::isfinite(x) || x < lo || x > hi) v.fail(MV_ERROR_INVALID_VALUE, int64_t(at), "numeric control outside allowed range");
    return x;
  };
  Controls c;
  for (size_t i = 0; i < count; ++i) {
    c.start.push_back(number(start, i, -std::numeric_limits<double>::max(), std::numeric_limits<double>::max()));
    c.extent.push_back(number(extent, i, 0, kTwoPi));
    c.score.push_back(number(score, i, 0, 1));
    c.overlap.push_back(number(overlap, i, 0, 1));
    const size_t mi = matches.size() == 1 ? 0 : i;
    const int64_t quota = matches.integer(mi);
    if (quota < 0) matches.fail(MV_ERROR_INVALID_VALUE, int64_t(mi), "match count must be nonnegative");
    c.matches.push_back(quota);
    const size_t si = subpixel.size() == 1 ? 0 : i;
    const std::string mode = subpixel.string(si);
    if (mode != "true" && mode != "false") subpixel.fail(MV_ERROR_UNSUPPORTED_VALUE, int64_t(si), "expected true or false");
    c.subpixel.push_back(mode == "true");
    size_t hi_at = 0, lo_at = 0;
    bool pair = false;
    if (levels.size() == count && count > 1) {
      hi_at = i;
    } else if (levels.size() == 2 * count) {
      hi_at = 2 * i;
      lo_at = hi_at + 1;
      pair = true;
    } else if (levels.size() == 2) {
      lo_at = 1;
      pair = true;
    }
    const int64_t highest = levels.integer(hi_at), lowest = pair ? levels.integer(lo_at) : 1;
    if (highest < 0 || highest > std::numeric_limits<int>::max() || lowest < 0 ||
        lowest > std::numeric_limits<int>::max())
      levels.fail(MV_ERROR_INVALID_VALUE, int64_t(hi_at), "invalid highest/lowest level pair");
    c.levels.push_back(int32_t(highest));
    c.levels.push_back(int32_t(std::max<int64_t>(1, lowest)));
  }
  c.n_matches = matches.size() == 1 ? 1 : int64_t(count);
  c.n_overlap = overlap.size() == 1 ? 1 : int64_t(count);
  return c;
}

}  // namespace
}  // namespace mvg::mv

using namespace mvg::mv;

extern "C" {

MvStatus mv_create_ncc_model(MvObject Template, MvTuple NumLevels, MvTuple AngleStart, MvTuple AngleExtent,
                             MvTuple AngleStep, MvTuple Metric, MvTuple* ModelID) {
  return run("create_ncc_model", [&] {
    Outputs output({ModelID});
    const ImageIn t = read_image(Template, "Template", false);
    const Control levels(NumLevels, "NumLevels"), start(AngleStart, "AngleStart"), extent(AngleExtent, "AngleExtent"),
        step(AngleStep, "AngleStep"), metric(Metric, "Metric");
    auto automatic = [](const Control& in) {
      if (in.size() != 1) in.fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one value required");
      if (in.kind(0) != MV_VALUE_STRING) return false;
      if (in.string(0) != "auto") in.fail(MV_ERROR_UNSUPPORTED_VALUE, 0, "expected auto");
      return true;
    };
    int32_t num_levels = 0;  // auto
    if (!automatic(levels)) {
      const int64_t count = levels.scalar_integer();
      if (count < 0 || count > 16) levels.fail(MV_ERROR_INVALID_VALUE, 0, "levels must be 0..16 or auto");
      num_levels = int32_t(count);
    }
    const double a0 = start.scalar_number(), ext = extent.scalar_number();
    double angle_step = 0;  // auto
    if (!automatic(step)) {
      angle_step = step.scalar_number();
      if (angle_step < 0 || angle_step > kPi / 16)
        step.fail(MV_ERROR_INVALID_VALUE, 0, "angle step must be in [0,pi/16] or auto");
    }
    if (metric.size() != 1) metric.fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one metric required");
    const std::string name = metric.string(0);
    int32_t m = MVG_METRIC_USE_POLARITY;
    if (name == "ignore_global_polarity") m = MVG_METRIC_IGNORE_GLOBAL_POLARITY;
    else if (name != "use_polarity") metric.fail(MV_ERROR_UNSUPPORTED_VALUE, 0, "unsupported NCC metric");
    mvg_ncc_model model = nullptr;
    const int32_t st = mvg_create_ncc_model(t.pixels, t.type, t.width, t.height, t.stride, t.domain(), num_levels, a0,
                                            ext, angle_step, m, &model);
    if (st != 0) library_failure(st);
    const MvHandle h = make_handle(MV_OBJECT_TYPE_NCC_MODEL, model, release_model);
    output.append_h(0, h);
    drop_handle(h);
    output.commit();
  });
}

MvStatus mv_get_ncc_model_params(MvTuple ModelID, MvTuple* NumLevels, MvTuple* AngleStart, MvTuple* AngleExtent,
                                 MvTuple* AngleStep, MvTuple* Metric) {
  return run("get_ncc_model_params", [&] {
    Outputs output({NumLevels, AngleStart, AngleExtent, AngleStep, Metric});
    const mvg_ncc_model model = control_model(ModelID);
    int32_t levels = 0, metric = 0;
    double start = 0, extent = 0, step = 0;
    const int32_t st = mvg_get_ncc_model_params(model, &levels, &start, &extent, &step, &metric);
    if (st != 0) library_failure(st);
    output.append_i(0, levels);
    output.append_d(1, start);
    output.append_d(2, extent);
    output.append_d(3, step);
    output.append_s(4, metric == MVG_METRIC_IGNORE_GLOBAL_POLARITY ? "ignore_global_polarity" : "use_polarity");
    output.commit();
  });
}

MvStatus mv_write_ncc_model(MvTuple ModelID, MvTuple FileName) {
  return run("write_ncc_model", [&] {
    const mvg_ncc_model model = control_model(ModelID);
    const std::string name = filename(FileName);
    const int32_t st = mvg_write_ncc_model(model, name.c_str());
    if (st != 0) library_failure(st, true);
  });
}

MvStatus mv_read_ncc_model(MvTuple FileName, MvTuple* ModelID) {
  return run("read_ncc_model", [&] {
    Outputs output({ModelID});
    const std::string name = filename(FileName);
    mvg_ncc_model model = nullptr;
    const int32_t st = mvg_read_ncc_model(name.c_str(), &model);
    if (st != 0) library_failure(st, true);
    const MvHandle h = make_handle(MV_OBJECT_TYPE_NCC_MODEL, model, release_model);
    output.append_h(0, h);
    drop_handle(h);
    output.commit();
  });
}

MvStatus mv_find_ncc_model(MvObject Image, MvTuple ModelID, MvTuple AngleStart, MvTuple AngleExtent, MvTuple MinScore,
                           MvTuple NumMatches, MvTuple MaxOverlap, MvTuple SubPixel, MvTuple NumLevels, MvTuple* Row,
                           MvTuple* Column, MvTuple* Angle, MvTuple* Score) {
  return run("find_ncc_model", [&] {
    Outputs output({Row, Column, Angle, Score});
    const ImageIn im = read_image(Image, "Image", true);
    const std::vector<mvg_ncc_model> models = ncc_models(ModelID, false);
    const Controls c = controls(1, AngleStart, AngleExtent, MinScore, NumMatches, MaxOverlap, SubPixel, NumLevels);
    if (!im.pixels) {
      output.commit();
      return;
    }
    std::vector<double> r, col, a, s;
    int64_t capacity = 256, count = 0;
    for (;;) {
      r.resize(size_t(capacity));
      col.resize(size_t(capacity));
      a.resize(size_t(capacity));
      s.resize(size_t(capacity));
      const int32_t st = mvg_find_ncc_model(im.pixels, im.type, im.width, im.height, im.stride, MVG_MEMORY_HOST,
                                            im.domain(), models[0], c.start[0], c.extent[0], c.score[0],
                                            c.matches[0], c.overlap[0], c.subpixel[0], c.levels[0], c.levels[1],
                                            r.data(), col.data(), a.data(), s.data(), capacity, &count, nullptr);
      if (st != 0) library_failure(st);
      if (count <= capacity) break;
      capacity = count;
    }
    for (int64_t i = 0; i < count; ++i) {
      output.append_d(0, r[size_t(i)]);
      output.append_d(1, col[size_t(i)]);
      output.append_d(2, a[size_t(i)]);
      output.append_d(3, s[size_t(i)]);
    }
    output.commit();
  });
}

MvStatus mv_find_ncc_models(MvObject Image, MvTuple ModelIDs, MvTuple AngleStart, MvTuple AngleExtent,
                            MvTuple MinScore, MvTuple NumMatches, MvTuple MaxOverlap, MvTuple SubPixel,
                            MvTuple NumLevels, MvTuple* Row, MvTuple* Column, MvTuple* Angle, MvTuple* Score,
                            MvTuple* Model) {
  return run("find_ncc_models", [&] {
    Outputs output({Row, Column, Angle, Score, Model});
    const ImageIn im = read_image(Image, "Image", true);
    const std::vector<mvg_ncc_model> models = ncc_models(ModelIDs, true);
    const Controls c =
        controls(models.size(), AngleStart, AngleExtent, MinScore, NumMatches, MaxOverlap, SubPixel, NumLevels);
    if (!im.pixels) {
      output.commit();
      return;
    }
    // per-model values, except NumMatches / MaxOverlap given once (a
    // selection over all models)
    const int64_t nm = int64_t(models.size());
    std::vector<double> r, col, a, s;
    std::vector<int64_t> mi;
    int64_t capacity = 256, count = 0;
    for (;;) {
      r.resize(size_t(capacity));
      col.resize(size_t(capacity));
      a.resize(size_t(capacity));
      s.resize(size_t(capacity));
      mi.resize(size_t(capacity));
      const int32_t st = mvg_find_ncc_models(
          im.pixels, im.type, im.width, im.height, im.stride, MVG_MEMORY_HOST, im.domain(), models.data(), nm,
          c.start.data(), nm, c.extent.data(), nm, c.score.data(), nm, c.matches.data(), c.n_matches,
          c.overlap.data(), c.n_overlap, c.subpixel.data(), nm, c.levels.data(), 2 * nm, r.data(), col.data(),
          a.data(), s.data(), mi.data(), capacity, &count, nullptr);
      if (st != 0) library_failure(st);
      if (count <= capacity) break;
      capacity = count;
    }
    for (int64_t i = 0; i < count; ++i) {
      output.append_d(0, r[size_t(i)]);
      output.append_d(1, col[size_t(i)]);
      output.append_d(2, a[size_t(i)]);
      output.append_d(3, s[size_t(i)]);
      output.append_i(4, mi[size_t(i)]);
    }
    output.commit();
  });
}

}  // extern "C"
