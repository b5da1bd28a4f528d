// Minimal tuple / handle / iconic-object layer with the reference's public C
// signatures (include/mvkit_gb300_mv.h), enough for callers of the NCC
// operators: tuples of int64 / real64 / string / handle values, reference
// counted handles, single-channel images with a domain, rectangle regions,
// and the thread-local structured error.  Statuses, error codes, parameter
// names and messages follow the reference's C layer:
//   tuples    src/c_api/tuple_api.cpp, tuple_input.hpp
//   handles   src/c_api/handle_api.cpp:57-66
//   iconic    src/c_api/iconic_api.cpp:23-46, iconic_handle.hpp
//   images    src/c_api/image_api.cpp:12-133, image_controls.hpp
//   regions   src/c_api/region_control_api.cpp:20-113, region_api.cpp:89-110
//   domains   src/c_api/image_processing_api.cpp:80-88,239-252
//   errors    src/c_api/error_state.cpp, error_state.hpp:29-57
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "mv_objects.h"

// ------------------------------------------------------------------ objects
struct MvHandleImpl {
  std::atomic<int64_t> refs{1};
  std::mutex m;
  uint64_t type = 0;
  bool cleared = false;
  void* object = nullptr;
  void (*release)(void*) = nullptr;
  // Releases the object now; returns false when it was cleared before.
  bool clear() {
    void* o = nullptr;
    void (*r)(void*) = nullptr;
    {
      std::lock_guard<std::mutex> lock(m);
      if (cleared) return false;
      cleared = true;
      o = object;
      r = release;
      object = nullptr;
      release = nullptr;
    }
    if (o && r) r(o);
    return true;
  }
  ~MvHandleImpl() { clear(); }
};

namespace {

void ref(MvHandleImpl* h) {
  if (h) h->refs.fetch_add(1, std::memory_order_relaxed);
}
void unref(MvHandleImpl* h) {
  if (h && h->refs.fetch_sub(1, std::memory_order_acq_rel) == 1) delete h;
}

// One tuple element.
struct Value {
  MvValueKind kind = MV_VALUE_EMPTY;
  int64_t i = 0;
  double d = 0;
  std::string s;
  MvHandleImpl* h = nullptr;
  Value() = default;
  Value(const Value& o) : kind(o.kind), i(o.i), d(o.d), s(o.s), h(o.h) { ref(h); }
  Value& operator=(const Value& o) {
    if (this != &o) {
      ref(o.h);
      unref(h);
      kind = o.kind;
      i = o.i;
      d = o.d;
      s = o.s;
      h = o.h;
    }
    return *this;
  }
  ~Value() { unref(h); }
};

struct Run {
  int64_t row, cb, ce;  // columns cb..ce inclusive
};

// A single-channel image (pixels shared between copies) with its domain, or
// a region.
struct Iconic {
  bool image = false;
  std::shared_ptr<const std::vector<uint8_t>> pixels;
  std::string type;  // "byte", "uint2", "int2", "int4", "real"
  int64_t width = 0, height = 0, bpp = 1;
  bool full_domain = true;
  std::vector<Run> runs;  // the domain of an image, the runs of a region
};

}  // namespace

struct MvTupleImpl {
  std::vector<Value> v;
};

struct MvObjectImpl {
  std::vector<Iconic> items;
};

namespace mvg::mv {
namespace {

struct ErrorState {
  MvStatus status = MV_STATUS_OK;
  MvErrorCode code = MV_ERROR_UNSPECIFIED;
  std::string operation, parameter, message, composed;
  int64_t index = MV_ERROR_PARAMETER_INDEX_NONE;
};
thread_local ErrorState t_error;

[[noreturn]] void null_output(const char* parameter) {
  fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, parameter, -1, "output pointer must not be null");
}
void require_output(const void* p, const char* parameter = "output") {
  if (!p) null_output(parameter);
}
void require_iconic(MvObject o, const char* parameter = "objects") {
  if (!o) fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, parameter, -1, "iconic handle must not be null");
}
void require_kind(MvObject o, bool image) {
  for (size_t k = 0; k < o->items.size(); ++k)
    if (o->items[k].image != image)
      fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, "Objects", int64_t(k),
           "iconic tuple contains an incompatible object kind");
}
void require_tuple(MvTuple t) {
  if (!t) fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, "tuple", -1, "tuple must not be null");
}
void require_index(MvTuple t, size_t i) {
  if (i >= t->v.size())
    fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_INDEX_OUT_OF_RANGE, "tuple", int64_t(i),
         "control tuple index out of range");
}
MvTuple new_tuple() { return new MvTupleImpl; }
MvObject new_object() { return new MvObjectImpl; }

int64_t bytes_per_sample(const std::string& type) {
  if (type == "byte") return 1;
  if (type == "uint2" || type == "int2") return 2;
  return 4;
}

// Type, size and pointer controls of the image generators
// (src/c_api/image_api.cpp:16-50, image_controls.hpp:8-11)
std::string pixel_type(MvTuple t) {
  const Control c(t, "Type");
  if (c.size() != 1) c.fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one string required");
  const std::string name = c.string(0);
  if (name == "byte" || name == "uint2" || name == "int2" || name == "int4" || name == "real") return name;
  c.fail(MV_ERROR_UNSUPPORTED_VALUE, 0, "unsupported image type");
}
int64_t extent(MvTuple t, const char* parameter) {
  const Control c(t, parameter);
  const int64_t n = c.scalar_integer();
  if (n <= 0) c.fail(MV_ERROR_INVALID_VALUE, 0, "positive image size required");
  return n;
}
uintptr_t address(MvTuple t, const char* parameter) {
  const Control c(t, parameter);
  const int64_t n = c.scalar_integer();
  if (n == 0) c.fail(MV_ERROR_INVALID_VALUE, 0, "invalid pointer value");
  return uintptr_t(uint64_t(n));
}

MvObject make_image(const std::string& type, int64_t w, int64_t h, const void* src) {
  Iconic im;
  im.image = true;
  im.type = type;
  im.width = w;
  im.height = h;
  im.bpp = bytes_per_sample(type);
  const uint64_t bytes = uint64_t(w) * uint64_t(h) * uint64_t(im.bpp);
  if (bytes / uint64_t(im.bpp) / uint64_t(h) != uint64_t(w) || bytes > (uint64_t(1) << 40))
    fail(MV_STATUS_OUT_OF_MEMORY, MV_ERROR_INTERNAL_FAILURE, "", -1, "image too large");
  auto px = std::make_shared<std::vector<uint8_t>>(size_t(bytes), uint8_t(0));
  if (src) std::memcpy(px->data(), src, size_t(bytes));
  im.pixels = std::move(px);
  MvObject o = new_object();
  o->items.push_back(std::move(im));
  return o;
}

// Runs of a region clipped to rows [0, h) and columns [0, w)
std::vector<Run> clip_runs(const std::vector<Run>& runs, int64_t w, int64_t h) {
  std::vector<Run> out;
  for (const Run& r : runs) {
    if (r.row < 0 || r.row >= h) continue;
    const int64_t b = std::max<int64_t>(r.cb, 0), e = std::min<int64_t>(r.ce, w - 1);
    if (b <= e) out.push_back({r.row, b, e});
  }
  return out;
}

}  // namespace

[[noreturn]] void fail(MvStatus status, MvErrorCode code, const std::string& parameter, int64_t index,
                       const std::string& message) {
  throw Failure{status, code, parameter, index, message};
}

void set_error(MvStatus status, const char* operation, const Failure& f) noexcept {
  try {
    ErrorState e;
    e.status = status;
    e.code = f.code;
    e.operation = operation ? operation : "";
    e.parameter = f.parameter;
    e.index = f.index;
    e.message = f.message;
    e.composed = e.operation.empty() ? e.message
                 : e.message.empty() ? e.operation
                                     : e.operation + ": " + e.message;
    t_error = std::move(e);
  } catch (...) {
    t_error.status = status;
    t_error.code = f.code;
  }
}

const std::string& error_text() noexcept { return t_error.composed; }

MvErrorInfo error_info() noexcept {
  auto view = [](const std::string& x) { return MvStringView{x.data(), x.size()}; };
  return MvErrorInfo{t_error.status, t_error.code, view(t_error.operation), view(t_error.parameter), t_error.index,
                     view(t_error.message)};
}

void clear_error() noexcept {
  t_error.status = MV_STATUS_OK;
  t_error.code = MV_ERROR_UNSPECIFIED;
  t_error.operation.clear();
  t_error.parameter.clear();
  t_error.message.clear();
  t_error.composed.clear();
  t_error.index = MV_ERROR_PARAMETER_INDEX_NONE;
}

// ------------------------------------------------------------------ Control
// Reads through the public tuple calls only (mv_length_tuple, mv_get_type,
// mv_get_i/d/s/h), as an operator linked against another tuple layer would.
Control::Control(MvTuple t, const char* parameter) : t_(t), parameter_(parameter) {
  if (t && mv_length_tuple(t, &n_) != MV_STATUS_OK) n_ = 0;
}

void Control::fail(MvErrorCode code, int64_t index, const std::string& message) const {
  mv::fail(code == MV_ERROR_INVALID_TYPE ? MV_STATUS_TYPE_MISMATCH : MV_STATUS_INVALID_ARGUMENT, code, parameter_,
           index, message);
}
void Control::index_check(size_t i) const {
  if (i >= n_) fail(MV_ERROR_INDEX_OUT_OF_RANGE, int64_t(i), "control tuple index out of range");
}
MvValueKind Control::kind(size_t i) const {
  index_check(i);
  MvValueKind k = MV_VALUE_EMPTY;
  mv_get_type(t_, i, &k);
  return k;
}
double Control::number(size_t i) const {
  const MvValueKind k = kind(i);
  if (k != MV_VALUE_INT64 && k != MV_VALUE_REAL64) fail(MV_ERROR_INVALID_TYPE, int64_t(i), "numeric control value required");
  if (k == MV_VALUE_INT64) {
    int64_t x = 0;
    mv_get_i(t_, i, &x);
    return double(x);
  }
  double x = 0;
  mv_get_d(t_, i, &x);
  return x;
}
int64_t Control::integer(size_t i) const {
  if (kind(i) != MV_VALUE_INT64) fail(MV_ERROR_INVALID_TYPE, int64_t(i), "integer control value required");
  int64_t x = 0;
  mv_get_i(t_, i, &x);
  return x;
}
std::string Control::string(size_t i) const {
  if (kind(i) != MV_VALUE_STRING) fail(MV_ERROR_INVALID_TYPE, int64_t(i), "string control value required");
  MvStringView v{nullptr, 0};
  mv_get_s(t_, i, &v);
  return std::string(v.data ? v.data : "", v.size);
}
MvHandle Control::handle(size_t i) const {
  if (kind(i) != MV_VALUE_HANDLE) fail(MV_ERROR_INVALID_TYPE, int64_t(i), "NCC model handle required");
  MvHandle h = nullptr;
  mv_get_h(t_, i, &h);
  return h;
}
double Control::scalar_number() const {
  if (n_ != 1) fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one control value required");
  const double x = number(0);
  if (!std::isfinite(x)) fail(MV_ERROR_INVALID_VALUE, 0, "finite control value required");
  return x;
}
int64_t Control::scalar_integer() const {
  if (n_ != 1) fail(MV_ERROR_INVALID_CARDINALITY, -1, "exactly one control value required");
  return integer(0);
}

// ------------------------------------------------------------------ Outputs
Outputs::Outputs(std::initializer_list<MvTuple*> destinations) : dest_(destinations) {
  for (size_t i = 0; i < dest_.size(); ++i) {
    if (!dest_[i]) fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, "Output", int64_t(i),
                        "output must not be null");
    const uintptr_t a = reinterpret_cast<uintptr_t>(dest_[i]);
    for (size_t j = 0; j < i; ++j) {
      const uintptr_t b = reinterpret_cast<uintptr_t>(dest_[j]);
      if ((a < b ? b - a : a - b) < sizeof(MvTuple))
        fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_INVALID_VALUE, "Output", int64_t(i),
             "output ranges must be distinct");
    }
  }
  for (size_t i = 0; i < dest_.size(); ++i) values_.push_back(new_tuple());
}
Outputs::~Outputs() {
  for (MvTuple t : values_) delete t;
}
void Outputs::append_d(size_t i, double x) {
  Value v;
  v.kind = MV_VALUE_REAL64;
  v.d = x;
  values_[i]->v.push_back(v);
}
void Outputs::append_i(size_t i, int64_t x) {
  Value v;
  v.kind = MV_VALUE_INT64;
  v.i = x;
  values_[i]->v.push_back(v);
}
void Outputs::append_s(size_t i, const std::string& x) {
  Value v;
  v.kind = MV_VALUE_STRING;
  v.s = x;
  values_[i]->v.push_back(v);
}
void Outputs::append_h(size_t i, MvHandle h) {
  Value v;
  v.kind = MV_VALUE_HANDLE;
  v.h = h;
  ref(h);
  values_[i]->v.push_back(v);
}
void Outputs::commit() {
  for (size_t i = 0; i < dest_.size(); ++i) {
    *dest_[i] = values_[i];
    values_[i] = nullptr;
  }
}

// ------------------------------------------------------------------ handles
MvHandle make_handle(uint64_t type, void* object, void (*release)(void*)) {
  auto* h = new MvHandleImpl;
  h->type = type;
  h->object = object;
  h->release = release;
  return h;
}
void* handle_object(MvHandle h, uint64_t type) {
  if (!h) return nullptr;
  std::lock_guard<std::mutex> lock(h->m);
  if (h->type != type) return nullptr;
  if (h->cleared)
    throw Failure{MV_STATUS_INVALID_STATE, MV_ERROR_INVALID_OBJECT_STATE, "ModelID", -1, "handle has been cleared",
                  "control handle"};
  return h->object;
}
void drop_handle(MvHandle h) { unref(h); }

}  // namespace mvg::mv

using namespace mvg::mv;

extern "C" {

// ------------------------------------------------------------------ tuples
MvStatus mv_create_tuple(MvTuple* tuple, size_t length) {
  return run("mv_create_tuple", [&] {
    require_output(tuple);
    MvTuple t = new_tuple();
    t->v.resize(length);
    *tuple = t;
  });
}

MvStatus mv_copy_tuple(MvTuple tuple, MvTuple* clone) {
  return run("mv_copy_tuple", [&] {
    require_tuple(tuple);
    require_output(clone);
    MvTuple t = new_tuple();
    t->v = tuple->v;
    *clone = t;
  });
}

MvStatus mv_destroy_tuple(MvTuple tuple) {
  return run("mv_destroy_tuple", [&] {
    require_tuple(tuple);
    delete tuple;
  });
}

MvStatus mv_length_tuple(MvTuple tuple, size_t* size) {
  return run("mv_length_tuple", [&] {
    require_tuple(tuple);
    require_output(size);
    *size = tuple->v.size();
  });
}

MvStatus mv_resize_tuple(MvTuple tuple, size_t length) {
  return run("mv_resize_tuple", [&] {
    require_tuple(tuple);
    tuple->v.resize(length);
  });
}

MvStatus mv_get_type(MvTuple tuple, size_t index, MvValueKind* kind) {
  return run("mv_get_type", [&] {
    require_tuple(tuple);
    require_output(kind);
    require_index(tuple, index);
    *kind = tuple->v[index].kind;
  });
}

MvStatus mv_get_i(MvTuple tuple, size_t index, int64_t* value) {
  return run("mv_get_i", [&] {
    require_tuple(tuple);
    require_output(value);
    require_index(tuple, index);
    const Value& v = tuple->v[index];
    if (v.kind != MV_VALUE_INT64)
      fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, "tuple", int64_t(index), "integer value required");
    *value = v.i;
  });
}

MvStatus mv_get_d(MvTuple tuple, size_t index, double* value) {
  return run("mv_get_d", [&] {
    require_tuple(tuple);
    require_output(value);
    require_index(tuple, index);
    const Value& v = tuple->v[index];
    if (v.kind == MV_VALUE_INT64) *value = double(v.i);
    else if (v.kind == MV_VALUE_REAL64) *value = v.d;
    else fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, "tuple", int64_t(index), "numeric control value required");
  });
}

MvStatus mv_get_s(MvTuple tuple, size_t index, MvStringView* value) {
  return run("mv_get_s", [&] {
    require_tuple(tuple);
    require_output(value);
    require_index(tuple, index);
    const Value& v = tuple->v[index];
    if (v.kind != MV_VALUE_STRING)
      fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, "tuple", int64_t(index), "string control value required");
    value->data = v.s.data();
    value->size = v.s.size();
  });
}

MvStatus mv_get_h(MvTuple tuple, size_t index, MvHandle* handle) {
  return run("mv_get_h", [&] {
    require_tuple(tuple);
    require_output(handle);
    require_index(tuple, index);
    const Value& v = tuple->v[index];
    if (v.kind != MV_VALUE_HANDLE)
      fail(MV_STATUS_TYPE_MISMATCH, MV_ERROR_INVALID_TYPE, "tuple", int64_t(index), "handle value required");
    *handle = v.h;
  });
}

MvStatus mv_set_i(MvTuple tuple, int64_t value, size_t index) {
  return run("mv_set_i", [&] {
    require_tuple(tuple);
    require_index(tuple, index);
    Value v;
    v.kind = MV_VALUE_INT64;
    v.i = value;
    tuple->v[index] = v;
  });
}

MvStatus mv_set_d(MvTuple tuple, double value, size_t index) {
  return run("mv_set_d", [&] {
    require_tuple(tuple);
    require_index(tuple, index);
    Value v;
    v.kind = MV_VALUE_REAL64;
    v.d = value;
    tuple->v[index] = v;
  });
}

MvStatus mv_set_s(MvTuple tuple, MvStringView value, size_t index) {
  return run("mv_set_s", [&] {
    require_tuple(tuple);
    if (!value.data && value.size)
      fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_NULL_ARGUMENT, "value", -1, "string data must not be null");
    require_index(tuple, index);
    Value v;
    v.kind = MV_VALUE_STRING;
    v.s.assign(value.data ? value.data : "", value.size);
    tuple->v[index] = v;
  });
}

MvStatus mv_set_h(MvTuple tuple, MvHandle value, size_t index) {
  return run("mv_set_h", [&] {
    require_tuple(tuple);
    require_output(value, "value");
    require_index(tuple, index);
    Value v;
    v.kind = MV_VALUE_HANDLE;
    v.h = value;
    ref(value);
    tuple->v[index] = v;
  });
}

// src/c_api/handle_api.cpp:57-66
MvStatus mv_clear_handle(MvTuple Handle) {
  return run("clear_handle", [&] {
    const Control c(Handle, "Handle");
    for (size_t i = 0; i < c.size(); ++i) {
      if (c.kind(i) != MV_VALUE_HANDLE) c.fail(MV_ERROR_INVALID_TYPE, int64_t(i), "control handle required");
      if (!Handle->v[i].h->clear())
        fail(MV_STATUS_INVALID_STATE, MV_ERROR_INVALID_OBJECT_STATE, "argument", -1,
             "handle has already been cleared");
    }
  });
}

// ------------------------------------------------------------------ iconic
MvStatus mv_gen_empty_obj(MvObject* objects) {
  return run("gen_empty_obj", [&] {
    require_output(objects, "EmptyObject");
    *objects = new_object();
  });
}

MvStatus mv_clear_obj(MvObject objects) {
  return run("mv_clear_obj", [&] {
    require_iconic(objects);
    delete objects;
  });
}

MvStatus mv_count_obj(MvObject objects, MvTuple* count) {
  return run("count_obj", [&] {
    require_iconic(objects, "Objects");
    require_output(count, "Number");
    MvTuple t = new_tuple();
    Value v;
    v.kind = MV_VALUE_INT64;
    v.i = int64_t(objects->items.size());
    t->v.push_back(v);
    *count = t;
  });
}

MvStatus mv_gen_image_const(MvObject* Image, MvTuple Type, MvTuple Width, MvTuple Height) {
  return run("gen_image_const", [&] {
    require_output(Image, "Image");
    const std::string type = pixel_type(Type);
    const int64_t w = extent(Width, "Width"), h = extent(Height, "Height");
    *Image = make_image(type, w, h, nullptr);
  });
}

MvStatus mv_gen_image1(MvObject* Image, MvTuple Type, MvTuple Width, MvTuple Height, MvTuple PixelPointer) {
  return run("gen_image1", [&] {
    require_output(Image, "Image");
    const uintptr_t p = address(PixelPointer, "PixelPointer");
    const std::string type = pixel_type(Type);
    const int64_t w = extent(Width, "Width"), h = extent(Height, "Height");
    *Image = make_image(type, w, h, reinterpret_cast<const void*>(p));
  });
}

MvStatus mv_get_image_pointer1(MvObject Image, MvTuple* Pointer, MvTuple* Type, MvTuple* Width, MvTuple* Height) {
  return run("get_image_pointer1", [&] {
    require_iconic(Image, "Image");
    require_kind(Image, true);
    Outputs out({Pointer, Type, Width, Height});
    for (const Iconic& im : Image->items) {
      out.append_i(0, int64_t(reinterpret_cast<uintptr_t>(im.pixels->data())));
      out.append_s(1, im.type);
      out.append_i(2, im.width);
      out.append_i(3, im.height);
    }
    out.commit();
  });
}

MvStatus mv_get_image_size(MvObject Image, MvTuple* Width, MvTuple* Height) {
  return run("get_image_size", [&] {
    require_iconic(Image, "Image");
    require_kind(Image, true);
    Outputs out({Width, Height});
    for (const Iconic& im : Image->items) {
      out.append_i(0, im.width);
      out.append_i(1, im.height);
    }
    out.commit();
  });
}

MvStatus mv_get_image_type(MvObject Image, MvTuple* Type) {
  return run("get_image_type", [&] {
    require_iconic(Image, "Image");
    require_kind(Image, true);
    Outputs out({Type});
    for (const Iconic& im : Image->items) out.append_s(0, im.type);
    out.commit();
  });
}

// src/c_api/region_control_api.cpp:20-38,102-113
MvStatus mv_gen_rectangle1(MvObject* Rectangle, MvTuple Row1, MvTuple Column1, MvTuple Row2, MvTuple Column2) {
  return run("mv_gen_rectangle1", [&] {
    require_output(Rectangle, "Rectangle");
    const Control in[4] = {Control(Row1, "Row1"), Control(Column1, "Column1"), Control(Row2, "Row2"),
                           Control(Column2, "Column2")};
    size_t count = 0;
    bool empty = false;
    for (const Control& c : in) {
      count = std::max(count, c.size());
      empty = empty || c.size() == 0;
    }
    if (empty) count = 0;
    for (const Control& c : in)
      if (c.size() != 1 && c.size() != count)
        c.fail(MV_ERROR_INVALID_CARDINALITY, -1, "generation controls must have matching lengths or be scalar");
    MvObject o = new_object();
    std::unique_ptr<MvObjectImpl> guard(o);
    for (size_t i = 0; i < count; ++i) {
      int64_t v[4];
      for (int k = 0; k < 4; ++k) {
        const size_t at = in[k].size() == 1 ? 0 : i;
        const double x = in[k].number(at);
        if (!std::isfinite(x)) in[k].fail(MV_ERROR_INVALID_VALUE, int64_t(at), "finite control value required");
        if (x < double(std::numeric_limits<int32_t>::min()) || x > double(std::numeric_limits<int32_t>::max()))
          mvg::mv::fail(MV_STATUS_OUT_OF_RANGE, MV_ERROR_INDEX_OUT_OF_RANGE, k == 0 ? "Row1" : k == 1 ? "Column1"
                                                                           : k == 2 ? "Row2" : "Column2",
                        int64_t(at), "coordinate exceeds int32 range");
        v[k] = int64_t(std::round(x));
      }
      Iconic r;
      if (v[0] <= v[2] && v[1] <= v[3])
        for (int64_t row = v[0]; row <= v[2]; ++row) r.runs.push_back({row, v[1], v[3]});
      o->items.push_back(std::move(r));
    }
    *Rectangle = guard.release();
  });
}

// src/c_api/region_api.cpp:89-110
MvStatus mv_get_region_runs(MvObject Region, MvTuple* Row, MvTuple* ColumnBegin, MvTuple* ColumnEnd) {
  return run("get_region_runs", [&] {
    Outputs out({Row, ColumnBegin, ColumnEnd});
    require_iconic(Region, "Region");
    require_kind(Region, false);
    if (Region->items.size() > 1)
      fail(MV_STATUS_INVALID_ARGUMENT, MV_ERROR_INVALID_CARDINALITY, "Region", -1,
           "one region or a zero-object array required");
    if (!Region->items.empty())
      for (const Run& r : Region->items[0].runs) {
        out.append_i(0, r.row);
        out.append_i(1, r.cb);
        out.append_i(2, r.ce);
      }
    out.commit();
  });
}

// src/c_api/image_processing_api.cpp:239-252: the first region, clipped to
// each image, becomes its domain
MvStatus mv_reduce_domain(MvObject Image, MvObject Region, MvObject* ImageReduced) {
  return run("reduce_domain", [&] {
    require_iconic(Image, "Image");
    require_iconic(Region, "Region");
    require_output(ImageReduced, "ImageReduced");
    require_kind(Region, false);
    require_kind(Image, true);
    MvObject o = new_object();
    std::unique_ptr<MvObjectImpl> guard(o);
    static const std::vector<Run> none;
    const std::vector<Run>& runs = Region->items.empty() ? none : Region->items[0].runs;
    for (const Iconic& im : Image->items) {
      Iconic r = im;
      r.runs = clip_runs(runs, im.width, im.height);
      int64_t area = 0;
      for (const Run& run_ : r.runs) area += run_.ce - run_.cb + 1;
      r.full_domain = area == im.width * im.height;
      if (r.full_domain) r.runs.clear();
      o->items.push_back(std::move(r));
    }
    *ImageReduced = guard.release();
  });
}

MvStatus mv_get_domain(MvObject Image, MvObject* Domain) {
  return run("get_domain", [&] {
    require_iconic(Image, "Image");
    require_output(Domain, "Domain");
    require_kind(Image, true);
    MvObject o = new_object();
    for (const Iconic& im : Image->items) {
      Iconic r;
      if (im.full_domain)
        for (int64_t row = 0; row < im.height; ++row) r.runs.push_back({row, 0, im.width - 1});
      else
        r.runs = im.runs;
      o->items.push_back(std::move(r));
    }
    *Domain = o;
  });
}

// ------------------------------------------------------------------ errors
// src/c_api/error_state.cpp:119-131: views of this thread's error state
MvStatus mv_get_last_error(MvStringView* error) {
  if (!error) return MV_STATUS_INVALID_ARGUMENT;
  const std::string& text = error_text();
  error->data = text.data();
  error->size = text.size();
  return MV_STATUS_OK;
}

MvStatus mv_get_last_error_info(MvErrorInfo* error) {
  if (!error) return MV_STATUS_INVALID_ARGUMENT;
  *error = error_info();
  return MV_STATUS_OK;
}

}  // extern "C"
