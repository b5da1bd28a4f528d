// GB300 NCC matching: header-only C++ forms of the reference's free functions
// (include/mvkit/cpp/mv_ncc_matching.hpp:382-482 of the reference; their
// implementation src/cpp_api/ncc_matching.cpp:82-90 forwards to the C ABI the
// same way) over include/mvkit_gb300_mv.h.  A caller of
//   mv::FindNccModel(Image, ModelID, AngleStart, AngleExtent, MinScore,
//                    NumMatches, MaxOverlap, SubPixel, NumLevels,
//                    &Row, &Column, &Angle, &Score)
// compiles unchanged.  MvTuple and MvObject here are small owning wrappers of
// the C handles (the subset of the reference classes these calls need:
// construction from numbers, strings and lists, element access, length);
// failures throw mv::MvException with the C status and message.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <utility>

#include "mvkit_gb300_mv.h"

namespace mv {

class MvException : public std::runtime_error {
 public:
  MvException(MvStatus status, const std::string& message) : std::runtime_error(message), status_(status) {}
  MvStatus Status() const noexcept { return status_; }

 private:
  MvStatus status_;
};

namespace detail {
inline void check(MvStatus status, const char* where) {
  if (status == MV_STATUS_OK) return;
  MvStringView v{nullptr, 0};
  ::mv_get_last_error(&v);
  throw MvException(status, std::string(where) + ": " + std::string(v.data ? v.data : "", v.size));
}
}  // namespace detail

class MvTuple {
 public:
  MvTuple() { detail::check(::mv_create_tuple(&t_, 0), "MvTuple"); }
  MvTuple(int value) : MvTuple(std::int64_t(value)) {}
  MvTuple(std::int64_t value) {
    detail::check(::mv_create_tuple(&t_, 1), "MvTuple");
    detail::check(::mv_set_i(t_, value, 0), "MvTuple");
  }
  MvTuple(double value) {
    detail::check(::mv_create_tuple(&t_, 1), "MvTuple");
    detail::check(::mv_set_d(t_, value, 0), "MvTuple");
  }
  MvTuple(const char* value) : MvTuple(std::string(value)) {}
  MvTuple(const std::string& value) {
    detail::check(::mv_create_tuple(&t_, 1), "MvTuple");
    detail::check(::mv_set_s(t_, MvStringView{value.data(), value.size()}, 0), "MvTuple");
  }
  MvTuple(std::initializer_list<double> values) {
    detail::check(::mv_create_tuple(&t_, values.size()), "MvTuple");
    std::size_t i = 0;
    for (double v : values) detail::check(::mv_set_d(t_, v, i++), "MvTuple");
  }
  MvTuple(std::initializer_list<std::int64_t> values) {
    detail::check(::mv_create_tuple(&t_, values.size()), "MvTuple");
    std::size_t i = 0;
    for (std::int64_t v : values) detail::check(::mv_set_i(t_, v, i++), "MvTuple");
  }
  MvTuple(const MvTuple& o) { detail::check(::mv_copy_tuple(o.t_, &t_), "MvTuple"); }
  MvTuple(MvTuple&& o) noexcept : t_(std::exchange(o.t_, nullptr)) {}
  MvTuple& operator=(MvTuple o) noexcept {
    std::swap(t_, o.t_);
    return *this;
  }
  ~MvTuple() {
    if (t_) ::mv_destroy_tuple(t_);
  }
  // Adopts an owned C tuple (an operator's output).
  static MvTuple Adopt(::MvTuple t) {
    MvTuple r;
    ::mv_destroy_tuple(r.t_);
    r.t_ = t;
    return r;
  }

  std::size_t Length() const {
    std::size_t n = 0;
    detail::check(::mv_length_tuple(t_, &n), "MvTuple::Length");
    return n;
  }
  double D(std::size_t i = 0) const {
    double v = 0;
    detail::check(::mv_get_d(t_, i, &v), "MvTuple::D");
    return v;
  }
  std::int64_t I(std::size_t i = 0) const {
    std::int64_t v = 0;
    detail::check(::mv_get_i(t_, i, &v), "MvTuple::I");
    return v;
  }
  std::string S(std::size_t i = 0) const {
    MvStringView v{nullptr, 0};
    detail::check(::mv_get_s(t_, i, &v), "MvTuple::S");
    return std::string(v.data ? v.data : "", v.size);
  }
  // The C handle, borrowed by a C call (the reference's ControlInput()).
  ::MvTuple ControlInput() const noexcept { return t_; }

 private:
  ::MvTuple t_ = nullptr;
};

class MvObject {
 public:
  MvObject() { detail::check(::mv_gen_empty_obj(&o_), "MvObject"); }
  explicit MvObject(::MvObject o) noexcept : o_(o) {}
  MvObject(const MvObject&) = delete;
  MvObject& operator=(const MvObject&) = delete;
  MvObject(MvObject&& o) noexcept : o_(std::exchange(o.o_, nullptr)) {}
  MvObject& operator=(MvObject&& o) noexcept {
    std::swap(o_, o.o_);
    return *this;
  }
  ~MvObject() {
    if (o_) ::mv_clear_obj(o_);
  }
  ::MvObject NativeHandle() const noexcept { return o_; }

 private:
  ::MvObject o_ = nullptr;
};

// One-channel image copied from `pixels` (mv_gen_image1); type "byte" or "uint2".
inline MvObject GenImage1(const char* type, std::int64_t width, std::int64_t height, const void* pixels) {
  ::MvObject o = nullptr;
  const MvTuple t(type), w(width), h(height), p(std::int64_t(reinterpret_cast<std::uintptr_t>(pixels)));
  detail::check(::mv_gen_image1(&o, t.ControlInput(), w.ControlInput(), h.ControlInput(), p.ControlInput()),
                "GenImage1");
  return MvObject(o);
}

inline void CreateNccModel(const MvObject& Template, const MvTuple& NumLevels, const MvTuple& AngleStart,
                           const MvTuple& AngleExtent, const MvTuple& AngleStep, const MvTuple& Metric,
                           MvTuple* ModelID) {
  ::MvTuple id = nullptr;
  detail::check(::mv_create_ncc_model(Template.NativeHandle(), NumLevels.ControlInput(), AngleStart.ControlInput(),
                                      AngleExtent.ControlInput(), AngleStep.ControlInput(), Metric.ControlInput(),
                                      &id),
                "CreateNccModel");
  *ModelID = MvTuple::Adopt(id);
}

inline void GetNccModelParams(const MvTuple& ModelID, MvTuple* NumLevels, MvTuple* AngleStart, MvTuple* AngleExtent,
                              MvTuple* AngleStep, MvTuple* Metric) {
  ::MvTuple o[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  detail::check(::mv_get_ncc_model_params(ModelID.ControlInput(), &o[0], &o[1], &o[2], &o[3], &o[4]),
                "GetNccModelParams");
  *NumLevels = MvTuple::Adopt(o[0]);
  *AngleStart = MvTuple::Adopt(o[1]);
  *AngleExtent = MvTuple::Adopt(o[2]);
  *AngleStep = MvTuple::Adopt(o[3]);
  *Metric = MvTuple::Adopt(o[4]);
}

inline void FindNccModel(const MvObject& Image, const MvTuple& ModelID, const MvTuple& AngleStart,
                         const MvTuple& AngleExtent, const MvTuple& MinScore, const MvTuple& NumMatches,
                         const MvTuple& MaxOverlap, const MvTuple& SubPixel, const MvTuple& NumLevels, MvTuple* Row,
                         MvTuple* Column, MvTuple* Angle, MvTuple* Score) {
  ::MvTuple o[4] = {nullptr, nullptr, nullptr, nullptr};
  detail::check(::mv_find_ncc_model(Image.NativeHandle(), ModelID.ControlInput(), AngleStart.ControlInput(),
                                    AngleExtent.ControlInput(), MinScore.ControlInput(), NumMatches.ControlInput(),
                                    MaxOverlap.ControlInput(), SubPixel.ControlInput(), NumLevels.ControlInput(),
                                    &o[0], &o[1], &o[2], &o[3]),
                "FindNccModel");
  *Row = MvTuple::Adopt(o[0]);
  *Column = MvTuple::Adopt(o[1]);
  *Angle = MvTuple::Adopt(o[2]);
  *Score = MvTuple::Adopt(o[3]);
}

inline void FindNccModels(const MvObject& Image, const MvTuple& ModelIDs, const MvTuple& AngleStart,
                          const MvTuple& AngleExtent, const MvTuple& MinScore, const MvTuple& NumMatches,
                          const MvTuple& MaxOverlap, const MvTuple& SubPixel, const MvTuple& NumLevels, MvTuple* Row,
                          MvTuple* Column, MvTuple* Angle, MvTuple* Score, MvTuple* Model) {
  ::MvTuple o[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  detail::check(::mv_find_ncc_models(Image.NativeHandle(), ModelIDs.ControlInput(), AngleStart.ControlInput(),
                                     AngleExtent.ControlInput(), MinScore.ControlInput(), NumMatches.ControlInput(),
                                     MaxOverlap.ControlInput(), SubPixel.ControlInput(), NumLevels.ControlInput(),
                                     &o[0], &o[1], &o[2], &o[3], &o[4]),
                "FindNccModels");
  *Row = MvTuple::Adopt(o[0]);
  *Column = MvTuple::Adopt(o[1]);
  *Angle = MvTuple::Adopt(o[2]);
  *Score = MvTuple::Adopt(o[3]);
  *Model = MvTuple::Adopt(o[4]);
}

inline void ReadNccModel(const MvTuple& FileName, MvTuple* ModelID) {
  ::MvTuple id = nullptr;
  detail::check(::mv_read_ncc_model(FileName.ControlInput(), &id), "ReadNccModel");
  *ModelID = MvTuple::Adopt(id);
}

inline void WriteNccModel(const MvTuple& ModelID, const MvTuple& FileName) {
  detail::check(::mv_write_ncc_model(ModelID.ControlInput(), FileName.ControlInput()), "WriteNccModel");
}

}  // namespace mv
