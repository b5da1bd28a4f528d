// Private side of the reference-signature C layer (include/mvkit_gb300_mv.h):
// the structured error every mv_* call reports, the control-tuple reader the
// operators use, and the model-handle calls that are not part of the public
// signatures.  Semantics follow the reference's C layer
// (src/c_api/tuple_input.hpp, error_state.cpp, control_operator_outputs.hpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mvkit_gb300_mv.h"

namespace mvg::mv {

// A failed mv_* call: status, error code, parameter and index as the
// reference's core::Exception carries them.
struct Failure {
  MvStatus status;
  MvErrorCode code;
  std::string parameter;
  int64_t index;
  std::string message;
  std::string operation = {};  // empty: the failing operator's name
};

[[noreturn]] void fail(MvStatus status, MvErrorCode code, const std::string& parameter, int64_t index,
                       const std::string& message);

// Runs fn as the reference's translate() does: success clears the thread's
// error, a Failure (or any exception) becomes the returned status and the
// thread's error with `operation`.
template <class Fn> MvStatus run(const char* operation, Fn&& fn) noexcept;
void set_error(MvStatus status, const char* operation, const Failure& f) noexcept;
void clear_error() noexcept;
const std::string& error_text() noexcept;
MvErrorInfo error_info() noexcept;

template <class Fn> MvStatus run(const char* operation, Fn&& fn) noexcept {
  try {
    fn();
    clear_error();
    return MV_STATUS_OK;
  } catch (const Failure& f) {
    set_error(f.status, f.operation.empty() ? operation : f.operation.c_str(), f);
    return f.status;
  } catch (const std::bad_alloc&) {
    set_error(MV_STATUS_OUT_OF_MEMORY, "", Failure{MV_STATUS_OUT_OF_MEMORY, MV_ERROR_INTERNAL_FAILURE, "", -1,
                                                     "out of memory"});
    return MV_STATUS_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_error(MV_STATUS_INTERNAL_ERROR, "",
              Failure{MV_STATUS_INTERNAL_ERROR, MV_ERROR_INTERNAL_FAILURE, "", -1, e.what()});
    return MV_STATUS_INTERNAL_ERROR;
  } catch (...) {
    set_error(MV_STATUS_INTERNAL_ERROR, "",
              Failure{MV_STATUS_INTERNAL_ERROR, MV_ERROR_INTERNAL_FAILURE, "", -1, "unknown internal error"});
    return MV_STATUS_INTERNAL_ERROR;
  }
}

// Read-only view of one control tuple of an operator (a null tuple reads as
// empty), through the public tuple calls only.  Failures carry the
// operator's parameter name; a type error is TypeMismatch, anything else
// InvalidArgument (tuple_input.hpp:184-188).
class Control {
 public:
  Control(MvTuple t, const char* parameter);
  size_t size() const { return n_; }
  MvValueKind kind(size_t i) const;
  double number(size_t i) const;        // int64 or real64
  int64_t integer(size_t i) const;      // int64 only
  std::string string(size_t i) const;   // string only
  MvHandle handle(size_t i) const;      // handle only
  double scalar_number() const;         // exactly one, finite
  int64_t scalar_integer() const;       // exactly one int64
  [[noreturn]] void fail(MvErrorCode code, int64_t index, const std::string& message) const;

 private:
  void index_check(size_t i) const;
  MvTuple t_;
  size_t n_ = 0;
  std::string parameter_;
};

// New owned output tuples of one operator, written to the caller's pointers
// only by commit() (control_operator_outputs.hpp:7-27): every destination
// must be non-null and distinct.
class Outputs {
 public:
  Outputs(std::initializer_list<MvTuple*> destinations);
  ~Outputs();
  MvTuple operator[](size_t i) const { return values_[i]; }
  void append_d(size_t i, double v);
  void append_i(size_t i, int64_t v);
  void append_s(size_t i, const std::string& v);
  void append_h(size_t i, MvHandle h);
  void commit();

 private:
  std::vector<MvTuple*> dest_;
  std::vector<MvTuple> values_;
};

// Model handles: a handle of type MV_OBJECT_TYPE_NCC_MODEL owning `object`
// (released with `release` when the last tuple drops it or mv_clear_handle
// clears it), and the object of a handle: nullptr when it is of another
// type; a cleared handle of the type fails with InvalidState as the
// reference's control objects do (src/c_api/control_object.hpp:36-40).
MvHandle make_handle(uint64_t type, void* object, void (*release)(void*));
void* handle_object(MvHandle h, uint64_t type);
void drop_handle(MvHandle h);  // the reference make_handle gave the caller

}  // namespace mvg::mv
