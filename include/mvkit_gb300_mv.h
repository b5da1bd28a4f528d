/* GB300 NCC matching: the reference's own C signatures (libmvkit_gb300_mv.so).
 *
 * A program written against mvkit's C API for NCC matching
 * (include/mvkit/c/mv_ncc_matching.h of the reference) compiles against this
 * header and links against libmvkit_gb300_mv.so unchanged: the operators
 * below have the reference's names, argument order and types, tuple
 * semantics, status codes and error texts, and run the search on the GPU
 * through libmvkit_gb300.so (include/mvkit_gb300_ncc.h).
 *
 * The library carries a minimal tuple / iconic-object layer of its own with
 * the reference's public signatures (the subset a caller of these operators
 * needs: tuples, handles, single-channel images, rectangle regions and
 * reduced domains, error state).  The operators read their inputs only
 * through that public layer (mv_get_*, mv_length_tuple, mv_count_obj,
 * mv_get_image_pointer1, mv_get_domain, mv_get_region_runs); only the model
 * handle is created by a private call of this library.
 *
 * Type names and constants are the reference's (include/mvkit/c/mv_status.h,
 * mv_string.h, mv_value.h, mv_tuple.h, mv_iconic.h, mv_api.h): a caller's
 * code uses the same identifiers. */
#ifndef MVKIT_GB300_MV_H
#define MVKIT_GB300_MV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MV_API __attribute__((visibility("default")))
#else
#define MV_API
#endif

/* include/mvkit/c/mv_status.h:12-24 */
typedef int32_t MvStatus;
#define MV_STATUS_OK ((int32_t)0)
#define MV_STATUS_INVALID_ARGUMENT ((int32_t)-1)
#define MV_STATUS_OUT_OF_RANGE ((int32_t)-2)
#define MV_STATUS_TYPE_MISMATCH ((int32_t)-3)
#define MV_STATUS_NOT_FOUND ((int32_t)-4)
#define MV_STATUS_OUT_OF_MEMORY ((int32_t)-5)
#define MV_STATUS_UNSUPPORTED ((int32_t)-6)
#define MV_STATUS_INVALID_STATE ((int32_t)-7)
#define MV_STATUS_IO_ERROR ((int32_t)-100)
#define MV_STATUS_DECODE_ERROR ((int32_t)-101)
#define MV_STATUS_ENCODE_ERROR ((int32_t)-102)
#define MV_STATUS_LIMIT_EXCEEDED ((int32_t)-103)
#define MV_STATUS_INTERNAL_ERROR ((int32_t)-1000)

/* include/mvkit/c/mv_string.h: a borrowed UTF-8 view (not NUL-terminated) */
typedef struct MvStringView {
  const char* data;
  size_t size;
} MvStringView;

/* include/mvkit/c/mv_value.h */
typedef struct MvHandleImpl* MvHandle;
typedef int32_t MvValueKind;
#define MV_VALUE_EMPTY ((int32_t)0)
#define MV_VALUE_INT64 ((int32_t)1)
#define MV_VALUE_REAL64 ((int32_t)2)
#define MV_VALUE_STRING ((int32_t)4)
#define MV_VALUE_HANDLE ((int32_t)16)

/* include/mvkit/c/mv_tuple.h, mv_iconic.h: opaque owned objects */
typedef struct MvTupleImpl* MvTuple;
typedef struct MvObjectImpl* MvObject;

/* include/mvkit/c/mv_handle.h: handle type of an NCC model */
typedef uint64_t MvObjectType;
#define MV_OBJECT_TYPE_NCC_MODEL ((uint64_t)9)

/* include/mvkit/c/mv_api.h:37-58: structured error of the last failed call */
typedef int32_t MvErrorCode;
#define MV_ERROR_UNSPECIFIED ((int32_t)0)
#define MV_ERROR_NULL_ARGUMENT ((int32_t)1)
#define MV_ERROR_INVALID_CARDINALITY ((int32_t)2)
#define MV_ERROR_INVALID_TYPE ((int32_t)3)
#define MV_ERROR_INVALID_VALUE ((int32_t)4)
#define MV_ERROR_INDEX_OUT_OF_RANGE ((int32_t)5)
#define MV_ERROR_MISSING_ITEM ((int32_t)6)
#define MV_ERROR_UNSUPPORTED_VALUE ((int32_t)7)
#define MV_ERROR_INVALID_OBJECT_STATE ((int32_t)8)
#define MV_ERROR_IO_FAILURE ((int32_t)9)
#define MV_ERROR_INTERNAL_FAILURE ((int32_t)10)
#define MV_ERROR_PARAMETER_INDEX_NONE ((int64_t)-1)

typedef struct MvErrorInfo {
  MvStatus status;
  MvErrorCode code;
  MvStringView operation;
  MvStringView parameter;
  int64_t parameter_index;
  MvStringView message;
} MvErrorInfo;

/* ------------------------------------------------------------ NCC operators
 * Controls are tuples, as in the reference (src/c_api/ncc_matching_api.cpp):
 * NumLevels "auto" or 0..16 and AngleStep "auto" or [0, pi/16] at creation;
 * AngleStart finite, AngleExtent [0, 2 pi], MinScore and MaxOverlap [0, 1],
 * NumMatches an integer >= 0 (0 = all), SubPixel "true"/"false", NumLevels
 * the highest level or a [highest, lowest] pair at search.  Output tuples are
 * new and owned by the caller (mv_destroy_tuple); they are written only when
 * the call succeeds.  The search runs on the current CUDA device. */

/* mv_create_ncc_model: include/mvkit/c/mv_ncc_matching.h:30-32.  The
 * template image's domain (mv_reduce_domain) is the model's ROI. */
MV_API MvStatus mv_create_ncc_model(MvObject Template, MvTuple NumLevels, MvTuple AngleStart, MvTuple AngleExtent,
                                    MvTuple AngleStep, MvTuple Metric, MvTuple* ModelID);

/* mv_get_ncc_model_params: include/mvkit/c/mv_ncc_matching.h:46-47 */
MV_API MvStatus mv_get_ncc_model_params(MvTuple ModelID, MvTuple* NumLevels, MvTuple* AngleStart,
                                        MvTuple* AngleExtent, MvTuple* AngleStep, MvTuple* Metric);

/* mv_find_ncc_model: include/mvkit/c/mv_ncc_matching.h:71-74.  The search
 * image's domain restricts the poses; an empty image object gives empty
 * outputs. */
MV_API MvStatus mv_find_ncc_model(MvObject Image, MvTuple ModelID, MvTuple AngleStart, MvTuple AngleExtent,
                                  MvTuple MinScore, MvTuple NumMatches, MvTuple MaxOverlap, MvTuple SubPixel,
                                  MvTuple NumLevels, MvTuple* Row, MvTuple* Column, MvTuple* Angle,
                                  MvTuple* Score);

/* mv_write_ncc_model / mv_read_ncc_model: include/mvkit/c/mv_ncc_matching.h:84,94
 * ("MVKIT_NCC 1" files, byte-identical to the reference's) */
MV_API MvStatus mv_write_ncc_model(MvTuple ModelID, MvTuple FileName);
MV_API MvStatus mv_read_ncc_model(MvTuple FileName, MvTuple* ModelID);

/* mv_find_ncc_models: include/mvkit/c/mv_ncc_matching.h:119-123.  Controls
 * one value or one per model; Model receives the 0-based model index. */
MV_API MvStatus mv_find_ncc_models(MvObject Image, MvTuple ModelIDs, MvTuple AngleStart, MvTuple AngleExtent,
                                   MvTuple MinScore, MvTuple NumMatches, MvTuple MaxOverlap, MvTuple SubPixel,
                                   MvTuple NumLevels, MvTuple* Row, MvTuple* Column, MvTuple* Angle,
                                   MvTuple* Score, MvTuple* Model);

/* ---------------------------------------------------------------- tuples
 * include/mvkit/c/mv_tuple.h.  mv_create_tuple makes `length` empty values;
 * mv_set_* replace the value at an existing index; mv_get_d reads integer
 * and real values, mv_get_i integers only; mv_get_s returns a view owned by
 * the tuple; mv_get_h a handle borrowed from the tuple. */
MV_API MvStatus mv_create_tuple(MvTuple* tuple, size_t length);
MV_API MvStatus mv_copy_tuple(MvTuple tuple, MvTuple* clone);
MV_API MvStatus mv_destroy_tuple(MvTuple tuple);
MV_API MvStatus mv_length_tuple(MvTuple tuple, size_t* size);
MV_API MvStatus mv_resize_tuple(MvTuple tuple, size_t length);
MV_API MvStatus mv_get_type(MvTuple tuple, size_t index, MvValueKind* kind);
MV_API MvStatus mv_get_i(MvTuple tuple, size_t index, int64_t* value);
MV_API MvStatus mv_get_d(MvTuple tuple, size_t index, double* value);
MV_API MvStatus mv_get_s(MvTuple tuple, size_t index, MvStringView* value);
MV_API MvStatus mv_get_h(MvTuple tuple, size_t index, MvHandle* handle);
MV_API MvStatus mv_set_i(MvTuple tuple, int64_t value, size_t index);
MV_API MvStatus mv_set_d(MvTuple tuple, double value, size_t index);
MV_API MvStatus mv_set_s(MvTuple tuple, MvStringView value, size_t index);
MV_API MvStatus mv_set_h(MvTuple tuple, MvHandle value, size_t index);

/* mv_clear_handle (include/mvkit/c/mv_handle.h): releases the objects of
 * every handle in the tuple now; later uses see an empty handle. */
MV_API MvStatus mv_clear_handle(MvTuple Handle);

/* ---------------------------------------------------------- iconic objects
 * include/mvkit/c/mv_iconic.h, mv_image.h, mv_region.h,
 * mv_image_processing.h.  Images are single channel ("byte", "uint2",
 * "int2", "int4", "real"; the NCC operators take "byte" and "uint2"),
 * copied in by mv_gen_image1 with a full domain. */
MV_API MvStatus mv_gen_empty_obj(MvObject* objects);
MV_API MvStatus mv_clear_obj(MvObject objects);
MV_API MvStatus mv_count_obj(MvObject objects, MvTuple* count);
MV_API MvStatus mv_gen_image_const(MvObject* Image, MvTuple Type, MvTuple Width, MvTuple Height);
MV_API MvStatus mv_gen_image1(MvObject* Image, MvTuple Type, MvTuple Width, MvTuple Height, MvTuple PixelPointer);
MV_API MvStatus mv_get_image_pointer1(MvObject Image, MvTuple* Pointer, MvTuple* Type, MvTuple* Width,
                                      MvTuple* Height);
MV_API MvStatus mv_get_image_size(MvObject Image, MvTuple* Width, MvTuple* Height);
MV_API MvStatus mv_get_image_type(MvObject Image, MvTuple* Type);
/* Rectangle with corners rounded to pixels, rows Row1..Row2 and columns
 * Column1..Column2 inclusive (empty when a corner pair is reversed). */
MV_API MvStatus mv_gen_rectangle1(MvObject* Rectangle, MvTuple Row1, MvTuple Column1, MvTuple Row2,
                                  MvTuple Column2);
/* Runs of one region: row, first and last column of each. */
MV_API MvStatus mv_get_region_runs(MvObject Region, MvTuple* Row, MvTuple* ColumnBegin, MvTuple* ColumnEnd);
/* The image with its domain set to the first region clipped to the image. */
MV_API MvStatus mv_reduce_domain(MvObject Image, MvObject Region, MvObject* ImageReduced);
MV_API MvStatus mv_get_domain(MvObject Image, MvObject* Domain);

/* ---------------------------------------------------------------- errors
 * include/mvkit/c/mv_api.h:75,87.  Thread-local, valid until this thread's
 * next call of this library; "operation: message" for mv_get_last_error. */
MV_API MvStatus mv_get_last_error(MvStringView* error);
MV_API MvStatus mv_get_last_error_info(MvErrorInfo* error);

#ifdef __cplusplus
}
#endif
#endif
