/* GB300 NCC matching: C ABI of libmvkit_gb300.so.
 *
 * Drop-in boundary for mvkit's NCC matching operators.  Each entry point
 * takes plain pointers and scalars: the control tuples of the reference
 * operators become one scalar each, the output tuples become caller-owned
 * double arrays.  Status codes are the reference's MvStatus values
 * (include/mvkit/c/mv_status.h:12-24): 0 ok, -1 invalid argument,
 * -3 type mismatch, -5 out of memory, -6 unsupported, -7 invalid state,
 * -100 I/O error, -101 decode error, -103 limit exceeded, -1000 internal
 * error.  On failure the thread-local
 * message of mvg_last_error() says why (reference: mv_get_last_error,
 * include/mvkit/c/mv_api.h:75).  No call throws across the ABI.
 *
 * Pixel types: 0 = byte (uint8), 1 = uint2 (uint16), one channel.
 * Search runs on the current CUDA device; results are synchronous. */
#ifndef MVKIT_GB300_NCC_H
#define MVKIT_GB300_NCC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MVG_API __attribute__((visibility("default")))
#else
#define MVG_API
#endif

typedef struct mvg_ncc_model_s* mvg_ncc_model;

#define MVG_PIXEL_BYTE 0
#define MVG_PIXEL_UINT2 1
#define MVG_METRIC_USE_POLARITY 0
#define MVG_METRIC_IGNORE_GLOBAL_POLARITY 1
#define MVG_MEMORY_HOST 0
#define MVG_MEMORY_DEVICE 1

/* Replaces mv_create_ncc_model (include/mvkit/c/mv_ncc_matching.h:30-32).
 * Template: pixels (row_stride bytes apart); domain: width*height bytes,
 * nonzero = inside the template ROI, NULL = whole image.  num_levels: 0 or
 * -1 = "auto" (both build as many levels as the template allows, as the
 * reference does for 0 and "auto"), else 1..16.  angle_step: 0 or negative
 * = "auto", else (0, pi/16].  metric: MVG_METRIC_*.  *model_id receives an
 * owned handle; free it with mvg_clear_ncc_model. */
MVG_API int32_t mvg_create_ncc_model(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                             int64_t row_stride, const uint8_t* domain, int32_t num_levels,
                             double angle_start, double angle_extent, double angle_step, int32_t metric,
                             mvg_ncc_model* model_id);

/* One FP64 raster of a model, as the model build made it
 * (the Patch of src/ncc_matching/model.hpp:30-43; model.cpp:39-242): level >= 0
 * and index select the rotated raster of that level and trained angle (the
 * reference's order), level < 0 the unrotated level-0 raster.  Fills
 * meta[0..3] = angle, origin row, origin column, weight sum, and *count =
 * samples; rows/cols (sample offsets as the model stores them) and weights
 * are written when count <= capacity.  A model whose rasters were built on
 * the device gets host copies built on the first call. */
MVG_API int32_t mvg_ncc_model_raster(mvg_ncc_model model_id, int32_t level, int32_t index, int32_t* rows,
                                     int32_t* cols, double* weights, int64_t capacity, double* meta,
                                     int64_t* count);

/* Replaces mv_get_ncc_model_params (include/mvkit/c/mv_ncc_matching.h:46-47).
 * angle_step is 0 for a model without angle range, as the reference reports. */
MVG_API int32_t mvg_get_ncc_model_params(mvg_ncc_model model_id, int32_t* num_levels, double* angle_start,
                                 double* angle_extent, double* angle_step, int32_t* metric);

/* Replaces mv_write_ncc_model (include/mvkit/c/mv_ncc_matching.h:84;
 * src/ncc_matching/persist.cpp:33-43,78-80).  Writes the reference's
 * "MVKIT_NCC 1" text file (FNV-1a 64 checksum), byte-identical to what the
 * reference writes for the same model.  file_name: UTF-8, nonempty. */
MVG_API int32_t mvg_write_ncc_model(mvg_ncc_model model_id, const char* file_name);

/* Replaces mv_read_ncc_model (include/mvkit/c/mv_ncc_matching.h:94;
 * src/ncc_matching/persist.cpp:44-83).  Reads a model file written by the
 * reference or by mvg_write_ncc_model and rebuilds the model; statuses as
 * the reference: IoError (-100), DecodeError (-101), Unsupported (-6) for
 * another format version, LimitExceeded (-103). */
MVG_API int32_t mvg_read_ncc_model(const char* file_name, mvg_ncc_model* model_id);

/* In-memory forms of the two calls above: the file bytes.  serialize
 * stores the byte count in *size and copies min(size, capacity) bytes to
 * buffer (buffer may be NULL to query the size). */
MVG_API int32_t mvg_serialize_ncc_model(mvg_ncc_model model_id, char* buffer, int64_t capacity, int64_t* size);
MVG_API int32_t mvg_deserialize_ncc_model(const char* bytes, int64_t size, mvg_ncc_model* model_id);

/* Where models are built (create and read): 0 (default) = the rotated
 * rasters on the current CUDA device when one is present, straight into the
 * find tables; 1 = on the host in FP64 (the reference's CPU order).  Both
 * give the same weights bit for bit; a process without a CUDA device builds
 * on the host. */
MVG_API int32_t mvg_set_model_build(int32_t where);

/* Extended mode: budgets of the calling thread's model builds and finds
 * (batched calls pass them to their workers).  The defaults (0) are the
 * reference's, and a model or search beyond one fails with
 * MV_STATUS_LIMIT_EXCEEDED as the reference's does: samples = rotated-raster
 * samples of a model, 16 000 000 (src/ncc_matching/model.cpp:15,237);
 * pixels = pixels of a search image, 32 000 000 (matcher.cpp:373-374);
 * candidates = coarse candidates of a find, 10 000 (model.hpp:21,
 * matcher.cpp:591).  Raising them lets templates of 160^2 and more over a
 * full circle, images such as 8192 x 8192, and searches with more coarse
 * candidates run where the reference refuses them; searches within the
 * default budgets give the same results either way.  Limits: samples <=
 * 2^31 - 1, pixels <= 2^30, candidates <= 2^21.  Device memory of a find grows
 * with its candidate budget (about 1.7 KB per candidate on the tensor-core
 * path).  A model keeps the sample
 * budget it was built with. */
MVG_API int32_t mvg_set_budgets(int64_t samples, int64_t pixels, int32_t candidates);
MVG_API int32_t mvg_get_budgets(int64_t* samples, int64_t* pixels, int32_t* candidates);

/* Test hook for the bounded waits of the tensor-core kernel (calling
 * thread's finds): on = 1 makes the kernel load no weights, so the MMA
 * thread's mbarrier wait runs out after one second, the kernel sets the
 * device error flag and leaves, and the find returns Internal (-1000); the
 * context stays usable.  on = 0 restores normal operation. */
MVG_API int32_t mvg_test_withhold_tensor_weights(int32_t on);

/* FNV-1a 64 digest of a model's find tables (patch descriptors, angles,
 * sample, weight and run tables of every level, trained patches only):
 * equal digests mean bit-identical tables.  Uploads the tables first. */
MVG_API int32_t mvg_ncc_model_tables_digest(mvg_ncc_model model_id, uint64_t* digest);

/* Releases a model (the reference frees it with the handle tuple,
 * mv_destroy_tuple; include/mvkit/c/mv_ncc_matching.h:64-67). */
MVG_API int32_t mvg_clear_ncc_model(mvg_ncc_model model_id);

/* Replaces mv_find_ncc_model (include/mvkit/c/mv_ncc_matching.h:71-74).
 * pixels: host memory (location MVG_MEMORY_HOST; copied to the device
 * inside the call) or device memory (MVG_MEMORY_DEVICE).  Controls as the
 * reference's tuples: angle_start/angle_extent in radians, min_score and
 * max_overlap in [0, 1], num_matches >= 0 (0 = all), subpixel 0/1
 * ("false"/"true"), highest_level >= 0 (0 = all model levels), lowest_level
 * >= 1 (the reference's [highest, lowest] NumLevels pair; pass 1 for a
 * single NumLevels value).  Outputs row/column/angle/score (capacity
 * entries each) in the operator's convention (edge-centred translation,
 * src/c_api/ncc_matching_api.cpp:171-176); *count receives the number of
 * matches (entries beyond capacity are dropped).  stream: a cudaStream_t or
 * NULL for the library's per-thread stream.  domain: the search image's
 * domain (the reference image object's reduced domain, image.domain() in
 * src/ncc_matching/matcher.cpp:375-393) as width x height bytes in host
 * memory, nonzero inside, or NULL for the whole image; only poses whose
 * nearest pixel lies in it are returned. */
MVG_API int32_t mvg_find_ncc_model(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                           int64_t row_stride, int32_t location, const uint8_t* domain, mvg_ncc_model model_id,
                           double angle_start, double angle_extent, double min_score, int64_t num_matches,
                           double max_overlap, int32_t subpixel, int32_t highest_level, int32_t lowest_level,
                           double* row, double* column, double* angle, double* score, int64_t capacity,
                           int64_t* count, void* stream);

/* Replaces mv_find_ncc_models (include/mvkit/c/mv_ncc_matching.h:119-123;
 * src/c_api/ncc_matching_api.cpp:191-201 over
 * mv::ncc_matching::find_models, src/ncc_matching/matcher.cpp:1077-1124).
 * Searches one image for num_models (1..4096) models.  Each control is an
 * array with its value count, as the reference's tuples: one value shared by
 * all models or one per model; num_levels holds 1 (highest), 2 (highest,
 * lowest), num_models (highest per model) or 2*num_models (pairs) values.
 * subpixel values are 0/1.  A shared NumMatches / MaxOverlap (one value) is a
 * limit / suppression over all models; per-model values apply per model,
 * and with a shared MaxOverlap the per-model quotas are applied before the
 * cross-model suppression (HALCON's rule, as the reference).  domain as
 * for mvg_find_ncc_model.  Outputs as mvg_find_ncc_model plus model[i], the
 * index into model_ids. */
MVG_API int32_t mvg_find_ncc_models(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                    int64_t row_stride, int32_t location, const uint8_t* domain,
                                    const mvg_ncc_model* model_ids,
                                    int64_t num_models, const double* angle_start, int64_t n_angle_start,
                                    const double* angle_extent, int64_t n_angle_extent, const double* min_score,
                                    int64_t n_min_score, const int64_t* num_matches, int64_t n_num_matches,
                                    const double* max_overlap, int64_t n_max_overlap, const int32_t* subpixel,
                                    int64_t n_subpixel, const int32_t* num_levels, int64_t n_num_levels,
                                    double* row, double* column, double* angle, double* score, int64_t* model,
                                    int64_t capacity, int64_t* count, void* stream);

/* Batched FindNccModels (no reference counterpart: a caller of the
 * reference loops over its images, one mv_find_ncc_models call each,
 * src/c_api/ncc_matching_api.cpp:191-201).  Searches num_images images for
 * the same models and controls as mvg_find_ncc_models, on `workers` (1..256)
 * host threads of the library, each with its own stream and workspace, so
 * several finds are in flight on the GPU.  Image i is images[i],
 * pixel_types[i], widths[i], heights[i], row_strides[i] (location shared:
 * all in host or all in device memory); domains is NULL or holds one mask
 * pointer (or NULL) per image.  Each image's result equals that of
 * mvg_find_ncc_models on it.  Matches are written image after image:
 * image i's occupy [image_offsets[i], image_offsets[i + 1]) (num_images + 1
 * entries) of row/column/angle/score/model, entries past capacity dropped;
 * *count receives the total.  statuses[i] receives image i's status (a
 * failed image has no matches).  Returns 0 when every image succeeded, else
 * the first failed image's status, with "image <i>: <message>" as the last
 * error; the outputs are filled either way.  The calling thread's
 * correlation path (mvg_set_correlation_path) and current device carry over
 * to the workers; its stage profile (mvg_profile_*) does not record the
 * batch's finds.  Concurrent batch calls run one after the other. */
MVG_API int32_t mvg_find_ncc_models_batch(const void* const* images, const int32_t* pixel_types,
                                          const int64_t* widths, const int64_t* heights,
                                          const int64_t* row_strides, int64_t num_images, int32_t location,
                                          const uint8_t* const* domains, const mvg_ncc_model* model_ids,
                                          int64_t num_models, const double* angle_start, int64_t n_angle_start,
                                          const double* angle_extent, int64_t n_angle_extent,
                                          const double* min_score, int64_t n_min_score, const int64_t* num_matches,
                                          int64_t n_num_matches, const double* max_overlap, int64_t n_max_overlap,
                                          const int32_t* subpixel, int64_t n_subpixel, const int32_t* num_levels,
                                          int64_t n_num_levels, int32_t workers, double* row, double* column,
                                          double* angle, double* score, int64_t* model, int64_t capacity,
                                          int64_t* image_offsets, int32_t* statuses, int64_t* count);

/* NCC adjoint with a scale degree of freedom (no counterpart in the rigid
 * reference).  For each of `count` poses (row, column, angle, scale; 4
 * doubles each, the matcher's pixel-centre image coordinates of the model
 * origin, as mvg_find_ncc_model_stage reports them, scale 1 = trained size)
 * it warps the model's unrotated level-0 raster by the similarity
 * transform, samples the image bilinearly and returns the NCC in score[i]
 * and its gradient d score / d (row, column, angle, scale) in
 * gradient[4 i .. 4 i + 3].  A pose with a sample outside the image or a flat
 * window gets score -inf and a zero gradient.  pixels/location as for
 * mvg_find_ncc_model. */
MVG_API int32_t mvg_ncc_score_gradient(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                       int64_t row_stride, int32_t location, mvg_ncc_model model_id,
                                       const double* poses, int64_t count, double* score, double* gradient,
                                       void* stream);

/* Gauss-Newton refinement of `count` similarity poses (row, column, angle,
 * scale; as for mvg_ncc_score_gradient, refined in place) on the NCC above:
 * the reference's refinement step (normal equations of the centred,
 * normalised samples, FP64 solve with partial pivoting, steps clipped to
 * 0.75 px, one trained angle step and 0.01 in scale, up to four halvings, a
 * step only on a strictly higher score) with scale as a fourth parameter;
 * at most `iterations` steps.  score[i]: NCC at the final pose. */
MVG_API int32_t mvg_ncc_refine_similarity(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                          int64_t row_stride, int32_t location, mvg_ncc_model model_id,
                                          double* poses, int64_t count, int32_t iterations, double* score,
                                          void* stream);

/* Candidate list of one internal stage of a find, in the matcher's
 * pixel-centre pose convention (mv::ncc_matching::find,
 * src/ncc_matching/matcher.cpp:1063): stage 0 = coarse candidates after
 * non-maximum suppression; k >= 1 = after the k-th coarse-to-fine tracking
 * step; 100 = scored and sorted full-resolution candidates; -1 = final
 * matches.  out holds capacity x 4 doubles (row, column, angle, score). */
MVG_API int32_t mvg_find_ncc_model_stage(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                 int64_t row_stride, int32_t location, const uint8_t* domain,
                                 mvg_ncc_model model_id,
                                 double angle_start, double angle_extent, double min_score,
                                 int64_t num_matches, double max_overlap, int32_t subpixel,
                                 int32_t highest_level, int32_t lowest_level, int32_t stage, double* out,
                                 int64_t capacity, int64_t* count);

/* Search-pyramid level of an image as the matcher holds it: exact integer
 * sums of 4^level input pixels over the crop the model implies (the
 * reference's FP64 level value is sum/4^level minus the crop's first pixel).
 * geom[0..4] = width, height, crop_row, crop_column, first crop pixel. */
MVG_API int32_t mvg_ncc_pyramid_level(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                              int64_t row_stride, mvg_ncc_model model_id, int32_t highest_level, int32_t level,
                              float* out, int64_t capacity, double* geom);

/* Search-pyramid level `level` of the whole image (sums of 4^level input
 * pixels, the same values as mvg_ncc_pyramid_level) for callers that cannot
 * allocate device memory: frameworks that own every device buffer through
 * their own pool, real-time loops where an allocation may stall, processes
 * with a device-memory budget fixed at start-up.  No counterpart in the
 * reference (its pyramid is an internal step of the find).
 *
 * pixels: the image in device memory of the current device (row_stride
 * bytes apart, aligned to the pixel size); out: a device buffer of the same
 * device, 4-byte aligned, of out_capacity floats that receives the level,
 * row-major, *out_width x *out_height.  A host pointer (pageable or
 * page-locked), a pointer into another device's memory or a misaligned
 * pointer is rejected with MV_STATUS_INVALID_ARGUMENT (-1) before anything
 * is launched; images taller than 524280 rows (the pyramid grid's limit)
 * with MV_STATUS_LIMIT_EXCEEDED.  Level sums at or above 2^24 (uint16 from
 * level 5) are not exact in float: the call returns MV_STATUS_UNSUPPORTED
 * (-6), as mvg_ncc_pyramid_level does.  Allocates nothing: the levels below the
 * requested one are built in one fixed device array of 6 Mi floats (24 MiB)
 * that the library holds on every GPU that loads it until the process exits;
 * images whose lower levels need more than that are rejected with
 * MV_STATUS_LIMIT_EXCEEDED (-103).  The first call on a device looks the
 * array's device address up (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address stays cached
 * for the process's life: after a cudaDeviceReset of a device, do not call
 * this entry point on that device again.  All calls share the
 * array: calls that overlap on the GPU (concurrent streams or threads on one
 * device) race and must be serialised by the caller.  stream: a cudaStream_t
 * or NULL; the call returns when the level is complete. */
MVG_API int32_t mvg_ncc_pyramid_level_noalloc(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                              int64_t row_stride, int32_t level, float* out, int64_t out_capacity,
                                              int64_t* out_width, int64_t* out_height, void* stream);

/* Thread-local message of the last failed call (empty after success). */
MVG_API const char* mvg_last_error(void);

/* Correlation path of the calling thread's finds: 0 (default) scores the
 * rotated patches of the coarse-to-fine tracking on the tensor cores
 * (tcgen05, fp16 halves of exact integer sums, FP32 accumulation) wherever a
 * level's sums allow it; 1 scores everything on the FP32 CUDA cores.  Both
 * return the same matches within the parity tolerances. */
MVG_API int32_t mvg_set_correlation_path(int32_t path);

/* Grid rows of tensor-core weights the calling thread's finds keep in flight
 * ahead of the MMAs (1..64; the weight ring gets at least two chunks of
 * grid rows, the window buffers the rest of shared memory).  A launch-shape
 * setting only: results do not depend on it.  Batch workers take the
 * calling thread's value. */
MVG_API int32_t mvg_set_tc_weight_lookahead(int32_t rows);

/* Per-thread stage profile of finds on this thread: CUDA events recorded on
 * the find's stream around each kernel group while enabled.  Stages 0..12:
 * upload, pyramid, prefix, coarse, nms, track, dedup, score, sort, select,
 * refine, track_tc (the tensor-core correlation kernel), tc_prep (its fp16
 * planes and candidate grouping).  ms: summed event time; launches: kernels launched (counted also
 * while disabled); work: algorithmic multiply-adds (coarse, track) or
 * bilinear taps (score); finds: completed finds since the last reset. */
MVG_API int32_t mvg_profile_enable(int32_t on);
MVG_API int32_t mvg_profile_reset(void);
MVG_API int32_t mvg_profile_read(int32_t stage, const char** name, double* ms, int64_t* launches, double* work,
                                 int64_t* finds);

/* Batched calls (mvg_find_ncc_models_batch) made from this thread can merge
 * the tensor-core correlation launches of their finds in flight.  The
 * workers form `cohorts` groups (worker w in group w mod cohorts; 1..16);
 * each tracking step and coarse scan of a find waits until every worker of
 * its group has reached one, then a single launch per launch shape covers
 * all of their tiles.  cohorts = 0 (default): every find launches its own,
 * which gives the higher throughput on the 2048^2 workload: merged finds move
 * in step and lose the overlap of their other kernels.  Results are the same
 * either way. */
MVG_API int32_t mvg_set_batch_merge(int32_t cohorts);

/* Merged tensor-core launches of batched calls since the last reset (any
 * thread): summed CUDA-event time of the launches on the batcher's stream
 * (ms), their count, the finds' jobs they carried, and the algorithmic and
 * issued multiply-adds of those finds' tensor-core work. */
MVG_API int32_t mvg_batch_profile_reset(void);
MVG_API int32_t mvg_batch_profile_read(double* ms, int64_t* launches, int64_t* jobs, double* macs,
                                       double* issued);

/* Multiply-adds the tensor cores were issued by the profiled finds of this
 * thread (M x N x K of every MMA, padding rows and columns included); the
 * track_tc stage's work is the algorithmic part of it. */
MVG_API int32_t mvg_profile_tensor_issued(double* macs);

/* Page-locked host buffers for zero-staging uploads, and device buffers for
 * callers without their own allocator. */
MVG_API int32_t mvg_host_alloc(size_t bytes, void** ptr);
MVG_API int32_t mvg_host_free(void* ptr);
MVG_API int32_t mvg_device_alloc(size_t bytes, void** ptr);
MVG_API int32_t mvg_device_free(void* ptr);
MVG_API int32_t mvg_copy_to_device(void* dst, const void* src, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
