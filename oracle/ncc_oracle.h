/* Test infrastructure only: FP64 CPU restatement of the reference mvkit NCC
 * matching path (src/ncc_matching/model.cpp, src/ncc_matching/matcher.cpp,
 * scalar build, no caches).  Used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  Pinned against the reference
 * compiled from its own sources (oracle/Makefile `ref`) and the fixtures in
 * tests/golden/.  The product never links or loads this library. */
#ifndef MVKIT_GB300_NCC_ORACLE_H
#define MVKIT_GB300_NCC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* pixel type: 0 = uint8, 1 = uint16.  mask: width*height bytes or NULL (full
 * domain).  levels 0 = automatic.  angle_step 0 = automatic.  Returns an
 * MvStatus-compatible code (0 ok, <0 error) and fills err. */
int orc_create(const void* pixels, int type, int64_t width, int64_t height, int64_t stride,
               const uint8_t* mask, int levels, double angle_start, double angle_extent,
               double angle_step, int ignore_polarity, void** model, char* err, int errlen);
void orc_free(void* model);
void orc_model_info(void* model, double* info);
void orc_level(void* model, int level, int64_t* dims, double* origin);
int64_t orc_patch(void* model, int level, int index, int32_t* rows, int32_t* cols, double* weights,
                  int64_t capacity, double* meta);

/* stage: -1 final matches (after greedy selection and refinement);
 *         0 coarse candidates after NMS;
 *         k>=1 candidates after the k-th coarse-to-fine tracking step;
 *         100 candidates after the full-resolution score, sorted.
 * out holds capacity x 4 doubles (row, column, angle, score), matcher-internal
 * pixel-centre convention; *count is the full list length. */
int orc_find(void* model, const void* image, int type, int64_t width, int64_t height, int64_t stride,
             const uint8_t* domain, double angle_start, double angle_extent, double min_score,
             int64_t num_matches, double max_overlap, int subpixel, int highest, int lowest,
             int stage, double* out, int64_t capacity, int64_t* count, char* err, int errlen);

/* Search pyramid level `level` as the matcher holds it (FP64 values
 * pixel/4^k-sums minus the crop DC), for a model/query pair.  geom[0..5] =
 * width, height, crop_row, crop_column, dc, level_count. */
int orc_pyramid(void* model, const void* image, int type, int64_t width, int64_t height,
                int64_t stride, int highest, int level, double* out, int64_t capacity,
                double* geom, char* err, int errlen);

/* Budgets of the following calls (process-wide): model raster samples,
 * search-image pixels, coarse candidates; 0 = the reference's (16 000 000,
 * 32 000 000, 10 000).  Lifted, they check the library's extended mode. */
void orc_set_budgets(int64_t samples, int64_t pixels, int64_t candidates);

/* Batch of independent finds over `n` images on `threads` host threads (one
 * image per thread at a time); returns the number of matches summed. */
int64_t orc_find_many(void* model, const void* const* images, int type, int64_t width,
                      int64_t height, int64_t stride, int n, int threads, double angle_start,
                      double angle_extent, double min_score, int64_t num_matches,
                      double max_overlap, int subpixel, int highest, int lowest);

#ifdef __cplusplus
}
#endif
#endif
