// Launch interface of the find kernels (ncc_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ncc_types.h"

namespace mvg {

// Integer-valued pyramid levels held as float (exact: every level value is an
// integer sum of 4^k input pixels, < 2^24).  Level 0 is the crop itself.
struct LevelImage {
  float* v = nullptr;
  int w = 0, h = 0;
  // row prefix moments of the level: (w+1) x h pairs {sum S, sum S^2}
  longlong2* prefix = nullptr;
};

// Valid-position interval of a patch on a level: the intersection of the
// raster-inside-image bounds and the domain test of its pose.
struct PosRange {
  int r0, r1, c0, c1;  // half-open [r0, r1) x [c0, c1)
};

struct CoarseArgs {
  LevelImage lev;
  LevelView view;
  const int32_t* plist;     // kept coarse patches (indices into view.patches)
  const PosRange* ranges;   // per kept coarse patch
  int nplist;
  float* planes;            // nplist x h x w scores
  int absolute;
};

struct NmsArgs {
  const float* planes;
  int nplist, w, h;
  const int32_t* plist;
  LevelView view;
  double crop_row, crop_col, scale, phase;
  float threshold;          // smallest float f with double(f) >= 0.4 * MinScore
  Cand* out;
  QueryState* state;
  int max_candidates;
};

struct TrackArgs {
  LevelImage lev;           // target level t
  LevelView view;
  const int32_t* plist;     // query patches of level t, reference iteration order
  const PosRange* ranges;   // per plist entry
  int nplist;
  // patches of level t inside the angle window of each source patch of level
  // t+1, as plist entries in reference order (CSR by source patch index)
  const int32_t* sel_off;
  const int32_t* sel_idx;
  const Cand* in;
  Cand* out;
  QueryState* state;
  int in_slot;              // state->count index holding the input count
  double crop_row, crop_col, step, offset;
  int exact32;              // lattice arithmetic is exact in FP32 (host-checked)
  int absolute;
  int staged_ok;            // set by the launcher: dynamic shared memory holds the window
};

struct DedupArgs {
  const Cand* in;
  Cand* out;
  int* table;
  QueryState* state;
  int in_slot, out_slot;
  double threshold;         // drop score < threshold; -inf keeps all finite
  int snap;                 // 1: snap poses outside the image into it first
  double height, width;     // image size for the snap (full domain)
};

struct ImageView {
  const float* v;           // finest level (float of pixel sums)
  int w, h;
};

struct ScoreArgs {
  ImageView img;
  OriginalView orig;
  Cand* cand;
  const QueryState* state;
  int slot;
  double crop_row, crop_col, scale, phase;
  int absolute;
};

struct SortArgs {
  const Cand* in;
  Cand* out;
  QueryState* state;
  int slot;
};

// Level-0 model rectangle about the origin: [left, right] x [top, bottom]
// (src/ncc_matching/matcher.cpp:257-258).
struct RectGeom {
  double left, right, top, bottom, area;
};

// Refinement / selection
struct SelectArgs {
  const Cand* sorted;
  const RectAux* aux;       // per sorted candidate
  Refined* refined;         // per sorted index
  int32_t* refined_flag;    // 0 none, 1 queued, 2 done
  int32_t* batch;           // indices to refine next
  Cand* accepted;
  RectAux* accepted_aux;
  int32_t* tested;          // per sorted candidate: accepted matches it was tested against
  uint8_t* sup;             // per sorted candidate: suppressed by an accepted match
  QueryState* state;
  int batch_limit;
  int64_t num_matches;
  double max_overlap;
  RectGeom geom;
};

struct RefineArgs {
  ImageView img;            // finest level
  OriginalView orig;
  LevelImage lev0;          // level 0 (for the discrete recovery search)
  LevelView view0;          // level 0 patches
  const int32_t* plist0;    // query patches of level 0 in reference order
  const PosRange* ranges0;
  int nplist0;
  const Cand* sorted;
  Refined* refined;
  int32_t* refined_flag;
  const int32_t* batch;
  const QueryState* state;
  double crop_row, crop_col, scale, phase;
  double angle_start, angle_end, angle_step, min_score;
  int rotate, subpixel, absolute, top, finest;
  double height, width;     // full image (domain test)
  RectGeom geom;
};

cudaError_t launch_pyramid0(const void* src, int type, int64_t pitch_elems, int crop_row, int crop_col, LevelImage dst,
                            int32_t* error_flag, cudaStream_t s);
cudaError_t launch_pyramid(const LevelImage& src, LevelImage dst, int32_t* error_flag, cudaStream_t s);
cudaError_t launch_prefix(const LevelImage& lev, cudaStream_t s);
cudaError_t launch_coarse(const CoarseArgs& a, int max_bh, int max_bw, cudaStream_t s, size_t smem_limit);
cudaError_t launch_nms(const NmsArgs& a, cudaStream_t s);
cudaError_t launch_track(const TrackArgs& a, int max_candidates, cudaStream_t s, size_t smem_limit);
cudaError_t launch_dedup(const DedupArgs& a, int max_candidates, cudaStream_t s);
cudaError_t launch_score(const ScoreArgs& a, int max_candidates, cudaStream_t s);
cudaError_t launch_sort(const SortArgs& a, cudaStream_t s);
cudaError_t launch_rects(const Cand* sorted, RectAux* aux, const QueryState* state, RectGeom g, int max_candidates,
                         cudaStream_t s);
cudaError_t launch_select(const SelectArgs& a, cudaStream_t s);
cudaError_t launch_refine(const RefineArgs& a, int batch_limit, cudaStream_t s);

}  // namespace mvg
