// Launch interface of the find kernels (ncc_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ncc_types.h"

namespace mvg {

struct TcGroup;  // tensor-core group (below)

// Entries of a candidate list that exist: a list's counter keeps counting
// past the cap-entry buffers when the coarse budget overflows (the find then
// ends with LimitExceeded), so readers clamp it.
#ifdef __CUDACC__
__device__ __forceinline__ int live_count(const QueryState* s, int slot) {
  return min(s->count[slot], s->cap);
}
#endif

// Integer-valued pyramid levels held as float (exact: every level value is an
// integer sum of 4^k input pixels, < 2^24).  Level 0 is the crop itself.
struct LevelImage {
  float* v = nullptr;
  int w = 0, h = 0;
  // row prefix moments of the level: (w+1) x h pairs {sum S, sum S^2}, as
  // int64 (prefix) or, when every run sum of S^2 is below 2^32, as uint32
  // modulo 2^32 (prefix32; differences of two entries are then exact)
  longlong2* prefix = nullptr;
  uint2* prefix32 = nullptr;
};

// Valid-position interval of a patch on a level: the intersection of the
// raster-inside-image bounds and the domain test of its pose.
struct PosRange {
  int r0, r1, c0, c1;  // half-open [r0, r1) x [c0, c1)
};

// Reduced search domain (the search image's ROI, image.domain() in the
// reference).  mask == nullptr: the full image, whose bounds the position
// ranges already encode.  Otherwise the position ranges encode the domain's
// bounding box and the kernels test each pose against the mask (one-pixel
// spacing) or, for a sparse domain, the mask's pixel count near the pose.
struct DomainView {
  const uint8_t* mask;      // h x w, nonzero inside (image coordinates)
  const int32_t* count;     // (h + 1) x (w + 1) 2-D prefix counts of mask (sparse domains)
  const int4* runs;         // (row, begin, end, 0) sorted by row and begin
  const int32_t* row_run;   // h + 1: first run of each row
  int w, h;
  int sparse;               // area < 0.7 x bounding-box area (matcher.cpp:505)
  double rmin, rmax, cmin, cmax;  // bounding box
};

struct CoarseArgs {
  LevelImage lev;
  LevelView view;
  const int32_t* plist;     // kept coarse patches (indices into view.patches)
  const PosRange* ranges;   // per kept coarse patch
  int nplist;
  float* planes;            // nplist x h x w scores
  int absolute;
  const uint8_t* skip;      // per kept patch: 1 = plane written by the tensor-core scan (nullable)
  DomainView dom;
  double crop_row, crop_col, scale, phase;
};

// Tensor-core coarse scan: a lattice of pseudo-candidates at stride 5 (each
// covers a 5x5 block of positions) per virtual source (up to 16 kept coarse
// patches), scored by tc_track_kernel; coarse_tc_score_kernel turns the dots
// into score planes.
struct CoarseTcArgs {
  LevelImage lev;
  LevelView view;
  const int32_t* plist;
  const PosRange* ranges;
  int nplist;
  const int32_t* src_of;    // per kept patch: its virtual source (-1: coarse_kernel's)
  const int32_t* k_of;      // per kept patch: index in the virtual source's list
  int lat_r, lat_c;         // lattice blocks per column / row
  const float* dots;        // kTcScoreStride per pseudo-candidate: sum w S
  const TcGroup* groups;    // by virtual source (weff_k for the first-sample shift)
  const int32_t* group_of_src;
  float* planes;
  int absolute;
  DomainView dom;
  double crop_row, crop_col, scale, phase;
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
  int split_off;            // set by the launcher: float offset of the moment-split scratch in
                            // dynamic shared memory (-1: no scratch, moments in one slice)
  // sum w S of the rotated patches of tensor-core groups (nullable),
  // kTcScoreStride per candidate, and their groups (for weff_k)
  const float* tc_dots;
  const int32_t* tc_group_of_src;
  const TcGroup* tc_groups;
  DomainView dom;
};

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes` (never lowers it; safe from several host threads).
cudaError_t reserve_dynamic_smem(const void* kernel, size_t bytes);

// Tensor-core tracking (ncc_tc.cu).  A tile is up to 16 candidates of one
// group (candidates found with the same source patch search the same target
// patches); MMA rows are (candidate, window row offset), MMA columns (grid
// row in the chunk, patch, column placement, weight half); K runs over the
// window columns, and the chunks of grid rows accumulate in tensor memory.
constexpr int kTcMaxP = 16;              // patches of one group (N = 10 P <= 160)
constexpr int kTcCands = 16;             // candidates per tile (M = 16 x 8 rows)
constexpr int kTcScoreStride = 16 * 25;  // dots per candidate: [selected patch][placement]
constexpr int kTcMaxGroups = 4096;       // groups of one tracking step
constexpr int kTcMaxTiles = kMaxCandidatesExt / kTcCands + kTcMaxGroups + 1;
constexpr int kTcMaxStages = 16;         // weight-chunk buffers
constexpr int kTcPlaneShifts = 8;        // column-shifted copies of a level plane
constexpr int kTcMaxParts = 4;           // fp16 parts of a level value (base-64 digits)
constexpr int kTcPlaneMargin = 8;        // plane columns left of the level
constexpr int kTcBlocksPerSm = 1;        // resident tensor-core blocks per SM (512 / this TMEM columns each)

struct TcGroup {
  const uint8_t* b;                      // ceil(kr / rg) chunks: N x K fp16 weights, canonical K-major
  long long macs;                        // algorithmic MACs per candidate (25 x samples of all patches)
  int kr, kw;                            // grid rows; window columns per part (multiple of 16)
  int parts;                             // planes per value (1..4): base-64 digits, the first signed
  int rmin, cmin;                        // grid origin relative to the placement centre
  int p, rg, n;                          // patches; grid rows per chunk (N columns side by side);
                                         // MMA N (10 p rg rounded up to 16)
  int rows_slab;                         // window rows per staged slab (>= 16)
  float inv_scale;                       // 1 / weight scale
  int k_of[kTcMaxP];                     // index in the candidate's selected list
  int r0[kTcMaxP], c0[kTcMaxP];          // first sample offset of each patch
  float weff[kTcMaxP];                   // sum of the fp16 weights / scale
  float ecorr[kTcMaxP];                  // sum over grid rows of the centring row sums / scale
  float weff_k[kTcMaxP];                 // weff by index in the selected list (0: not in the group)
};

struct TcTiles {
  int count;
  int next;                              // unused (tiles are handed out per launch, TcLaunch::next)
  int group[kTcMaxTiles], first[kTcMaxTiles], last[kTcMaxTiles];
};

struct TcArgs {
  LevelImage lev;
  const Cand* in;
  const QueryState* state;
  QueryState* state_rw;                  // MAC counters
  int in_slot;
  const TcGroup* groups;
  const int32_t* group_of_src;           // source patch -> group (-1: CUDA-core path)
  TcTiles* tiles;
  int32_t* order;
  float* dots;                           // kTcScoreStride per candidate: sum w S (consumers
                                         // subtract S0 weff_k, S0 the first sample)
  double crop_row, crop_col, step, offset;
  int exact32;
  int stages;                            // weight-chunk buffers in use
  int stage_bytes, abuf_bytes;           // bytes per weight buffer / per window buffer
  int sets, npad;                        // accumulator sets (grid row y -> set y mod sets), columns per set
  float plane_offset;                    // level value subtracted in the planes (dyn_offset 0)
  int dyn_offset;                        // 1: the offset is the mid-range of the level's values,
                                         // level_mult x (pix_min + pix_max) / 2 from the state
  float level_mult;                      // 4^level (pixels summed into a level value)
  const uint16_t* planes;                // fp16 planes (launch_tc_planes)
  int plane_pitch;                       // elements per plane row
  const int2* rc;                        // candidate lattice positions given directly (nullable)
  int32_t* error;
  int withhold_weights;                  // test hook: load no weights (waits run out, error flag set)
};

// One tensor-core launch: the tiles of `njobs` jobs (a job is one find's
// tracking step or coarse scan, TcArgs in device memory), handed out in job
// order from one counter.  Every job of a launch has the same launch shape
// (stages, stage_bytes, abuf_bytes, sets, npad, dynamic shared memory).
constexpr int kTcMaxJobs = 64;
struct TcLaunch {
  const TcArgs* jobs;  // nullptr: the one job `single`
  int njobs;
  int* next;           // tiles handed out after the first gridDim.x; zero at launch (a job table's:
                       // zeroed by launch_tc_track; a single job's: its tile list's, reset by the planner)
  TcArgs single;
};

// fp16 planes of a level for the tensor-core tracking: parts x 8 shifted
// copies (plane d holds level column x - kTcPlaneMargin + d at x), `pitch`
// columns (a multiple of 8, at least the level width + 8), column-blocked:
// (row y, column x) at ((x / 8) h + y) 8 + x mod 8.
cudaError_t launch_tc_planes(const LevelImage& lev, uint16_t* planes, int pitch, int parts, float offset,
                             cudaStream_t s, const QueryState* state = nullptr, float level_mult = 1.f);
// Range of the level-0 crop into state->pix_min / pix_max (uint16 finds).
cudaError_t launch_level_range(const LevelImage& lev0, QueryState* state, cudaStream_t s);
#ifdef __CUDACC__
// Offset of the fp16 planes of a level: fixed, or (state given) the
// mid-range of the level's values, floor(mult (min + max) / 2) of the level-0
// range; exact in float (below 2^24).
__device__ __forceinline__ float tc_plane_offset(float fixed, const QueryState* state, float mult) {
  if (!state) return fixed;
  const long long s = (long long)(state->pix_min + state->pix_max) * (long long)mult;
  return float(s >> 1);
}
#endif
size_t tc_kernel_static_smem();
// Groups the step's candidates into tiles (counts, tile list, order).
cudaError_t launch_tc_group(const TcArgs& a, int ngroups, int32_t* counts, int32_t* offsets, int32_t* cursor,
                            int max_candidates, cudaStream_t s);
cudaError_t launch_tc_track(const TcLaunch& l, size_t smem, int grid, cudaStream_t s);

// Pseudo-candidates in source order, their lattice centres, the identity
// order and the tile list (16 consecutive candidates of one source per tile).
cudaError_t launch_coarse_lattice(Cand* cand, int2* rc, int nsrc, int nbr, int nbc, const int32_t* group_of_src,
                                  int32_t* order, TcTiles* tiles, QueryState* state, int slot, cudaStream_t s);
cudaError_t launch_coarse_tc_score(const CoarseTcArgs& a, cudaStream_t s);
// (h + 1) x (w + 1) prefix counts of a domain mask (DomainView::count)
cudaError_t launch_domain_count(const uint8_t* mask, int w, int h, int32_t* count, cudaStream_t s);

// half2 pairs (v[x], v[min(x + 1, w - 1)]) of a level whose values are exact
// in fp16, w x h entries.
cudaError_t launch_pairs(const float* v, int w, int h, uint32_t* pairs, cudaStream_t s);

struct DedupArgs {
  const Cand* in;
  Cand* out;
  int* table;
  QueryState* state;
  int in_slot, out_slot;
  double threshold;         // drop score < threshold; -inf keeps all finite
  int snap;                 // 1: snap poses outside the domain into it first
  double height, width;     // image size for the snap (full domain)
  DomainView dom;
  int hash_slots;           // entries of `table`: a power of two >= 3 x the candidate budget
};

struct ImageView {
  const float* v;           // finest level (float of pixel sums)
  int w, h;
  // optional: per pixel the fp16 pair (v[x], v[x+1]) as half2 bits, for
  // levels whose values are exact in fp16 (two loads per bilinear tap)
  const uint32_t* pairs = nullptr;
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

// NCC of the unrotated original raster warped by a similarity pose (row,
// column, angle, scale; pixel-centre image coordinates, the model origin at
// (row, column)) and its gradient in the four parameters.  One block per pose.
struct AdjointArgs {
  ImageView img;            // level 0: the search image as float
  OriginalView orig;
  const double* poses;      // n x 4
  int n;
  double* score;            // n (-inf where a sample leaves the image or the window is flat)
  double* grad;             // n x 4 (0 where the score is -inf)
  int absolute;             // ignore_global_polarity
};

// Gauss-Newton refinement of similarity poses (row, column, angle, scale)
// on the NCC above: the reference's refinement step (3 parameters,
// src/ncc_matching/matcher.cpp:170-240, 903-982) with scale as a fourth.
struct Refine4Args {
  ImageView img;
  OriginalView orig;
  double* poses;            // n x 4, refined in place
  double* score;            // n: score at the final pose (-inf if unscorable)
  int n;
  int iterations;           // Gauss-Newton steps (at most)
  int absolute;
  double max_shift, max_angle, max_scale;  // step limits per iteration
};

// Candidate sort.  Lists of up to kRankSortMax candidates are rank-sorted
// in one launch; longer ones (candidate budgets above it) by a bitonic sort
// of (key, index) pairs in `keys` / `idx` (npow entries each, npow the power
// of two at or above the budget; null when the budget is at most
// kRankSortMax).  Both give the same order.
constexpr int kRankSortMax = 16384;
struct SortArgs {
  const Cand* in;
  Cand* out;
  QueryState* state;
  int slot;
  unsigned long long* keys;
  int32_t* idx;
  int npow;
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
  const QueryState* state;  // batch size in state->batch_count, unless
  int batch_count;          // ... this is >= 0 (a host-chosen batch)
  double crop_row, crop_col, scale, phase;
  double angle_start, angle_end, angle_step, min_score;
  int rotate, subpixel, absolute, top, finest;
  double height, width;     // full image (domain test)
  RectGeom geom;
  DomainView dom;
};

// Level 0 (float crop); with `pairs`, also its fp16 pairs (launch_pairs' output)
cudaError_t launch_pyramid0(const void* src, int type, int64_t pitch_elems, int crop_row, int crop_col, LevelImage dst,
                            int32_t* error_flag, cudaStream_t s, uint32_t* pairs = nullptr);
cudaError_t launch_pyramid(const LevelImage& src, LevelImage dst, int32_t* error_flag, cudaStream_t s);
cudaError_t launch_prefix(const LevelImage& lev, cudaStream_t s);
cudaError_t launch_coarse(const CoarseArgs& a, int max_bh, int max_bw, cudaStream_t s, size_t smem_limit);
cudaError_t launch_nms(const NmsArgs& a, cudaStream_t s);
cudaError_t launch_track(const TrackArgs& a, int max_candidates, cudaStream_t s, size_t smem_limit);
cudaError_t launch_dedup(const DedupArgs& a, int max_candidates, cudaStream_t s);
cudaError_t launch_score(const ScoreArgs& a, int max_candidates, cudaStream_t s);
cudaError_t launch_adjoint(const AdjointArgs& a, cudaStream_t s);
cudaError_t launch_refine4(const Refine4Args& a, cudaStream_t s);
cudaError_t launch_sort(const SortArgs& a, int max_candidates, cudaStream_t s);
cudaError_t launch_rects(const Cand* sorted, RectAux* aux, const QueryState* state, RectGeom g, int max_candidates,
                         cudaStream_t s);
cudaError_t launch_select(const SelectArgs& a, cudaStream_t s);
cudaError_t launch_refine(const RefineArgs& a, int batch_limit, cudaStream_t s);

}  // namespace mvg
