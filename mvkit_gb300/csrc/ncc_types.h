// Shared host/device layouts of the GB300 NCC matcher.
#pragma once
#include <cstdint>

#include <vector_types.h>

namespace mvg {

constexpr int kMaxLevels = 16;
constexpr int kMaxCandidates = 10000;        // FindOptions::max_candidates (src/ncc_matching/model.hpp:21)
constexpr int kMaxCandidatesExt = 1 << 21;   // largest candidate budget of an extended find
constexpr int kHashSlots = 32768;            // >= 3 x kMaxCandidates, power of two (dedup table of a default find)

// Status codes (MvStatus, include/mvkit/c/mv_status.h:12-24 in the reference).
enum Status : int32_t {
  kOk = 0,
  kInvalidArgument = -1,
  kTypeMismatch = -3,
  kOutOfMemory = -5,
  kUnsupported = -6,
  kInvalidState = -7,
  kIoError = -100,
  kDecodeError = -101,
  kLimitExceeded = -103,
  kInternal = -1000,
};

// One rotated template raster on the device.  Sample offsets are relative to
// the patch reference point (the level origin for rotated patches, the level's
// top-left corner for the unrotated one, src/ncc_matching/model.cpp:66-98).
struct PatchDesc {
  double angle;
  double orow, ocol;            // added to the integer position to get the pose
  int32_t rmin, rmax, cmin, cmax;
  int32_t n;                    // samples
  int32_t sample_off;           // into the level's sample arrays
  int32_t nruns;                // contiguous row spans
  int32_t run_off;
  float wsum;                   // sum of the float sample weights
  int32_t pad_;
};

// Device view of one model level (its patches and their samples).
struct LevelView {
  const PatchDesc* patches;
  const int32_t* offs;          // packed (row << 16) | (col & 0xffff), int16 each
  const float* w;               // sample weights (float of the FP64 model weight)
  const int2* sw;               // interleaved {offs, float bits of w} per sample
  const int2* lw;               // interleaved {row * lin_pitch + col, float bits of w} per sample
  int32_t lin_pitch;            // row pitch of lw offsets (= 5 mod 32)
  int32_t lin_rows;             // rows of a window that holds any 5x5 placement set
  const int32_t* runs;          // packed row(16) | begin; end in runs_end
  const int32_t* runs_end;
  const int2* run2;             // the same interleaved: {packed row | begin, end}
  int32_t npatches;
};

// Unrotated full-resolution template used for continuous scoring and the
// Gauss-Newton fit (Model::original, src/ncc_matching/model.cpp:182-204).
struct OriginalView {
  const float* dr;              // sample row - level origin row
  const float* dc;              // sample column - level origin column
  const float* w;
  const float4* dcw;            // the same samples packed {dr, dc, w, 0}
  float dr_min, dr_max, dc_min, dc_max;  // sample offset box
  int32_t n;
};

// A candidate pose carried between stages.  (row, column, angle) follow the
// reference's FP64 expressions exactly; score is the stage's score.
struct Cand {
  double row, col, angle;
  double score;
  int32_t patch;                // patch index on the candidate's level (-1 off the lattice)
  int32_t pad;
};

// Rotated template rectangle of a pose for the MaxOverlap test: FP64 cos/sin
// and a conservative FP32 axis-aligned box in image coordinates.
struct RectAux {
  double ca, sa;
  float x0, y0, x1, y1;
};

// Result of refining one candidate (src/ncc_matching/matcher.cpp:878-1061).
struct Refined {
  double row, col, angle, score;
  int32_t ok;                   // score >= MinScore and inside the domain
  int32_t pad;
  RectAux rect;
};

// Per-query device state that kernels read and write.
struct QueryState {
  int32_t count[kMaxLevels + 2];   // candidates per stage
  int32_t overflow;                // coarse candidate budget exceeded
  int32_t error;                   // kernel-side failure code
  int32_t sorted_count;            // finite full-resolution candidates
  int32_t accepted;                // matches accepted by the greedy selection
  int32_t next;                    // next candidate index to examine
  int32_t need;                    // 1: refinement results missing for `next`
  int32_t done;
  int32_t batch_count;             // entries in the refinement batch
  int32_t cap;                     // candidate budget of the find (list buffers hold this many)
  int32_t pix_min, pix_max;        // range of the level-0 crop (uint16 finds: tensor-core plane offsets)
  unsigned long long track_macs;   // algorithmic MACs of the CUDA-core tracking (25 positions x samples per patch)
  unsigned long long tc_macs;      // algorithmic MACs of the tensor-core tracking
  unsigned long long tc_issued;    // MACs issued to the tensor cores (M x N x K per MMA)
};

}  // namespace mvg
