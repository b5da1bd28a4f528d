// CreateNccModel's rotated rasters built on the device (ncc_build.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "ncc_model.h"
#include "ncc_types.h"

namespace mvg {

// One level's find tables, as DevLevel holds them (host copies).
struct LevelTables {
  std::vector<PatchDesc> desc;
  std::vector<double> angles;
  std::vector<int32_t> offs, runs, runs_end;
  std::vector<float> w;
  std::vector<int2> sw, lw;
};

// Rotates and normalises every level's rasters of `m` (levels, angles and
// level-0 moments from rebuild_model without rasters) on the current device
// and returns each level's tables; lin_pitch per level is the row pitch of
// the lw offsets.  Weights equal the host build bit for bit; the reference's
// errors are raised in its order (degenerate raster, sample budget, rotated
// box budget).
void build_tables_device(const HostModel& m, const std::vector<int32_t>& lin_pitch, std::vector<LevelTables>& out,
                         cudaStream_t s);

}  // namespace mvg
