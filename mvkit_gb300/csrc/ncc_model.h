// Host-side NCC model (CreateNccModel).  The model is built once on the host
// in FP64, exactly as the reference builds it, then uploaded to HBM as flat
// sample/run tables that the find kernels read.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "ncc_types.h"

namespace mvg {

struct Error : std::runtime_error {
  int32_t status;
  Error(int32_t s, const std::string& m) : std::runtime_error(m), status(s) {}
};
[[noreturn]] inline void raise(int32_t status, const std::string& message) { throw Error(status, message); }

struct CreateParams {
  int levels = 0;               // 0 = automatic (up to 16)
  bool ignore_polarity = false; // Metric "ignore_global_polarity"
  double angle_start = 0, angle_extent = 0, angle_step = 0;  // step 0 = automatic
};

// One template raster: samples in raster order with FP64 unit-energy weights.
struct Raster {
  double angle = 0, orow = 0, ocol = 0;
  int32_t rmin = 0, rmax = 0, cmin = 0, cmax = 0;
  std::vector<int32_t> rows, cols;
  std::vector<double> w;
  double wsum = 0;
  std::vector<int32_t> run_row, run_begin, run_end;
  size_t size() const { return w.size(); }
};

struct ModelLevel {
  size_t width = 0, height = 0;
  double orow = 0, ocol = 0;
  std::vector<double> gray;
  std::vector<uint8_t> mask;
  std::vector<Raster> patches;
};

// Limits of the model build (src/ncc_matching/model.cpp:14-18).
constexpr size_t kModelTemplatePixels = 1048576, kModelAngles = 4096, kModelSampleBudget = 16000000;

struct HostModel {
  CreateParams params;          // params.angle_step holds the resolved step
  size_t sample_count = 0;
  double origin_row = 0, origin_col = 0;
  Raster original;              // unrotated level-0 raster (row/col absolute)
  std::vector<ModelLevel> levels;
  // trained angles (the same list on every level) and the level-0 moments
  // that the unrotated level-0 raster reuses
  std::vector<double> angles;
  double level0_mean = 0, level0_energy = 0;
  bool rasters = true;          // levels[l].patches built (false: built on the device)
  size_t sample_budget = kModelSampleBudget;  // raster samples allowed (the building thread's budget)
};


// Budgets of this thread's model builds and finds.  By default the
// reference's: rotated-raster samples of a model (model.cpp:15,237), pixels
// of a search image (matcher.cpp:373-374), coarse candidates of a find
// (model.hpp:21, matcher.cpp:591), each exceeded with LimitExceeded.  An
// explicit extended mode (mvg_set_budgets) raises them; what fits the
// default budgets gives the same results either way.
struct Budgets {
  size_t samples = kModelSampleBudget;
  int64_t pixels = 32000000;
  int candidates = kMaxCandidates;
};
Budgets& thread_budgets();

// CreateNccModel on a byte (type 0) or uint16 (type 1) template.  `mask`
// (width*height bytes, nonzero = inside) is the template domain; NULL means
// the whole image.  Throws Error with an MvStatus code.
HostModel create_model(const void* pixels, int type, int64_t width, int64_t height, int64_t stride_bytes,
                       const uint8_t* mask, const CreateParams& params, bool rasters = true);

// The model from its mean-free level-0 raster (gray minus the template mean,
// mask, size and centroid) and the trained options: the path shared by
// create and by reading a model file.  Throws Error.
HostModel rebuild_model(ModelLevel first, const CreateParams& params, double origin_row, double origin_col,
                        bool rasters = true);

// The rotated rasters of every level and trained angle, in the reference's
// order (levels, then angles), with its errors.  Fills levels[l].patches.
void build_rasters(HostModel& m);

// Model files ("MVKIT_NCC 1", src/ncc_matching/persist.cpp:33-83): text body
// of the trained options, the level-0 raster and its centroid, prefixed by an
// FNV-1a 64 checksum of the body.  deserialize_model rebuilds the model.
std::string serialize_model(const HostModel& model);
HostModel deserialize_model(std::string_view bytes, bool rasters = true);
void write_model_file(const HostModel& model, const std::string& path);
HostModel read_model_file(const std::string& path, bool rasters = true);

// Geometry of one rotated raster (src/ncc_matching/model.cpp:66-80): the
// unrotated raster keeps the level's own pixels; a rotated one scans the
// integer offsets [r0, r1] x [c0, c1] about the level origin, sampling the
// level at (ca r + sa c + orow, -sa r + ca c + ocol).  too_large: the box
// exceeds the reference's budget (LimitExceeded).
struct RasterBox {
  double angle = 0, ca = 1, sa = 0;
  bool unrotated = false, too_large = false;
  int r0 = 0, r1 = -1, c0 = 0, c1 = -1;
};
RasterBox raster_box(const ModelLevel& level, double angle);

// Raster of `level` rotated by `angle` (used for query-range endpoints that
// fall between trained angles).  Empty when the rotation is degenerate.
Raster rotate_level(const ModelLevel& level, double angle);

}  // namespace mvg
