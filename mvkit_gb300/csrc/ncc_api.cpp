// Host side of the GB300 NCC find: query planning (crop, patch lists,
// position ranges) in FP64 exactly as the reference plans it, the kernel
// sequence on one CUDA stream, and the C ABI of include/mvkit_gb300_ncc.h.
//   prepare  src/ncc_matching/matcher.cpp:343-851
//   find     src/ncc_matching/matcher.cpp:1063-1076
//   C API    src/c_api/ncc_matching_api.cpp:29-203
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/mvkit_gb300_ncc.h"
#include "ncc_build.h"
#include "ncc_kernels.h"
#include "ncc_model.h"

namespace mvg {
namespace {

thread_local std::string g_last_error;

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) raise(kOutOfMemory, std::string(what) + ": " + cudaGetErrorString(e));
    raise(kInternal, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

template <class T> struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void reserve(size_t count) {
    if (count <= n && p) return;
    release();
    check(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), "cudaMalloc");
    n = std::max<size_t>(count, 1);
  }
  void upload(const std::vector<T>& v, cudaStream_t s) {
    reserve(v.size());
    if (!v.empty()) check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
};

// ------------------------------------------------------------------ model
// Tensor-core groups of one tracking step (cached per target level and query
// plan): group table, source patch -> group, weight matrices, launch shape.
struct TcPlan {
  int parts = 1;          // fp16 planes per level value
  float offset = 0;       // level value subtracted in the planes
  int stages = 2;         // weight-chunk buffers
  int sets = 1, npad = 32;  // accumulator sets, tensor-memory columns per set
  int stage_bytes = 0, abuf_bytes = 0;  // weight buffer, window buffer
  int rows_slab = 16;     // staged window rows (one TMA box)
  size_t smem = 0;        // dynamic shared memory of the launch
  std::vector<TcGroup> groups;
  std::vector<int32_t> group_of_src;
  std::vector<std::unique_ptr<DevBuf<uint8_t>>> weights;
};

struct DevLevel {
  int32_t lin_pitch = 0, lin_rows = 0;  // staged tracking window geometry
  std::vector<PatchDesc> desc;      // host copy (model patches + query endpoints)
  std::vector<double> angles;
  size_t model_patches = 0;         // trained patches; endpoints follow
  std::vector<int32_t> offs, runs, runs_end;
  std::vector<float> w;
  std::vector<int2> sw, lw;
  DevBuf<PatchDesc> d_desc;
  DevBuf<int32_t> d_offs, d_runs, d_runs_end;
  DevBuf<float> d_w;
  DevBuf<int2> d_sw, d_lw, d_run2;
  // Window geometry for a level of width x height: any rotation's raster
  // fits the diagonal; 5x5 placements and centre rounding add 8 cells.
  void set_geometry(size_t width, size_t height) {
    const int diag = int(std::ceil(std::hypot(double(width), double(height)))) + 1;
    lin_rows = diag + 8;
    lin_pitch = lin_rows + ((5 - lin_rows) % 32 + 32) % 32;
  }
  void append(const Raster& r) {
    PatchDesc d{};
    d.angle = r.angle;
    d.orow = r.orow;
    d.ocol = r.ocol;
    d.rmin = r.rmin;
    d.rmax = r.rmax;
    d.cmin = r.cmin;
    d.cmax = r.cmax;
    d.n = int32_t(r.size());
    d.sample_off = int32_t(offs.size());
    d.nruns = int32_t(r.run_row.size());
    d.run_off = int32_t(runs.size());
    double wsum = 0;
    for (size_t i = 0; i < r.size(); ++i) {
      const int32_t o = int32_t((uint32_t(uint16_t(int16_t(r.rows[i]))) << 16) | uint16_t(int16_t(r.cols[i])));
      const float wf = float(r.w[i]);
      int32_t wbits;
      std::memcpy(&wbits, &wf, sizeof(wbits));
      offs.push_back(o);
      w.push_back(wf);
      sw.push_back(make_int2(o, wbits));
      lw.push_back(make_int2(r.rows[i] * lin_pitch + r.cols[i], wbits));
      wsum += double(wf);
    }
    d.wsum = float(wsum);
    for (size_t j = 0; j < r.run_row.size(); ++j) {
      runs.push_back(int32_t((uint32_t(uint16_t(int16_t(r.run_row[j]))) << 16) | uint16_t(int16_t(r.run_begin[j]))));
      runs_end.push_back(r.run_end[j]);
    }
    desc.push_back(d);
    angles.push_back(r.angle);
  }
  // tensor-core plans of tracking steps into this level, by query plan
  std::map<std::vector<int32_t>, std::shared_ptr<const TcPlan>> tc_plans;
  // Replaced device tables stay allocated until the model is cleared: finds
  // on other threads may still be reading them.
  std::vector<void*> retired;
  ~DevLevel() {
    for (void* p : retired) cudaFree(p);
  }
  template <class T> void retire(DevBuf<T>& b) {
    if (b.p) retired.push_back(b.p);
    b.p = nullptr;
    b.n = 0;
  }
  void upload() {
    retire(d_desc);
    retire(d_offs);
    retire(d_runs);
    retire(d_runs_end);
    retire(d_w);
    retire(d_sw);
    retire(d_lw);
    retire(d_run2);
    std::vector<int2> run2(runs.size());
    for (size_t i = 0; i < runs.size(); ++i) run2[i] = make_int2(runs[i], runs_end[i]);
    d_run2.upload(run2, nullptr);
    d_desc.upload(desc, nullptr);
    d_sw.upload(sw, nullptr);
    d_lw.upload(lw, nullptr);
    d_offs.upload(offs, nullptr);
    d_runs.upload(runs, nullptr);
    d_runs_end.upload(runs_end, nullptr);
    d_w.upload(w, nullptr);
    check(cudaDeviceSynchronize(), "model upload");
  }
  LevelView view() const {
    LevelView v;
    v.patches = d_desc.p;
    v.offs = d_offs.p;
    v.w = d_w.p;
    v.sw = d_sw.p;
    v.lw = d_lw.p;
    v.lin_pitch = lin_pitch;
    v.lin_rows = lin_rows;
    v.runs = d_runs.p;
    v.runs_end = d_runs_end.p;
    v.run2 = d_run2.p;
    v.npatches = int32_t(desc.size());
    return v;
  }
};

struct OrigDev {
  DevBuf<float> dr, dc, w;
  DevBuf<float4> dcw;
  float box[4] = {0, 0, 0, 0};
  int32_t n = 0;
  void set(const Raster& r, double orow, double ocol) {
    std::vector<float> a(r.size()), b(r.size()), c(r.size());
    std::vector<float4> packed(r.size());
    box[0] = box[2] = INFINITY;
    box[1] = box[3] = -INFINITY;
    for (size_t i = 0; i < r.size(); ++i) {
      a[i] = float(double(r.rows[i]) - orow);
      b[i] = float(double(r.cols[i]) - ocol);
      c[i] = float(r.w[i]);
      packed[i] = make_float4(a[i], b[i], c[i], 0.f);
      box[0] = std::min(box[0], a[i]);
      box[1] = std::max(box[1], a[i]);
      box[2] = std::min(box[2], b[i]);
      box[3] = std::max(box[3], b[i]);
    }
    dr.upload(a, nullptr);
    dc.upload(b, nullptr);
    w.upload(c, nullptr);
    dcw.upload(packed, nullptr);
    n = int32_t(r.size());
    check(cudaDeviceSynchronize(), "model upload");
  }
  OriginalView view() const {
    return OriginalView{dr.p, dc.p, w.p, dcw.p, box[0], box[1], box[2], box[3], n};
  }
};

}  // namespace
}  // namespace mvg

struct mvg_ncc_model_s {
  mvg::HostModel host;
  // device tables, uploaded by the first find (under `mutex`) to the device
  // current then; a model is built and saved on the host alone
  std::vector<std::unique_ptr<mvg::DevLevel>> levels;
  mvg::OrigDev original;
  // unrotated rasters of coarser finest levels (lowest_level > 1), by level
  std::vector<std::unique_ptr<mvg::OrigDev>> coarse_original;
  std::mutex mutex;  // guards the endpoint caches
  int device = 0;
};

namespace mvg {
namespace {

// Test hook (this thread's finds): the tensor-core kernel loads no weights, so
// its bounded waits run out and the find reports the device error flag.
thread_local int t_withhold_weights = 0;

// Where models are built: 0 = the rotated rasters on the device when one is
// present, 1 = on the host (the reference's order in FP64 on the CPU).
std::atomic<int> g_model_build{0};

// Rotated rasters of a model whose pyramid and angles are built: on the
// device (straight into the find tables, uploaded now) or on the host (tables
// packed and uploaded by the first find).
void finish_model(mvg_ncc_model_s& m) {
  int ndev = 0;
  if (g_model_build.load() != 0 || cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    build_rasters(m.host);
    return;
  }
  check(cudaGetDevice(&m.device), "cudaGetDevice");
  std::vector<std::unique_ptr<DevLevel>> levels;
  std::vector<int32_t> pitch;
  for (const ModelLevel& L : m.host.levels) {
    auto d = std::make_unique<DevLevel>();
    d->set_geometry(L.width, L.height);
    pitch.push_back(d->lin_pitch);
    levels.push_back(std::move(d));
  }
  std::vector<LevelTables> t;
  build_tables_device(m.host, pitch, t, nullptr);
  for (size_t l = 0; l < levels.size(); ++l) {
    DevLevel& d = *levels[l];
    d.desc = std::move(t[l].desc);
    d.angles = std::move(t[l].angles);
    d.offs = std::move(t[l].offs);
    d.w = std::move(t[l].w);
    d.sw = std::move(t[l].sw);
    d.lw = std::move(t[l].lw);
    d.runs = std::move(t[l].runs);
    d.runs_end = std::move(t[l].runs_end);
    d.model_patches = d.desc.size();
    d.upload();
  }
  m.original.set(m.host.original, m.host.levels.front().orow, m.host.levels.front().ocol);
  m.levels = std::move(levels);
}

// The model's sample, run and raster tables in HBM (once per model).
void ensure_device(mvg_ncc_model_s& m) {
  if (!m.levels.empty()) return;
  check(cudaGetDevice(&m.device), "cudaGetDevice");
  std::vector<std::unique_ptr<DevLevel>> levels;
  for (const ModelLevel& L : m.host.levels) {
    auto d = std::make_unique<DevLevel>();
    d->set_geometry(L.width, L.height);
    for (const Raster& r : L.patches) d->append(r);
    d->model_patches = d->desc.size();
    d->upload();
    levels.push_back(std::move(d));
  }
  m.original.set(m.host.original, m.host.levels.front().orow, m.host.levels.front().ocol);
  m.levels = std::move(levels);
}

// Index of the raster at `angle` on `level` among the query endpoints,
// building and uploading it on first use.  -1 when degenerate.
int endpoint_patch(mvg_ncc_model_s& m, size_t level, double angle) {
  DevLevel& L = *m.levels[level];
  for (size_t i = L.model_patches; i < L.desc.size(); ++i)
    if (L.angles[i] == angle) return int(i);
  Raster r = rotate_level(m.host.levels[level], angle);
  if (r.w.empty()) return -1;
  L.append(r);
  L.upload();
  return int(L.desc.size() - 1);
}

const OrigDev& coarse_original(mvg_ncc_model_s& m, size_t level) {
  if (m.coarse_original.size() <= level) m.coarse_original.resize(level + 1);
  if (!m.coarse_original[level]) {
    Raster r = rotate_level(m.host.levels[level], 0.);
    auto o = std::make_unique<OrigDev>();
    o->set(r, m.host.levels[level].orow, m.host.levels[level].ocol);
    m.coarse_original[level] = std::move(o);
  }
  return *m.coarse_original[level];
}

// Dynamic shared memory one tensor-core block may use: kTcBlocksPerSm blocks
// share an SM (228 KB, each with its static part and 1 KB reserved).
size_t tc_smem_budget(size_t optin) {
  const size_t per_sm = 228 * 1024;
  const size_t share = per_sm / kTcBlocksPerSm - tc_kernel_static_smem() - 1024;
  return std::min(share, optin - tc_kernel_static_smem()) - 1024;
}
// Launch size of a plan: with one block per SM, more than half the SM's
// shared memory keeps a second block (and its tensor-memory allocation) off.
size_t tc_launch_smem(const TcPlan& P, size_t optin) {
  return kTcBlocksPerSm == 1 ? std::max(P.smem, optin / 2 + 1024) : P.smem;
}

// Correlation path of this thread's finds: tensor cores where applicable
// (0) or FP32 CUDA cores only (1).
thread_local int t_path = 0;
// grid rows of tensor-core weights in flight ahead of the MMAs (launch shape only)
thread_local int t_tc_lookahead = 8;
// Batched calls from this thread: cohorts of workers whose finds' tensor-core
// launches are merged (0, default: every find launches its own).
thread_local int t_merge_tc = 0;

uint16_t half_bits(double x) {
  const _Float16 h = static_cast<_Float16>(x);
  uint16_t b;
  std::memcpy(&b, &h, sizeof(b));
  return b;
}
double half_value(uint16_t b) {
  _Float16 h;
  std::memcpy(&h, &b, sizeof(b));
  return double(h);
}

// fp16 planes of level t: the level minus `offset` as base-64 digits, each
// an exact fp16 integer: the first signed (|d| <= 2048), the others in
// [0, 64) (parts 1: the value itself; 2: 64 h + l; up to 4 for uint16
// level sums); 0 when even four parts do not hold it (the CUDA-core path
// scores that level).
int tc_parts(int type, size_t t, float* offset) {
  const double maxv = (type == 1 ? 65535.0 : 255.0) * std::ldexp(1., int(2 * t));
  const double off = std::floor((maxv + 1) * .5);
  *offset = float(off);
  const double range = std::max(off, maxv - off);
  for (int parts = 1; parts <= kTcMaxParts; ++parts)
    if (range <= 2048.0 * std::ldexp(1.0, 6 * (parts - 1))) return parts;
  return 0;
}

// ------------------------------------------------------------- query plan
struct FindParams {
  double angle_start = 0, angle_extent = 0, min_score = .8, max_overlap = .5;
  int64_t num_matches = 1;
  bool subpixel = true;
  int highest = 0, lowest = 1;
};

// Largest/smallest integer r in [lo, hi) with pred(r) true, for predicates
// monotone over r.  Returns an empty range when none holds.
template <class Pred> void clip_increasing(int& lo, int& hi, Pred below_min) {
  // below_min(r) true for small r, false from some r on (monotone).
  int a = lo, b = hi;
  while (a < b) {
    const int mid = a + (b - a) / 2;
    if (below_min(mid)) a = mid + 1;
    else b = mid;
  }
  lo = a;
}
template <class Pred> void clip_decreasing(int& lo, int& hi, Pred above_max) {
  // above_max(r) false for small r, true from some r on.
  int a = lo, b = hi;
  while (a < b) {
    const int mid = a + (b - a) / 2;
    if (above_max(mid)) b = mid;
    else a = mid + 1;
  }
  hi = a;
}

// Position interval on a level where the pose lies in the search domain's
// bounding box [box_lo, box_hi] as the reference tests it (may_contain,
// matcher.cpp:507-534).  For the full image that is the whole test; a
// reduced domain is tested per pose on the device as well.
void pose_interval(int& lo, int& hi, double crop, double step, double o, double off, double box_lo, double box_hi) {
  auto pose = [&](int r) { return crop + step * (r + o) + off; };
  if (step == 1) {
    // domain_contains: box_lo <= floor(pose + .5) <= box_hi
    clip_increasing(lo, hi, [&](int r) { return std::floor(pose(r) + .5) < box_lo; });
    clip_decreasing(lo, hi, [&](int r) { return std::floor(pose(r) + .5) > box_hi; });
  } else {
    const double margin = 2 * step;
    clip_increasing(lo, hi, [&](int r) { return pose(r) < box_lo - margin; });
    clip_decreasing(lo, hi, [&](int r) { return pose(r) > box_hi + margin; });
  }
  if (hi < lo) hi = lo;
}

struct LevelPlan {
  std::vector<int32_t> plist;  // query patch order
  std::vector<PosRange> ranges;
  // tracking into this level: plist entries inside the angle window of each
  // source patch of the next coarser level (CSR by source patch index)
  std::vector<int32_t> sel_off, sel_idx;
};

// True when a value is a multiple of 2^-4 of magnitude <= 2048: then every
// lattice expression of the tracking step is exact in FP32.
bool lattice_exact32(double v) {
  const double s = v * 16;
  return std::abs(v) <= 2048 && s == std::floor(s);
}

// Builds the tensor-core groups of the tracking step into level T (query
// plan `lp`, `nsrc` patches on the source level).  A group is the rotated
// patches (origin on the lattice) of one source patch's selected list; the
// sources with identical lists share it.  Weights: per chunk of rg grid
// rows, an N x K fp16 matrix in the canonical K-major no-swizzle layout
// (8 x 8 core matrices of 128 bytes, K-adjacent cores 128 bytes apart,
// N-adjacent cores K/8 x 128 bytes apart); column (((p 5 + dc) rg + y mod
// rg) 2 + half) holds the high or low fp16 half of sigma w_p(y, x - dc), row
// x + part kw the same for each plane part (x 64 per digit above the last).
// The slots of one output sit side by side, so 32 accumulator columns hold
// 16 / rg whole outputs (rg is 1, 2 or 4).  The last 16 rows hold the
// column's row sum for grid row y as two fp16 terms (x 64 likewise), which
// the centring columns of the window multiply.
std::shared_ptr<const TcPlan> build_tc_plan(const DevLevel& T, size_t nsrc, const LevelPlan& lp, int parts,
                                            float offset, size_t budget, int lookahead) {
  auto plan = std::make_shared<TcPlan>();
  plan->parts = parts;
  plan->offset = offset;
  plan->group_of_src.assign(nsrc, -1);
  struct Proto {
    std::vector<int32_t> ks, descs;
    int rmin = INT32_MAX, rmax = INT32_MIN, cmin = INT32_MAX, cmax = INT32_MIN;
    int kr = 0, kw = 0, rg = 1, n = 0;
  };
  std::vector<Proto> protos;
  std::map<std::vector<int32_t>, int> by_key;
  for (size_t src = 0; src < nsrc && protos.size() < size_t(kTcMaxGroups); ++src) {
    const int b = lp.sel_off[src], e = lp.sel_off[src + 1];
    if (e == b || e - b > kTcMaxP) continue;
    Proto pr;
    for (int k = 0; k < e - b; ++k) {
      const int32_t di = lp.plist[size_t(lp.sel_idx[size_t(b + k)])];
      const PatchDesc& d = T.desc[size_t(di)];
      if (d.orow != 0 || d.ocol != 0) continue;
      pr.ks.push_back(k);
      pr.descs.push_back(di);
      pr.rmin = std::min(pr.rmin, d.rmin);
      pr.rmax = std::max(pr.rmax, d.rmax);
      pr.cmin = std::min(pr.cmin, d.cmin);
      pr.cmax = std::max(pr.cmax, d.cmax);
    }
    if (pr.descs.empty()) continue;
    std::vector<int32_t> key(pr.descs);
    key.insert(key.end(), pr.ks.begin(), pr.ks.end());
    const auto it = by_key.find(key);
    if (it != by_key.end()) {
      plan->group_of_src[src] = it->second;
      continue;
    }
    pr.kr = pr.rmax - pr.rmin + 1;
    pr.kw = (pr.cmax - pr.cmin + 1 + 4 + 15) / 16 * 16;
    // grid rows per chunk: a power of two (whole outputs per 32 accumulator
    // columns), as many as keep N <= 256, and <= 4 (placement row + chunk
    // row stays within the 8 rows of a candidate)
    const int P = int(pr.descs.size());
    pr.rg = 4;
    while (pr.rg > 1 && (10 * P * pr.rg + 15) / 16 * 16 > 256) pr.rg >>= 1;
    pr.n = (10 * P * pr.rg + 15) / 16 * 16;
    by_key[key] = int(protos.size());
    plan->group_of_src[src] = int(protos.size());
    protos.push_back(std::move(pr));
  }
  if (protos.empty()) return plan;
  // costliest groups first: their tiles come first in the tile list, and the
  // kernel hands tiles out in list order (longest tiles first balances the
  // blocks' last tiles)
  {
    auto cost = [&](const Proto& pr) {
      return double((pr.kr + pr.rg - 1) / pr.rg) * double(parts * pr.kw + 16) * double(pr.n);
    };
    std::vector<int> order(protos.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return cost(protos[size_t(x)]) > cost(protos[size_t(y)]); });
    std::vector<int> rank(protos.size());
    std::vector<Proto> sorted;
    sorted.reserve(protos.size());
    for (size_t i = 0; i < order.size(); ++i) {
      rank[size_t(order[i])] = int(i);
      sorted.push_back(std::move(protos[size_t(order[i])]));
    }
    protos = std::move(sorted);
    for (int32_t& g : plan->group_of_src)
      if (g >= 0) g = rank[size_t(g)];
  }
  // one launch shape for the step: weight buffers from the largest chunk, the
  // window slab as tall as every group allows
  size_t max_chunk = 0;
  int max_kr = 0;
  int max_n = 0;
  int min_rg = 4;
  for (const Proto& pr : protos) {
    min_rg = std::min(min_rg, pr.rg);
    max_chunk = std::max(max_chunk, size_t(pr.n) * size_t(parts * pr.kw + 16) * 2);
    max_kr = std::max(max_kr, pr.kr);
    max_n = std::max(max_n, pr.n);
  }
  plan->npad = (max_n + 31) / 32 * 32;
  // two accumulator regions (the next tile's MMAs run while the epilogue
  // reads the last one), each sets x npad columns
  plan->sets = std::max(1, std::min(4, 256 / kTcBlocksPerSm / plan->npad));
  // shared memory: weight ring | two window buffers (rows_slab rows each).
  // The ring holds `lookahead` grid rows of weights (at least two chunks)
  // ahead of the MMAs, for the L2 latency; the window buffers take the rest,
  // at least 16 rows each.  Neither changes a result.
  int max_nseg = 0;
  for (const Proto& pr : protos) max_nseg = std::max(max_nseg, parts * pr.kw / 8 + 2);
  const size_t per_row = size_t(kTcCands) * size_t(max_nseg) * 16;
  const size_t min_windows = 2 * per_row * 16 + 1024;
  if (min_windows + 2 * max_chunk > budget) {
    plan->group_of_src.assign(nsrc, -1);
    return plan;
  }
  const int stages = int(std::min<size_t>({size_t(kTcMaxStages), size_t(std::max(2, (lookahead + min_rg - 1) / min_rg)),
                                           (budget - min_windows) / max_chunk}));
  const size_t ring = size_t(stages) * max_chunk + 1024;
  // a slab holds whole chunks of grid rows plus the 7 placement rows; more
  // rows than the tallest group's grid plus that need are never used
  const int rows = std::min(std::min(256, max_kr + 3 + 7), int((budget - ring) / 2 / per_row));
  if (rows < 16) {
    // a slab must hold at least one chunk of grid rows plus the 7 placement
    // rows of the window; otherwise the step stays on the CUDA cores
    plan->group_of_src.assign(nsrc, -1);
    return plan;
  }
  plan->stages = stages;
  plan->rows_slab = rows;
  plan->stage_bytes = int(max_chunk);
  plan->abuf_bytes = int(per_row * size_t(rows));
  plan->smem = ring + 2 * per_row * size_t(rows);
  for (const Proto& pr : protos) {
    const int P = int(pr.descs.size()), K = parts * pr.kw + 16, N = pr.n;
    const size_t chunk_elems = size_t(N) * size_t(K);
    double maxw = 0, maxrow = 0;
    for (int32_t di : pr.descs) {
      const PatchDesc& d = T.desc[size_t(di)];
      std::vector<double> row(size_t(pr.kr), 0.0);
      for (int i = 0; i < d.n; ++i) {
        const double w = double(T.w[size_t(d.sample_off + i)]);
        maxw = std::max(maxw, std::abs(w));
        row[size_t((T.offs[size_t(d.sample_off + i)] >> 16) - pr.rmin)] += std::abs(w);
      }
      for (double r : row) maxrow = std::max(maxrow, r);
    }
    // weight scale: a power of two keeping the weights (x 64 for a split
    // level) and the centring row sums (x 64 likewise) within fp16 range
    const double m64 = std::ldexp(1.0, 6 * (parts - 1));  // multiplier of the first part
    const double limit = std::min(maxw > 0 ? 16384.0 / (maxw * m64) : 1e30, maxrow > 0 ? 16384.0 / (maxrow * m64) : 1e30);
    const double sigma = limit < 1e30 ? std::ldexp(1., int(std::floor(std::log2(limit)))) : 1.0;
    const int rg = pr.rg, chunks = (pr.kr + rg - 1) / rg;
    std::vector<uint16_t> host(size_t(chunks) * chunk_elems, 0);
    TcGroup g{};
    g.kr = pr.kr;
    g.kw = pr.kw;
    g.parts = parts;
    g.rmin = pr.rmin;
    g.cmin = pr.cmin;
    g.p = P;
    g.rg = rg;
    g.n = N;
    g.rows_slab = rows;
    g.inv_scale = float(1.0 / sigma);
    g.macs = 0;
    // element of grid row y, column (patch q, placement dc, half), K index k:
    // chunk y / rg, N column ((q 5 + dc) rg + y mod rg) 2 + half
    auto at = [&](size_t y, int q, int dc, int half, int k) {
      const int n = ((q * 5 + dc) * rg + int(y % size_t(rg))) * 2 + half;
      return (y / size_t(rg)) * chunk_elems + size_t(n / 8) * size_t(K / 8) * 64 + size_t(k / 8) * 64 +
             size_t(n % 8) * 8 + size_t(k % 8);
    };
    for (int q = 0; q < P; ++q) {
      const PatchDesc& d = T.desc[size_t(pr.descs[size_t(q)])];
      double sum = 0;
      std::vector<double> rs(size_t(pr.kr) * 2, 0.0);  // row sums of the two halves
      for (int i = 0; i < d.n; ++i) {
        const int32_t o = T.offs[size_t(d.sample_off + i)];
        const int row = o >> 16, col = int(int16_t(o & 0xffff));
        const double ws = double(T.w[size_t(d.sample_off + i)]) * sigma;
        const uint16_t hi = half_bits(ws);
        const double hv = half_value(hi);
        const uint16_t lo = half_bits(ws - hv);
        const double lv = half_value(lo);
        sum += hv + lv;
        const size_t y = size_t(row - pr.rmin);
        rs[y * 2] += hv;
        rs[y * 2 + 1] += lv;
        for (int dc = 0; dc < 5; ++dc) {
          const int x = col - pr.cmin + dc;
          for (int part = 0; part < parts; ++part) {
            const double mult = std::ldexp(1.0, 6 * (parts - 1 - part));
            const int k = part * pr.kw + x;
            for (int half = 0; half < 2; ++half)
              host[at(y, q, dc, half, k)] = half_bits((half ? lv : hv) * mult);
          }
        }
      }
      // centring rows: the row sum of each column as two fp16 terms
      double ecorr = 0;
      const int kc0 = parts * pr.kw;
      for (size_t y = 0; y < size_t(pr.kr); ++y)
        for (int half = 0; half < 2; ++half) {
          const double r = rs[y * 2 + size_t(half)];
          const uint16_t f1 = half_bits(r);
          const uint16_t f2 = half_bits(r - half_value(f1));
          ecorr += half_value(f1) + half_value(f2);
          // part q of the centre meets 64^(parts - 1 - q) x the row sum
          for (int dc = 0; dc < 5; ++dc)
            for (int part = 0; part < parts; ++part) {
              const double mult = std::ldexp(1.0, 6 * (parts - 1 - part));
              host[at(y, q, dc, half, kc0 + 2 * part)] = half_bits(mult * half_value(f1));
              host[at(y, q, dc, half, kc0 + 2 * part + 1)] = half_bits(mult * half_value(f2));
            }
        }
      g.ecorr[q] = float(ecorr / sigma);
      g.k_of[q] = pr.ks[size_t(q)];
      const int32_t o0 = T.offs[size_t(d.sample_off)];
      g.r0[q] = o0 >> 16;
      g.c0[q] = int(int16_t(o0 & 0xffff));
      g.weff[q] = float(sum / sigma);
      g.weff_k[pr.ks[size_t(q)]] = g.weff[q];
      g.macs += 25ll * d.n;
    }
    auto buf = std::make_unique<DevBuf<uint8_t>>();
    buf->reserve(host.size() * 2);
    check(cudaMemcpy(buf->p, host.data(), host.size() * 2, cudaMemcpyHostToDevice), "tc weights");
    g.b = buf->p;
    plan->weights.push_back(std::move(buf));
    plan->groups.push_back(g);
  }
  return plan;
}

// ------------------------------------------------------------- workspace
struct Workspace {
  int device = -1;
  cudaStream_t own_stream = nullptr;
  DevBuf<uint8_t> image;
  DevBuf<float> lev_v[kMaxLevels];
  DevBuf<longlong2> lev_p[kMaxLevels];
  DevBuf<float> planes;
  DevBuf<Cand> cand_a, cand_b, tmp, sorted, accepted;
  DevBuf<unsigned long long> sort_keys;  // bitonic sort of long lists (budgets above kRankSortMax)
  DevBuf<int32_t> sort_idx;
  DevBuf<RectAux> aux, accepted_aux;
  DevBuf<int32_t> tested;
  DevBuf<uint8_t> sup;
  DevBuf<int> table;
  DevBuf<Refined> refined;
  DevBuf<int32_t> refined_flag, batch;
  DevBuf<QueryState> state;
  DevBuf<float> tc_dots, coarse_dots;
  DevBuf<Cand> coarse_cand;
  DevBuf<int2> coarse_rc;
  DevBuf<uint32_t> pairs;            // fp16 pairs of the finest level
  int pairs_level = -1;              // the level `pairs` holds
  DevBuf<uint8_t> dom_mask;          // search domain of the current find
  DevBuf<int32_t> dom_count, dom_row_run;
  DevBuf<int4> dom_runs;
  DevBuf<double> adj_poses, adj_score, adj_grad;  // NCC adjoint calls
  DevBuf<uint16_t> tc_planes;
  DevBuf<int32_t> tc_order, tc_counts, tc_offsets, tc_cursor;
  DevBuf<TcTiles> tc_tiles;
  DevBuf<uint8_t> tables;            // query patch lists and ranges, one upload
  uint8_t* h_tables = nullptr;       // pinned staging of the same
  size_t h_tables_size = 0;
  QueryState* h_state = nullptr;
  int32_t* h_error = nullptr;
  size_t smem_optin = 0;
  int sm_count = 0;
  cudaEvent_t tc_ready = nullptr;    // this find's tensor-core inputs are complete (merged launches)
  ~Workspace() {
    if (h_tables) cudaFreeHost(h_tables);
    if (h_state) cudaFreeHost(h_state);
    if (tc_ready) cudaEventDestroy(tc_ready);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
  void init() {
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    if (device == dev) return;
    device = dev;
    check(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    check(cudaEventCreateWithFlags(&tc_ready, cudaEventDisableTiming), "cudaEventCreate");
    check(cudaMallocHost(&h_state, sizeof(QueryState)), "cudaMallocHost");
    int optin = 0;
    check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attribute");
    smem_optin = size_t(optin);
    check(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev), "attribute");
    cand_a.reserve(kMaxCandidates);
    cand_b.reserve(kMaxCandidates);
    tmp.reserve(kMaxCandidates);
    sorted.reserve(kMaxCandidates);
    accepted.reserve(kMaxCandidates);
    aux.reserve(kMaxCandidates);
    accepted_aux.reserve(kMaxCandidates);
    tested.reserve(kMaxCandidates);
    sup.reserve(kMaxCandidates);
    table.reserve(kHashSlots);
    refined.reserve(kMaxCandidates);
    refined_flag.reserve(kMaxCandidates);
    batch.reserve(64);
    state.reserve(1);
  }
  // Stages `bytes` of query tables; returns the pinned host pointer.
  uint8_t* stage_tables(size_t bytes) {
    if (bytes > h_tables_size) {
      if (h_tables) cudaFreeHost(h_tables);
      h_tables = nullptr;
      h_tables_size = 0;
      check(cudaMallocHost(&h_tables, bytes), "cudaMallocHost");
      h_tables_size = bytes;
    }
    tables.reserve(bytes);
    return h_tables;
  }
};

thread_local std::unique_ptr<Workspace> t_workspace;

Workspace& workspace() {
  if (!t_workspace) t_workspace = std::make_unique<Workspace>();
  t_workspace->init();
  return *t_workspace;
}

// Zeroes the query state on the device and sets its candidate budget, from
// the pinned host copy (no readback of the state is in flight between finds).
void init_state(Workspace& ws, cudaStream_t s, int cap) {
  *ws.h_state = QueryState{};
  ws.h_state->cap = cap;
  ws.h_state->pix_min = std::numeric_limits<int32_t>::max();
  ws.h_state->pix_max = std::numeric_limits<int32_t>::min();
  check(cudaMemcpyAsync(ws.state.p, ws.h_state, sizeof(QueryState), cudaMemcpyHostToDevice, s), "state");
}

// Power of two >= 3 x the candidate budget (the dedup table of a find).
int hash_slots(int cap) {
  int n = kHashSlots;
  while (n < 3 * cap) n *= 2;
  return n;
}

// Per-thread stage profile: CUDA events on the find's stream around each
// kernel group (only while enabled), launch counts and algorithmic work.
enum Stage { kStUpload, kStPyramid, kStPrefix, kStCoarse, kStNms, kStTrack, kStDedup, kStScore, kStSort, kStSelect,
             kStRefine, kStTrackTc, kStTcPrep, kStages };
const char* const kStageNames[kStages] = {"upload", "pyramid", "prefix", "coarse",   "nms",      "track",  "dedup",
                                          "score",  "sort",    "select", "refine",   "track_tc", "tc_prep"};
struct Profiler {
  bool on = false;
  struct Mark {
    int stage;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  std::vector<Mark> marks;
  double ms[kStages] = {};
  int64_t launches[kStages] = {};
  double work[kStages] = {};
  double issued_tc = 0;  // MACs issued to the tensor cores, padding included
  int64_t finds = 0;
  ~Profiler() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
  cudaEvent_t event() {
    if (used == pool.size()) {
      cudaEvent_t e;
      check(cudaEventCreate(&e), "cudaEventCreate");
      pool.push_back(e);
    }
    return pool[used++];
  }
  int open(int stage, cudaStream_t s) {
    if (!on) return -1;
    Mark m{stage, event(), event()};
    check(cudaEventRecord(m.a, s), "cudaEventRecord");
    marks.push_back(m);
    return int(marks.size()) - 1;
  }
  void close(int i, cudaStream_t s) {
    if (i >= 0) check(cudaEventRecord(marks[size_t(i)].b, s), "cudaEventRecord");
  }
  // after the stream has synchronised
  void collect() {
    for (const Mark& m : marks) {
      float t = 0;
      if (cudaEventElapsedTime(&t, m.a, m.b) == cudaSuccess) ms[m.stage] += t;
    }
    marks.clear();
    used = 0;
  }
  void reset() {
    marks.clear();
    used = 0;
    for (int i = 0; i < kStages; ++i) ms[i] = 0, launches[i] = 0, work[i] = 0;
    issued_tc = 0;
    finds = 0;
  }
};
thread_local Profiler t_prof;

struct Span {
  int index;
  cudaStream_t stream;
  Span(int stage, cudaStream_t s, int nlaunch = 1) : stream(s) {
    index = t_prof.open(stage, s);
    t_prof.launches[stage] += nlaunch;
  }
  ~Span() { t_prof.close(index, stream); }
};

// ----------------------------------------------------- merged tensor-core launches
// The tensor-core correlation launches of the finds a batched call keeps in
// flight, merged: each find (one host thread, its own stream) submits its
// tracking step or coarse scan as a job and waits; when every member thread
// of the batch is waiting, the jobs are launched together, one
// tc_track_kernel per launch shape (jobs of the same plan share it), after
// the events of the jobs' streams, and each stream then waits for its
// launch.  A member that will submit nothing more leaves.  A single launch
// then covers the tiles of all finds in flight: its blocks stay busy and its
// tail is one launch's instead of one per find.  Statistics of the merged
// launches (CUDA events on the batcher's stream) serve the measurement.
class TcBatcher {
 public:
  struct Stats {
    double ms = 0;
    int64_t launches = 0, jobs = 0;
    double macs = 0, issued = 0;  // algorithmic / issued multiply-adds of the merged jobs' finds
  };

  // Tensor-core work of a completed find of the batch.
  void add_work(double macs, double issued) {
    std::lock_guard<std::mutex> lk(m_);
    macs_ += macs;
    issued_ += issued;
  }

  // Start of a batch: `members` threads on `device` (current).
  void begin(int members, int device, int sm_count) {
    std::lock_guard<std::mutex> lk(m_);
    members_ = members;
    waiting_ = 0;
    pending_.clear();
    sm_count_ = sm_count;
    if (device_ != device) {
      device_ = device;
      check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
      jobs_.reserve(size_t(kTcMaxJobs) * kDoneSlots);
      next_.reserve(kDoneSlots);
      for (int i = 0; i < 2 * kDoneSlots; ++i) check(cudaEventCreateWithFlags(&done_[i], cudaEventDisableTiming), "event");
    }
  }

  // One find's launch: returns once it is enqueued; `s` then waits for it.
  // `ready` is recorded on `s` (the job's inputs are complete there).
  void submit(const TcArgs& job, size_t smem, cudaStream_t s, cudaEvent_t ready) {
    check(cudaEventRecord(ready, s), "cudaEventRecord");
    std::unique_lock<std::mutex> lk(m_);
    Pending p{job, smem, ready, nullptr};
    pending_.push_back(&p);
    const uint64_t round = round_;
    if (++waiting_ >= members_) {
      launch_locked();
    } else {
      // a member that never arrives would stall the others: after a minute
      // the waiting jobs are launched without it
      if (!cv_.wait_for(lk, std::chrono::seconds(60), [&] { return round_ != round; })) launch_locked();
    }
    if (p.error) raise(kInternal, p.error);
    check(cudaStreamWaitEvent(s, p.done, 0), "cudaStreamWaitEvent");
  }

  // A member that submits no more jobs.
  void leave() {
    std::lock_guard<std::mutex> lk(m_);
    --members_;
    if (waiting_ > 0 && waiting_ >= members_) launch_locked();
  }

  // Event time, launches and jobs of the merged launches since begin(); waits
  // for them.
  Stats stats() {
    std::lock_guard<std::mutex> lk(m_);
    Stats st;
    st.ms = folded_ms_;
    for (auto& t : timing_) {
      float ms = 0;
      if (cudaEventSynchronize(t.second) == cudaSuccess && cudaEventElapsedTime(&ms, t.first, t.second) == cudaSuccess)
        st.ms += ms;
    }
    st.launches = launches_;
    st.jobs = jobs_count_;
    st.macs = macs_;
    st.issued = issued_;
    return st;
  }
  void reset_stats() {
    std::lock_guard<std::mutex> lk(m_);
    launches_ = jobs_count_ = 0;
    macs_ = issued_ = 0;
    folded_ms_ = 0;
    for (auto& t : timing_) {
      cudaEventDestroy(t.first);
      cudaEventDestroy(t.second);
    }
    timing_.clear();
  }

 private:
  static constexpr int kDoneSlots = 8;  // launches per round (distinct shapes) before slots repeat
  struct Pending {
    TcArgs job;
    size_t smem;
    cudaEvent_t ready, done;
    const char* error = nullptr;
  };

  // Keeps the timing events bounded: past 1024 launches since the last
  // reset, the oldest 512 (long complete) are summed and released.
  void fold_timing_locked() {
    if (timing_.size() <= 1024) return;
    for (size_t i = 0; i < 512; ++i) {
      float ms = 0;
      if (cudaEventSynchronize(timing_[i].second) == cudaSuccess &&
          cudaEventElapsedTime(&ms, timing_[i].first, timing_[i].second) == cudaSuccess)
        folded_ms_ += ms;
      cudaEventDestroy(timing_[i].first);
      cudaEventDestroy(timing_[i].second);
    }
    timing_.erase(timing_.begin(), timing_.begin() + 512);
  }

  // Launches every pending job, grouped by launch shape (at most kTcMaxJobs
  // a launch), and wakes the waiters.  Done events alternate between two
  // halves by round: a round's events are re-recorded two rounds later, when
  // every waiter of that round has passed its cudaStreamWaitEvent.
  void launch_locked() {
    std::vector<Pending*> todo;
    todo.swap(pending_);
    std::stable_sort(todo.begin(), todo.end(), [](const Pending* x, const Pending* y) {
      return std::make_tuple(x->smem, x->job.stages, x->job.stage_bytes, x->job.abuf_bytes, x->job.sets,
                             x->job.npad) < std::make_tuple(y->smem, y->job.stages, y->job.stage_bytes,
                                                            y->job.abuf_bytes, y->job.sets, y->job.npad);
    });
    int slot = 0;
    const int half = int(round_ & 1) * kDoneSlots;
    for (size_t b = 0; b < todo.size();) {
      size_t e = b + 1;
      auto same = [&](const Pending* x) {
        const Pending* y = todo[b];
        return x->smem == y->smem && x->job.stages == y->job.stages && x->job.stage_bytes == y->job.stage_bytes &&
               x->job.abuf_bytes == y->job.abuf_bytes && x->job.sets == y->job.sets && x->job.npad == y->job.npad;
      };
      while (e < todo.size() && e - b < size_t(kTcMaxJobs) && same(todo[e])) ++e;
      const char* err = nullptr;
      if (slot >= kDoneSlots) {
        err = "tensor-core batch: too many launch shapes in one round";
      } else {
        std::vector<TcArgs> jobs;
        for (size_t i = b; i < e; ++i) {
          jobs.push_back(todo[i]->job);
          if (cudaStreamWaitEvent(stream_, todo[i]->ready, 0) != cudaSuccess) err = "cudaStreamWaitEvent";
        }
        TcArgs* dev_jobs = jobs_.p + size_t(slot) * kTcMaxJobs;
        // pageable source: staged by the driver before the call returns
        if (!err && cudaMemcpyAsync(dev_jobs, jobs.data(), jobs.size() * sizeof(TcArgs), cudaMemcpyHostToDevice,
                                    stream_) != cudaSuccess)
          err = "tensor-core batch: job upload";
        cudaEvent_t t0 = nullptr, t1 = nullptr;
        if (!err) {
          cudaEventCreate(&t0);
          cudaEventCreate(&t1);
          cudaEventRecord(t0, stream_);
          TcLaunch l{};
          l.jobs = dev_jobs;
          l.njobs = int(jobs.size());
          l.next = next_.p + slot;
          if (launch_tc_track(l, todo[b]->smem, std::min(kTcMaxTiles, sm_count_ * kTcBlocksPerSm), stream_) !=
              cudaSuccess)
            err = "tensor-core batch: launch";
          cudaEventRecord(t1, stream_);
          timing_.emplace_back(t0, t1);
          fold_timing_locked();
          ++launches_;
          jobs_count_ += int64_t(jobs.size());
        }
        if (!err && cudaEventRecord(done_[half + slot], stream_) != cudaSuccess) err = "cudaEventRecord";
      }
      for (size_t i = b; i < e; ++i) {
        todo[i]->done = done_[half + std::min(slot, kDoneSlots - 1)];
        todo[i]->error = err;
      }
      ++slot;
      b = e;
    }
    waiting_ = 0;
    ++round_;
    cv_.notify_all();
  }

  std::mutex m_;
  std::condition_variable cv_;
  int members_ = 0, waiting_ = 0, device_ = -1, sm_count_ = 1;
  uint64_t round_ = 0;
  std::vector<Pending*> pending_;
  cudaStream_t stream_ = nullptr;
  DevBuf<TcArgs> jobs_;
  DevBuf<int> next_;
  cudaEvent_t done_[2 * kDoneSlots] = {};
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timing_;
  double folded_ms_ = 0;  // event time of launches whose events were released
  int64_t launches_ = 0, jobs_count_ = 0;
  double macs_ = 0, issued_ = 0;
};

// Cohorts of a batch's workers: worker w merges with the workers of cohort
// w mod cohorts only, so cohorts drift out of phase and one cohort's
// merged launch overlaps other cohorts' other kernels.
constexpr int kMaxCohorts = 16;
TcBatcher& tc_batcher(int cohort) {
  static TcBatcher* b = new TcBatcher[kMaxCohorts];  // live with the find pool's threads
  return b[cohort];
}

// The batcher of this thread's finds (worker threads of a batched call), or none.
thread_local TcBatcher* t_batcher = nullptr;

struct Match {
  double row, col, angle, score;
};

struct FindOutput {
  std::vector<Match> matches;
  std::vector<Match> stage;   // requested stage dump
};

constexpr double kMissing = -std::numeric_limits<double>::infinity();

void fetch_stage(Workspace& ws, cudaStream_t s, const Cand* src, int slot, FindOutput& out) {
  t_prof.marks.clear();
  t_prof.used = 0;
  check(cudaMemcpyAsync(ws.h_state, ws.state.p, sizeof(QueryState), cudaMemcpyDeviceToHost, s), "state");
  check(cudaStreamSynchronize(s), "sync");
  const int n = slot < 0 ? ws.h_state->sorted_count : std::min(ws.h_state->count[slot], ws.h_state->cap);
  std::vector<Cand> h(size_t(std::max(n, 0)));
  if (n > 0) check(cudaMemcpyAsync(h.data(), src, size_t(n) * sizeof(Cand), cudaMemcpyDeviceToHost, s), "stage");
  check(cudaStreamSynchronize(s), "sync");
  for (const Cand& c : h) out.stage.push_back({c.row, c.col, c.angle, c.score});
}

// The caller's search domain (a W x H mask, nonzero inside) as the
// reference's region: runs in (row, begin) order, first run per row, area,
// bounding box and the sparse flag of matcher.cpp:505.
struct DomainHost {
  std::vector<int4> runs;
  std::vector<int32_t> row_run;
  int64_t area = 0;
  int64_t rmin = 0, rmax = -1, cmin = 0, cmax = -1;
  bool sparse = false;
};

DomainHost scan_domain(const uint8_t* mask, int64_t W, int64_t H) {
  DomainHost d;
  d.row_run.resize(size_t(H) + 1);
  d.rmin = H;
  d.cmin = W;
  for (int64_t r = 0; r < H; ++r) {
    d.row_run[size_t(r)] = int32_t(d.runs.size());
    const uint8_t* row = mask + r * W;
    int64_t c = 0;
    while (c < W) {
      while (c < W && !row[c]) ++c;
      if (c >= W) break;
      const int64_t b = c;
      while (c < W && row[c]) ++c;
      d.runs.push_back(make_int4(int(r), int(b), int(c - 1), 0));
      d.area += c - b;
      d.rmin = std::min(d.rmin, r);
      d.rmax = std::max(d.rmax, r);
      d.cmin = std::min(d.cmin, b);
      d.cmax = std::max(d.cmax, c - 1);
    }
  }
  d.row_run[size_t(H)] = int32_t(d.runs.size());
  if (d.area)
    d.sparse = double(d.area) < .7 * double(d.rmax - d.rmin + 1) * double(d.cmax - d.cmin + 1);
  return d;
}

// The device error flag of a find: the pyramid's exact-float check
// (Unsupported) or a tensor-core wait that ran out (Internal).
[[noreturn]] void raise_device_error(int32_t status) {
  raise(status, status == kInternal ? "tensor-core correlation: a pipeline wait ran out (device error flag)"
                                    : "pyramid sums exceed the exact float range");
}

// A find's tensor-core launch: merged with the other finds of a batched
// call (TcBatcher), or on its own stream.
void tc_launch(Workspace& ws, const TcArgs& job, size_t smem, cudaStream_t s) {
  if (t_batcher) {
    t_batcher->submit(job, smem, s, ws.tc_ready);
    return;
  }
  TcLaunch l{};
  l.jobs = nullptr;
  l.njobs = 1;
  l.next = &ws.tc_tiles.p->next;
  l.single = job;
  check(launch_tc_track(l, smem, std::min(kTcMaxTiles, ws.sm_count * kTcBlocksPerSm), s), "tc track");
}

// One model's query prepared for a multi-model selection
// (matcher.cpp:1077-1101): its sorted candidates with finite scores and what
// refining one of them needs.  The refinement reads the workspace's pyramid,
// which every model of one image shares (same crop, same levels).
struct Prepared {
  RefineArgs ra;               // candidate buffers are set per launch
  RectGeom geom;               // the model's level-0 box (make_rect)
  int finest = 0;
  std::vector<Cand> cands;
  DevBuf<int32_t> plist0;      // own copies of the level-0 query tables
  DevBuf<PosRange> ranges0;
  // with a reduced domain each model crops the image differently: own
  // copies of the refinement's images
  bool owned = false;
  DevBuf<float> lev0, fine;
  DevBuf<uint32_t> pairs;
};

// One find on the current device.  stage >= 0 stops after that stage and
// returns its candidate list.  With `prep`, the find stops after the sort and
// fills *prep instead of selecting.
FindOutput run_find(mvg_ncc_model_s& m, const void* pixels, int type, int64_t W, int64_t H, int64_t stride,
                    int location, const uint8_t* domain, const FindParams& req, cudaStream_t user_stream, int stage,
                    Prepared* prep = nullptr) {
  FindOutput out;
  const HostModel& hm = m.host;
  // src/ncc_matching/matcher.cpp:349-374 (validation and range clipping)
  if (type != 0 && type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
  if (!pixels) raise(kInvalidArgument, "image pixels must not be null");
  if (hm.levels.empty()) raise(kInvalidState, "model is empty");
  if (req.highest < 0 || req.lowest < 1) raise(kInvalidArgument, "invalid pyramid levels");
  const size_t level_count = req.highest ? std::min(hm.levels.size(), size_t(req.highest)) : hm.levels.size();
  const size_t finest = std::min(size_t(req.lowest), level_count) - 1;
  FindParams opt = req;
  if (!std::isfinite(opt.angle_start) || !std::isfinite(opt.angle_extent) || opt.angle_extent < 0 ||
      !std::isfinite(opt.min_score) || opt.min_score < 0 || opt.min_score > 1 || !std::isfinite(opt.max_overlap) ||
      opt.max_overlap < 0 || opt.max_overlap > 1 || opt.num_matches < 0)
    raise(kInvalidArgument, "invalid query range, score, overlap or candidate budget");
  const double angle_end = opt.angle_start + opt.angle_extent;  // unclipped, as the reference
  if (!std::isfinite(angle_end)) raise(kInvalidArgument, "query angle range must be finite");
  const double cs = std::max(opt.angle_start, hm.params.angle_start);
  const double ce = std::min(angle_end, hm.params.angle_start + hm.params.angle_extent);
  if (cs > ce + 1e-12) return out;
  opt.angle_start = cs;
  opt.angle_extent = std::max(0., ce - cs);
  if (W <= 0 || H <= 0 || W > std::numeric_limits<int>::max() || H > std::numeric_limits<int>::max() ||
      H > thread_budgets().pixels / W)
    raise(kLimitExceeded, "search image exceeds pixel budget");
  const int64_t bpp = type == 1 ? 2 : 1;
  if (stride < W * bpp || stride % bpp) raise(kInvalidArgument, "invalid row stride");

  // search domain (matcher.cpp:375-382): the whole image, or the caller's
  // mask; an empty domain finds nothing
  DomainHost dh;
  if (domain) {
    dh = scan_domain(domain, W, H);
    if (dh.area == 0) return out;
  } else {
    dh.rmin = 0;
    dh.rmax = H - 1;
    dh.cmin = 0;
    dh.cmax = W - 1;
  }
  // crop of the domain's box with halo on the pyramid lattice (matcher.cpp:383-393)
  const ModelLevel& base = hm.levels.front();
  const double radius = std::hypot(std::max(base.orow, double(base.height - 1) - base.orow),
                                   std::max(base.ocol, double(base.width - 1) - base.ocol));
  const int64_t lattice = int64_t(size_t{1} << (level_count - 1));
  const int64_t halo = int64_t(std::ceil(radius)) + 4 * lattice;
  const int64_t crop_row = std::max<int64_t>(0, dh.rmin - halo) / lattice * lattice;
  const int64_t crop_col = std::max<int64_t>(0, dh.cmin - halo) / lattice * lattice;
  const int64_t crop_bottom = std::min<int64_t>(H, ((dh.rmax + halo) / lattice + 1) * lattice);
  const int64_t crop_right = std::min<int64_t>(W, ((dh.cmax + halo) / lattice + 1) * lattice);

  Workspace& ws = workspace();
  cudaStream_t s = user_stream ? user_stream : ws.own_stream;
  // candidate budget and the list buffers it sizes
  const int cap = thread_budgets().candidates;
  const int slots = hash_slots(cap);
  for (DevBuf<Cand>* b : {&ws.cand_a, &ws.cand_b, &ws.tmp, &ws.sorted, &ws.accepted}) b->reserve(size_t(cap));
  ws.aux.reserve(size_t(cap));
  ws.accepted_aux.reserve(size_t(cap));
  ws.tested.reserve(size_t(cap));
  ws.sup.reserve(size_t(cap));
  ws.refined.reserve(size_t(cap));
  ws.refined_flag.reserve(size_t(cap));
  ws.table.reserve(size_t(slots));
  // Planning reads (and may extend) the model's endpoint rasters: serialise
  // it per model and snapshot the device views used by this find.
  std::unique_lock<std::mutex> lock(m.mutex);
  ensure_device(m);
  LevelView views[kMaxLevels];

  // query patch lists (matcher.cpp:463-482)
  std::vector<LevelPlan> plan(level_count);
  for (size_t li = 0; li < level_count; ++li) {
    DevLevel& L = *m.levels[li];
    auto& list = plan[li].plist;
    for (size_t p = 0; p < L.model_patches; ++p)
      if (L.angles[p] >= opt.angle_start - 1e-12 && L.angles[p] <= angle_end + 1e-12) list.push_back(int32_t(p));
    for (const double a : {opt.angle_start, angle_end}) {
      bool found = false;
      for (int32_t p : list)
        if (std::abs(L.angles[size_t(p)] - a) < 1e-12) found = true;
      if (found) continue;
      const int e = endpoint_patch(m, li, a);
      if (e >= 0) list.push_back(e);
    }
  }
  const size_t top = level_count - 1;
  const double coarse_radius = .5 * std::hypot(double(hm.levels[top].width), double(hm.levels[top].height));
  const size_t angle_stride = std::max<size_t>(1, size_t(std::min(double(plan[top].plist.size()),
      std::ceil(.5 / std::max(1e-20, coarse_radius * hm.params.angle_step)))));
  {
    auto& ca = plan[top].plist;
    const DevLevel& L = *m.levels[top];
    std::sort(ca.begin(), ca.end(), [&](int32_t x, int32_t y) { return L.angles[size_t(x)] < L.angles[size_t(y)]; });
    size_t kept = 0;
    for (size_t i = 0; i < ca.size(); ++i)
      if (i % angle_stride == 0 || i + 1 == ca.size()) ca[kept++] = ca[i];
    ca.resize(kept);
  }
  // level geometry of the crop
  int lw[kMaxLevels], lh[kMaxLevels];
  lw[0] = int(crop_right - crop_col);
  lh[0] = int(crop_bottom - crop_row);
  for (size_t l = 1; l < level_count; ++l) {
    lw[l] = std::max(1, lw[l - 1] / 2);
    lh[l] = std::max(1, lh[l - 1] / 2);
  }
  // position ranges per level and patch
  const double Hd = double(H), Wd = double(W);
  for (size_t li = 0; li < level_count; ++li) {
    const DevLevel& L = *m.levels[li];
    const double step = std::ldexp(1., int(li)), off = (step - 1) * .5;
    for (int32_t p : plan[li].plist) {
      const PatchDesc& d = L.desc[size_t(p)];
      PosRange rg;
      rg.r0 = std::max(0, -d.rmin);
      rg.r1 = lh[li] - d.rmax;
      rg.c0 = std::max(0, -d.cmin);
      rg.c1 = lw[li] - d.cmax;
      if (li == top) {
        // coarse scan bounds (matcher.cpp:549-553)
        const double margin = step == 1 ? .5 : 2 * step;
        rg.r0 = std::max(rg.r0, int(std::ceil((double(dh.rmin) - margin - double(crop_row) - off) / step - d.orow)));
        rg.r1 = std::min(rg.r1,
                         int(std::floor((double(dh.rmax) + margin - double(crop_row) - off) / step - d.orow)) + 1);
        rg.c0 = std::max(rg.c0, int(std::ceil((double(dh.cmin) - margin - double(crop_col) - off) / step - d.ocol)));
        rg.c1 = std::min(rg.c1,
                         int(std::floor((double(dh.cmax) + margin - double(crop_col) - off) / step - d.ocol)) + 1);
      }
      if (rg.r1 < rg.r0) rg.r1 = rg.r0;
      if (rg.c1 < rg.c0) rg.c1 = rg.c0;
      pose_interval(rg.r0, rg.r1, double(crop_row), step, d.orow, off, double(dh.rmin), double(dh.rmax));
      pose_interval(rg.c0, rg.c1, double(crop_col), step, d.ocol, off, double(dh.cmin), double(dh.cmax));
      plan[li].ranges.push_back(rg);
    }
  }

  // angle windows of the tracking steps (matcher.cpp:680): for target level
  // t, the source is level t+1; the first step from the top level widens the
  // window by the coarse angle stride
  bool exact32 = std::max(W, H) <= 8192 && level_count <= 5;
  for (size_t t = 0; t + 1 < level_count; ++t) {
    const DevLevel& S = *m.levels[t + 1];
    const DevLevel& T = *m.levels[t];
    const double limit = hm.params.angle_step * double(t + 1 == top ? angle_stride : 1) * 1.01;
    auto& off = plan[t].sel_off;
    auto& idx = plan[t].sel_idx;
    off.assign(S.desc.size() + 1, 0);
    for (size_t src = 0; src < S.desc.size(); ++src) {
      off[src] = int32_t(idx.size());
      for (size_t j = 0; j < plan[t].plist.size(); ++j)
        if (!(std::abs(T.angles[size_t(plan[t].plist[j])] - S.angles[src]) > limit)) idx.push_back(int32_t(j));
    }
    off[S.desc.size()] = int32_t(idx.size());
  }
  for (size_t li = 0; li < level_count && exact32; ++li)
    for (int32_t p : plan[li].plist) {
      const PatchDesc& d = m.levels[li]->desc[size_t(p)];
      if (!lattice_exact32(d.orow) || !lattice_exact32(d.ocol)) exact32 = false;
    }
  // longest run of any patch per level (bounds a run's moment sums)
  int max_run[kMaxLevels] = {};
  for (size_t li = 0; li < level_count; ++li)
    for (const PatchDesc& d : m.levels[li]->desc) max_run[li] = std::max(max_run[li], d.cmax - d.cmin + 1);
  // tensor-core plans of the tracking steps (cached per target level)
  std::vector<std::shared_ptr<const TcPlan>> tc(level_count);
  if (t_path == 0) {
    const size_t budget = tc_smem_budget(ws.smem_optin);
    for (size_t t = std::max(finest, size_t(opt.subpixel ? 1 : 0)); t + 1 < level_count; ++t) {
      float offset = 0;
      const int parts = tc_parts(type, t, &offset);
      if (!parts) continue;
      DevLevel& T = *m.levels[t];
      const size_t nsrc = m.levels[t + 1]->desc.size();
      std::vector<int32_t> key{int32_t(parts), int32_t(nsrc), t_tc_lookahead};
      key.insert(key.end(), plan[t].plist.begin(), plan[t].plist.end());
      key.insert(key.end(), plan[t].sel_off.begin(), plan[t].sel_off.end());
      key.insert(key.end(), plan[t].sel_idx.begin(), plan[t].sel_idx.end());
      auto it = T.tc_plans.find(key);
      if (it == T.tc_plans.end()) {
        if (T.tc_plans.size() >= 32) T.tc_plans.clear();  // finds in flight keep their plans alive
        it = T.tc_plans.emplace(std::move(key), build_tc_plan(T, nsrc, plan[t], parts, offset, budget, t_tc_lookahead))
                 .first;
      }
      if (!it->second->groups.empty()) tc[t] = it->second;
    }
  }
  // tensor-core coarse scan: the kept coarse patches with their origin on the
  // lattice, 16 per virtual source; a lattice of pseudo-candidates at stride
  // 5 covers every top-level position (the rest stays on coarse_kernel)
  std::shared_ptr<const TcPlan> tc_coarse;
  std::vector<int32_t> vsel_off, vsel_idx;
  std::vector<uint8_t> coarse_skip(plan[top].plist.size(), 0);
  std::vector<int32_t> co_src(plan[top].plist.size(), -1), co_k(plan[top].plist.size(), 0);
  const int lat_r = (lh[top] + 4) / 5, lat_c = (lw[top] + 4) / 5;
  int coarse_nsrc = 0;
  if (t_path == 0) {
    float offset = 0;
    const int parts = tc_parts(type, top, &offset);
    DevLevel& T = *m.levels[top];
    std::vector<int32_t> elig;
    for (size_t j = 0; j < plan[top].plist.size(); ++j) {
      const PatchDesc& d = T.desc[size_t(plan[top].plist[j])];
      if (d.orow == 0 && d.ocol == 0) elig.push_back(int32_t(j));
    }
    vsel_off.push_back(0);
    for (size_t i = 0; i < elig.size(); i += kTcMaxP) {
      for (size_t k = i; k < std::min(elig.size(), i + kTcMaxP); ++k) vsel_idx.push_back(elig[k]);
      vsel_off.push_back(int32_t(vsel_idx.size()));
    }
    const size_t nsrc = vsel_off.size() - 1;
    const size_t ncand = nsrc * size_t(lat_r) * size_t(lat_c);
    if (parts && nsrc > 0 && ncand / kTcCands + nsrc + 1 <= size_t(kTcMaxTiles)) {
      LevelPlan vp;
      vp.plist = plan[top].plist;
      vp.sel_off = vsel_off;
      vp.sel_idx = vsel_idx;
      std::vector<int32_t> key{-1, int32_t(parts), int32_t(nsrc), t_tc_lookahead};
      key.insert(key.end(), vp.plist.begin(), vp.plist.end());
      key.insert(key.end(), vsel_off.begin(), vsel_off.end());
      key.insert(key.end(), vsel_idx.begin(), vsel_idx.end());
      const size_t budget = tc_smem_budget(ws.smem_optin);
      auto it = T.tc_plans.find(key);
      if (it == T.tc_plans.end()) {
        if (T.tc_plans.size() >= 32) T.tc_plans.clear();
        it = T.tc_plans.emplace(std::move(key), build_tc_plan(T, nsrc, vp, parts, offset, budget, t_tc_lookahead))
                 .first;
      }
      // every virtual source must have its group: the lattice covers them all
      bool all = !it->second->groups.empty();
      for (int32_t g : it->second->group_of_src) all = all && g >= 0;
      if (all) {
        tc_coarse = it->second;
        coarse_nsrc = int(nsrc);
        for (size_t v = 0; v + 1 < vsel_off.size(); ++v)
          for (int32_t q = vsel_off[v]; q < vsel_off[v + 1]; ++q) {
            const size_t j = size_t(vsel_idx[size_t(q)]);
            coarse_skip[j] = 1;
            co_src[j] = int32_t(v);
            co_k[j] = q - vsel_off[v];
          }
      }
    }
  }
  const size_t finest_level = finest;
  const OriginalView orig = finest_level ? coarse_original(m, finest_level).view() : m.original.view();
  for (size_t li = 0; li < level_count; ++li) views[li] = m.levels[li]->view();
  std::vector<PatchDesc> top_desc(m.levels[top]->desc);
  lock.unlock();

  // upload image and query tables (one pinned copy for the tables)
  const void* dev_pixels = pixels;
  int64_t pitch_elems = stride / bpp;
  if (location == MVG_MEMORY_HOST) {
    const size_t bytes = size_t(stride) * size_t(H - 1) + size_t(W * bpp);
    ws.image.reserve(bytes);
    Span sp(kStUpload, s, 0);
    check(cudaMemcpyAsync(ws.image.p, pixels, bytes, cudaMemcpyHostToDevice, s), "image upload");
    dev_pixels = ws.image.p;
  }
  const int32_t* d_plist[kMaxLevels];
  const PosRange* d_ranges[kMaxLevels];
  const int32_t* d_sel_off[kMaxLevels];
  const int32_t* d_sel_idx[kMaxLevels];
  const TcGroup* d_tc_groups[kMaxLevels];
  const int32_t* d_tc_gsrc[kMaxLevels];
  const int32_t *d_co_src = nullptr, *d_co_k = nullptr, *d_co_gsrc = nullptr;
  const TcGroup* d_co_groups = nullptr;
  const uint8_t* d_co_skip = nullptr;
  {
    size_t total = 0;
    std::vector<size_t> at(4 * level_count);
    auto reserve = [&](size_t k, size_t bytes) {
      at[k] = total;
      total += (bytes + 15) & ~size_t(15);
    };
    for (size_t li = 0; li < level_count; ++li) {
      reserve(4 * li, plan[li].plist.size() * sizeof(int32_t));
      reserve(4 * li + 1, plan[li].ranges.size() * sizeof(PosRange));
      reserve(4 * li + 2, plan[li].sel_off.size() * sizeof(int32_t));
      reserve(4 * li + 3, plan[li].sel_idx.size() * sizeof(int32_t));
    }
    std::vector<size_t> tc_at(2 * level_count);
    for (size_t li = 0; li < level_count; ++li) {
      tc_at[2 * li] = total;
      total += tc[li] ? (tc[li]->groups.size() * sizeof(TcGroup) + 15) & ~size_t(15) : 0;
      tc_at[2 * li + 1] = total;
      total += tc[li] ? (tc[li]->group_of_src.size() * sizeof(int32_t) + 15) & ~size_t(15) : 0;
    }
    // tensor-core coarse scan: virtual sources, groups, skip flags
    size_t co_at[5] = {0, 0, 0, 0, 0};
    if (tc_coarse) {
      const size_t sizes[5] = {co_src.size() * sizeof(int32_t), co_k.size() * sizeof(int32_t),
                               tc_coarse->groups.size() * sizeof(TcGroup),
                               tc_coarse->group_of_src.size() * sizeof(int32_t), coarse_skip.size()};
      for (int q = 0; q < 5; ++q) {
        co_at[q] = total;
        total += (sizes[q] + 15) & ~size_t(15);
      }
    }
    uint8_t* h = ws.stage_tables(std::max<size_t>(total, 16));
    if (tc_coarse) {
      std::memcpy(h + co_at[0], co_src.data(), co_src.size() * sizeof(int32_t));
      std::memcpy(h + co_at[1], co_k.data(), co_k.size() * sizeof(int32_t));
      std::memcpy(h + co_at[2], tc_coarse->groups.data(), tc_coarse->groups.size() * sizeof(TcGroup));
      std::memcpy(h + co_at[3], tc_coarse->group_of_src.data(), tc_coarse->group_of_src.size() * sizeof(int32_t));
      std::memcpy(h + co_at[4], coarse_skip.data(), coarse_skip.size());
      d_co_src = reinterpret_cast<const int32_t*>(ws.tables.p + co_at[0]);
      d_co_k = reinterpret_cast<const int32_t*>(ws.tables.p + co_at[1]);
      d_co_groups = reinterpret_cast<const TcGroup*>(ws.tables.p + co_at[2]);
      d_co_gsrc = reinterpret_cast<const int32_t*>(ws.tables.p + co_at[3]);
      d_co_skip = reinterpret_cast<const uint8_t*>(ws.tables.p + co_at[4]);
    }
    for (size_t li = 0; li < level_count; ++li) {
      std::memcpy(h + at[4 * li], plan[li].plist.data(), plan[li].plist.size() * sizeof(int32_t));
      std::memcpy(h + at[4 * li + 1], plan[li].ranges.data(), plan[li].ranges.size() * sizeof(PosRange));
      std::memcpy(h + at[4 * li + 2], plan[li].sel_off.data(), plan[li].sel_off.size() * sizeof(int32_t));
      std::memcpy(h + at[4 * li + 3], plan[li].sel_idx.data(), plan[li].sel_idx.size() * sizeof(int32_t));
      d_plist[li] = reinterpret_cast<const int32_t*>(ws.tables.p + at[4 * li]);
      d_ranges[li] = reinterpret_cast<const PosRange*>(ws.tables.p + at[4 * li + 1]);
      d_sel_off[li] = reinterpret_cast<const int32_t*>(ws.tables.p + at[4 * li + 2]);
      d_sel_idx[li] = reinterpret_cast<const int32_t*>(ws.tables.p + at[4 * li + 3]);
      if (tc[li]) {
        std::memcpy(h + tc_at[2 * li], tc[li]->groups.data(), tc[li]->groups.size() * sizeof(TcGroup));
        std::memcpy(h + tc_at[2 * li + 1], tc[li]->group_of_src.data(),
                    tc[li]->group_of_src.size() * sizeof(int32_t));
      }
      d_tc_groups[li] = reinterpret_cast<const TcGroup*>(ws.tables.p + tc_at[2 * li]);
      d_tc_gsrc[li] = reinterpret_cast<const int32_t*>(ws.tables.p + tc_at[2 * li + 1]);
    }
    check(cudaMemcpyAsync(ws.tables.p, h, total, cudaMemcpyHostToDevice, s), "tables");
  }
  init_state(ws, s, cap);

  // search domain on the device (reduced domains only)
  DomainView dv{};
  dv.w = int(W);
  dv.h = int(H);
  dv.rmin = double(dh.rmin);
  dv.rmax = double(dh.rmax);
  dv.cmin = double(dh.cmin);
  dv.cmax = double(dh.cmax);
  if (domain) {
    const size_t px = size_t(W) * size_t(H);
    ws.dom_mask.reserve(px);
    check(cudaMemcpyAsync(ws.dom_mask.p, domain, px, cudaMemcpyHostToDevice, s), "domain");
    ws.dom_runs.upload(dh.runs, s);
    ws.dom_row_run.upload(dh.row_run, s);
    dv.mask = ws.dom_mask.p;
    dv.runs = ws.dom_runs.p;
    dv.row_run = ws.dom_row_run.p;
    dv.sparse = dh.sparse;
    if (dh.sparse) {
      ws.dom_count.reserve((size_t(W) + 1) * (size_t(H) + 1));
      check(launch_domain_count(ws.dom_mask.p, int(W), int(H), ws.dom_count.p, s), "domain count");
      dv.count = ws.dom_count.p;
    }
  }

  // pyramid (levels finest..top as needed; level 0 always feeds the rest)
  LevelImage lev[kMaxLevels];
  for (size_t l = 0; l < level_count; ++l) {
    ws.lev_v[l].reserve(size_t(lw[l]) * size_t(lh[l]));
    lev[l].v = ws.lev_v[l].p;
    lev[l].w = lw[l];
    lev[l].h = lh[l];
  }
  QueryState* st = ws.state.p;
  int32_t* err_flag = &st->error;
  // an fp16-exact level 0 that is also the finest: its half2 pairs come with it
  const bool pairs0 = finest == 0 && (type == 1 ? 65535.0 : 255.0) <= 2048.0;
  if (pairs0) ws.pairs.reserve(size_t(lw[0]) * size_t(lh[0]));
  {
    Span sp(kStPyramid, s, int(level_count));
    check(launch_pyramid0(dev_pixels, type, pitch_elems, int(crop_row), int(crop_col), lev[0], err_flag, s,
                          pairs0 ? ws.pairs.p : nullptr),
          "pyramid0");
    for (size_t l = 1; l < level_count; ++l) check(launch_pyramid(lev[l - 1], lev[l], err_flag, s), "pyramid");
    // uint16: the tensor-core planes are centred on the data's own range
    // (a 12-bit image sits far below the type's mid-range)
    if (type == 1) check(launch_level_range(lev[0], st, s), "level range");
  }
  const size_t first_target = std::max(finest, size_t(opt.subpixel ? 1 : 0));
  for (size_t l = 0; l < level_count; ++l) {
    const bool need = l == top || (l + 1 <= top && l >= first_target);
    if (!need) continue;
    ws.lev_p[l].reserve(size_t(lw[l] + 1) * size_t(lh[l]));
    lev[l].prefix = ws.lev_p[l].p;
    // 8-byte prefixes (uint32 modulo 2^32) when a run's sum of S^2 fits
    const double maxv = (type == 1 ? 65535.0 : 255.0) * std::ldexp(1., int(2 * l));
    lev[l].prefix32 =
        double(max_run[l]) * maxv * maxv < 4294967296.0 ? reinterpret_cast<uint2*>(ws.lev_p[l].p) : nullptr;
    Span sp(kStPrefix, s);
    check(launch_prefix(lev[l], s), "prefix");
  }

  // coarse scan + NMS
  const double scale = std::ldexp(1., int(top)), phase = (scale - 1) * .5;
  const int nplist = int(plan[top].plist.size());
  int max_bh = 0, max_bw = 0;
  for (int32_t p : plan[top].plist) {
    max_bh = std::max(max_bh, top_desc[size_t(p)].rmax - top_desc[size_t(p)].rmin);
    max_bw = std::max(max_bw, top_desc[size_t(p)].cmax - top_desc[size_t(p)].cmin);
  }
  ws.planes.reserve(size_t(std::max(nplist, 1)) * size_t(lw[top]) * size_t(lh[top]));
  if (tc_coarse) {
    // tensor-core scan of the rotated coarse patches into their planes
    const TcPlan& P = *tc_coarse;
    const int ncand = coarse_nsrc * lat_r * lat_c;
    const int pitch = (lw[top] + kTcPlaneMargin + 7) & ~7;
    const int slot_c = kMaxLevels + 1;
    ws.coarse_cand.reserve(size_t(ncand));
    ws.coarse_rc.reserve(size_t(ncand));
    ws.coarse_dots.reserve(size_t(ncand) * kTcScoreStride);
    ws.tc_planes.reserve(size_t(P.parts) * kTcPlaneShifts * size_t(lh[top]) * size_t(pitch));
    ws.tc_order.reserve(std::max(size_t(ncand), size_t(cap)));
    ws.tc_tiles.reserve(1);
    TcArgs tca{};
    tca.lev = lev[top];
    tca.in = ws.coarse_cand.p;
    tca.state = st;
    tca.state_rw = st;
    tca.in_slot = slot_c;
    tca.groups = d_co_groups;
    tca.group_of_src = d_co_gsrc;
    tca.tiles = ws.tc_tiles.p;
    tca.order = ws.tc_order.p;
    tca.dots = ws.coarse_dots.p;
    tca.step = scale;
    tca.offset = phase;
    tca.exact32 = 0;
    tca.stages = P.stages;
    tca.stage_bytes = P.stage_bytes;
    tca.abuf_bytes = P.abuf_bytes;
    tca.sets = P.sets;
    tca.npad = P.npad;
    tca.plane_offset = P.offset;
    tca.dyn_offset = type == 1;
    tca.level_mult = float(std::ldexp(1., int(2 * top)));
    tca.planes = ws.tc_planes.p;
    tca.plane_pitch = pitch;
    tca.rc = ws.coarse_rc.p;
    tca.error = &st->error;
    tca.withhold_weights = t_withhold_weights;
    {
      Span spp(kStTcPrep, s, 2);
      check(launch_tc_planes(lev[top], ws.tc_planes.p, pitch, P.parts, P.offset, s, type == 1 ? st : nullptr,
                             tca.level_mult),
            "tc planes");
      check(launch_coarse_lattice(ws.coarse_cand.p, ws.coarse_rc.p, coarse_nsrc, lat_r, lat_c, d_co_gsrc,
                                  ws.tc_order.p, ws.tc_tiles.p, st, slot_c, s),
            "coarse lattice");
    }
    {
      Span spt(kStTrackTc, s);
      tc_launch(ws, tca, tc_launch_smem(P, ws.smem_optin), s);
    }
    CoarseTcArgs cs;
    cs.lev = lev[top];
    cs.view = views[top];
    cs.plist = d_plist[top];
    cs.ranges = d_ranges[top];
    cs.nplist = nplist;
    cs.src_of = d_co_src;
    cs.k_of = d_co_k;
    cs.lat_r = lat_r;
    cs.lat_c = lat_c;
    cs.dots = ws.coarse_dots.p;
    cs.groups = d_co_groups;
    cs.group_of_src = d_co_gsrc;
    cs.planes = ws.planes.p;
    cs.absolute = hm.params.ignore_polarity;
    cs.dom = dv;
    cs.crop_row = double(crop_row);
    cs.crop_col = double(crop_col);
    cs.scale = scale;
    cs.phase = phase;
    Span sp(kStCoarse, s);
    check(launch_coarse_tc_score(cs, s), "coarse tc score");
  }
  if (nplist > 0) {
    CoarseArgs ca;
    ca.lev = lev[top];
    ca.view = views[top];
    ca.plist = d_plist[top];
    ca.ranges = d_ranges[top];
    ca.nplist = nplist;
    ca.planes = ws.planes.p;
    ca.absolute = hm.params.ignore_polarity;
    ca.skip = d_co_skip;
    ca.dom = dv;
    ca.crop_row = double(crop_row);
    ca.crop_col = double(crop_col);
    ca.scale = scale;
    ca.phase = phase;
    {
      Span sp(kStCoarse, s);
      const cudaError_t e = launch_coarse(ca, max_bh, max_bw, s, ws.smem_optin);
      if (e == cudaErrorInvalidConfiguration) raise(kUnsupported, "coarse template raster exceeds on-chip tile");
      check(e, "coarse");
    }
    for (int k = 0; k < nplist; ++k) {
      if (coarse_skip[size_t(k)]) continue;  // counted with the tensor-core work
      const PosRange& rg = plan[top].ranges[size_t(k)];
      t_prof.work[kStCoarse] += double(std::max(0, rg.r1 - rg.r0)) * double(std::max(0, rg.c1 - rg.c0)) *
                                double(top_desc[size_t(plan[top].plist[size_t(k)])].n);
    }
    NmsArgs na;
    na.planes = ws.planes.p;
    na.nplist = nplist;
    na.w = lw[top];
    na.h = lh[top];
    na.plist = d_plist[top];
    na.view = views[top];
    na.crop_row = double(crop_row);
    na.crop_col = double(crop_col);
    na.scale = scale;
    na.phase = phase;
    {
      // smallest float whose double value is >= 0.4*MinScore (the
      // reference's FP64 comparison, matcher.cpp:582)
      const double thr = opt.min_score * .4;
      float f = float(thr);
      if (double(f) < thr) f = std::nextafter(f, std::numeric_limits<float>::infinity());
      na.threshold = f;
    }
    na.out = ws.cand_a.p;
    na.state = st;
    na.max_candidates = cap;
    Span sp(kStNms, s);
    check(launch_nms(na, s), "nms");
  }
  if (stage == 0) {
    fetch_stage(ws, s, ws.cand_a.p, 0, out);
    if (ws.h_state->error) raise_device_error(ws.h_state->error);
    if (ws.h_state->overflow) raise(kLimitExceeded, "coarse candidate budget exceeded");
    return out;
  }

  // coarse-to-fine tracking (matcher.cpp:630-761)
  Cand* cur = ws.cand_a.p;
  Cand* nxt = ws.cand_b.p;
  int slot = 0, step_no = 0;
  for (size_t l = top; l > finest; --l) {
    const bool snap = l == 1 && opt.subpixel;
    if (!snap) {
      const size_t t = l - 1;
      TrackArgs ta;
      ta.lev = lev[t];
      ta.view = views[t];
      ta.plist = d_plist[t];
      ta.ranges = d_ranges[t];
      ta.nplist = int(plan[t].plist.size());
      ta.in = cur;
      ta.out = ws.tmp.p;
      ta.state = st;
      ta.in_slot = slot;
      ta.sel_off = d_sel_off[t];
      ta.sel_idx = d_sel_idx[t];
      ta.crop_row = double(crop_row);
      ta.crop_col = double(crop_col);
      ta.step = std::ldexp(1., int(t));
      ta.offset = (ta.step - 1) * .5;
      ta.exact32 = exact32;
      ta.absolute = hm.params.ignore_polarity;
      ta.tc_dots = nullptr;
      ta.tc_group_of_src = nullptr;
      ta.tc_groups = nullptr;
      ta.dom = dv;
      if (tc[t]) {
        const TcPlan& P = *tc[t];
        const int ng = int(P.groups.size());
        const int pitch = (lev[t].w + kTcPlaneMargin + 7) & ~7;
        ws.tc_dots.reserve(size_t(cap) * kTcScoreStride);
        ws.tc_planes.reserve(size_t(P.parts) * kTcPlaneShifts * size_t(lev[t].h) * size_t(pitch));
        ws.tc_order.reserve(size_t(cap));
        ws.tc_counts.reserve(size_t(ng));
        ws.tc_offsets.reserve(size_t(ng));
        ws.tc_cursor.reserve(size_t(ng));
        ws.tc_tiles.reserve(1);
        TcArgs tca;
        tca.lev = lev[t];
        tca.in = cur;
        tca.state = st;
        tca.state_rw = st;
        tca.in_slot = slot;
        tca.groups = d_tc_groups[t];
        tca.group_of_src = d_tc_gsrc[t];
        tca.tiles = ws.tc_tiles.p;
        tca.order = ws.tc_order.p;
        tca.dots = ws.tc_dots.p;
        tca.crop_row = double(crop_row);
        tca.crop_col = double(crop_col);
        tca.step = ta.step;
        tca.offset = ta.offset;
        tca.exact32 = exact32;
        tca.stages = P.stages;
        tca.stage_bytes = P.stage_bytes;
        tca.abuf_bytes = P.abuf_bytes;
        tca.sets = P.sets;
        tca.npad = P.npad;
        tca.plane_offset = P.offset;
        tca.dyn_offset = type == 1;
        tca.level_mult = float(std::ldexp(1., int(2 * t)));
        tca.planes = ws.tc_planes.p;
        tca.plane_pitch = pitch;
        tca.rc = nullptr;
        tca.error = &st->error;
        tca.withhold_weights = t_withhold_weights;
        {
          Span spp(kStTcPrep, s, 4);
          check(launch_tc_planes(lev[t], ws.tc_planes.p, pitch, P.parts, P.offset, s, type == 1 ? st : nullptr,
                                 tca.level_mult),
                "tc planes");
          check(launch_tc_group(tca, ng, ws.tc_counts.p, ws.tc_offsets.p, ws.tc_cursor.p, cap, s),
                "tc group");
        }
        {
          Span spt(kStTrackTc, s);
          tc_launch(ws, tca, tc_launch_smem(P, ws.smem_optin), s);
        }
        ta.tc_dots = ws.tc_dots.p;
        ta.tc_group_of_src = d_tc_gsrc[t];
        ta.tc_groups = d_tc_groups[t];
      }
      Span sp(kStTrack, s);
      check(launch_track(ta, cap, s, ws.smem_optin), "track");
    }
    check(cudaMemsetAsync(ws.table.p, 0xff, sizeof(int) * size_t(slots), s), "memset");
    DedupArgs da;
    da.in = snap ? cur : ws.tmp.p;
    da.out = nxt;
    da.table = ws.table.p;
    da.state = st;
    da.in_slot = slot;
    da.out_slot = slot + 1;
    da.threshold = snap ? kMissing : opt.min_score * .4;
    da.snap = snap;
    da.height = Hd;
    da.width = Wd;
    da.dom = dv;
    da.hash_slots = slots;
    {
      Span sp(kStDedup, s, snap ? 2 : 1);
      check(launch_dedup(da, cap, s), "dedup");
    }
    std::swap(cur, nxt);
    ++slot;
    ++step_no;
    if (stage == step_no) {
      fetch_stage(ws, s, cur, slot, out);
      return out;
    }
    if (snap) break;
  }

  // full-resolution score (matcher.cpp:813-822) and sort (824-827)
  const double fscale = std::ldexp(1., int(finest)), fphase = (fscale - 1) * .5;
  ImageView fine{lev[finest].v, lw[finest], lh[finest]};
  if ((type == 1 ? 65535.0 : 255.0) * std::ldexp(1., int(2 * finest)) <= 2048.0) {
    // fp16-exact level: half2 pairs halve the bilinear loads of the
    // continuous score and the Gauss-Newton passes
    if (!pairs0) {
      ws.pairs.reserve(size_t(lw[finest]) * size_t(lh[finest]));
      Span sp(kStScore, s, 1);
      check(launch_pairs(lev[finest].v, lw[finest], lh[finest], ws.pairs.p, s), "pairs");
    }
    fine.pairs = ws.pairs.p;
    ws.pairs_level = int(finest);
  }
  {
    ScoreArgs sa;
    sa.img = fine;
    sa.orig = orig;
    sa.cand = cur;
    sa.state = st;
    sa.slot = slot;
    sa.crop_row = double(crop_row);
    sa.crop_col = double(crop_col);
    sa.scale = fscale;
    sa.phase = fphase;
    sa.absolute = hm.params.ignore_polarity;
    {
      Span sp(kStScore, s);
      check(launch_score(sa, cap, s), "score");
    }
    SortArgs so;
    so.in = cur;
    so.out = ws.sorted.p;
    so.state = st;
    so.slot = slot;
    so.keys = nullptr;
    so.idx = nullptr;
    so.npow = 0;
    if (cap > kRankSortMax) {
      int np = 4096;
      while (np < cap) np <<= 1;
      ws.sort_keys.reserve(size_t(np));
      ws.sort_idx.reserve(size_t(np));
      so.keys = ws.sort_keys.p;
      so.idx = ws.sort_idx.p;
      so.npow = np;
    }
    Span sp(kStSort, s);
    check(launch_sort(so, cap, s), "sort");
  }
  if (stage == 100) {
    fetch_stage(ws, s, ws.sorted.p, -1, out);
    return out;
  }

  // greedy selection with refinement (matcher.cpp:1063-1076)
  check(cudaMemsetAsync(ws.refined_flag.p, 0, sizeof(int32_t) * size_t(cap), s), "memset");
  check(cudaMemsetAsync(ws.tested.p, 0, sizeof(int32_t) * size_t(cap), s), "memset");
  check(cudaMemsetAsync(ws.sup.p, 0, size_t(cap), s), "memset");
  // speculative refinement batch: the next NumMatches unsuppressed,
  // mutually non-overlapping candidates (32 when all matches are wanted)
  const int batch_limit = int(std::min<int64_t>(64, opt.num_matches > 0 ? opt.num_matches : 32));
  RectGeom geom;
  geom.left = -base.ocol - .5;
  geom.right = double(base.width) - base.ocol - .5;
  geom.top = -base.orow - .5;
  geom.bottom = double(base.height) - base.orow - .5;
  geom.area = double(base.width) * double(base.height);
  SelectArgs se;
  se.sorted = ws.sorted.p;
  se.aux = ws.aux.p;
  se.refined = ws.refined.p;
  se.refined_flag = ws.refined_flag.p;
  se.batch = ws.batch.p;
  se.accepted = ws.accepted.p;
  se.accepted_aux = ws.accepted_aux.p;
  se.tested = ws.tested.p;
  se.sup = ws.sup.p;
  se.state = st;
  se.batch_limit = batch_limit;
  se.num_matches = opt.num_matches;
  se.max_overlap = opt.max_overlap;
  se.geom = geom;
  RefineArgs ra;
  ra.img = fine;
  ra.orig = orig;
  ra.lev0 = lev[0];
  ra.view0 = views[0];
  ra.plist0 = d_plist[0];
  ra.ranges0 = d_ranges[0];
  ra.nplist0 = int(plan[0].plist.size());
  ra.sorted = ws.sorted.p;
  ra.refined = ws.refined.p;
  ra.refined_flag = ws.refined_flag.p;
  ra.batch = ws.batch.p;
  ra.state = st;
  ra.batch_count = -1;
  ra.crop_row = double(crop_row);
  ra.crop_col = double(crop_col);
  ra.scale = fscale;
  ra.phase = fphase;
  ra.angle_start = opt.angle_start;
  ra.angle_end = opt.angle_start + opt.angle_extent;
  ra.angle_step = hm.params.angle_step;
  ra.min_score = opt.min_score;
  ra.rotate = opt.angle_extent > 0;
  ra.subpixel = opt.subpixel;
  ra.absolute = hm.params.ignore_polarity;
  ra.top = int(top);
  ra.finest = int(finest);
  ra.height = Hd;
  ra.width = Wd;
  ra.dom = dv;
  ra.geom = geom;
  if (prep) {
    // multi-model selection: the sorted list to the host, the level-0 query
    // tables to buffers of the prepared query (the workspace's are reused)
    check(cudaMemcpyAsync(ws.h_state, st, sizeof(QueryState), cudaMemcpyDeviceToHost, s), "state");
    check(cudaStreamSynchronize(s), "sync");
    if (ws.h_state->error) raise_device_error(ws.h_state->error);
    if (ws.h_state->overflow) raise(kLimitExceeded, "coarse candidate budget exceeded");
    const int n = std::max(0, std::min(ws.h_state->sorted_count, cap));
    prep->cands.resize(size_t(n));
    if (n > 0)
      check(cudaMemcpyAsync(prep->cands.data(), ws.sorted.p, size_t(n) * sizeof(Cand), cudaMemcpyDeviceToHost, s),
            "sorted");
    prep->plist0.reserve(plan[0].plist.size());
    prep->ranges0.reserve(plan[0].ranges.size());
    if (!plan[0].plist.empty())
      check(cudaMemcpyAsync(prep->plist0.p, d_plist[0], plan[0].plist.size() * sizeof(int32_t),
                            cudaMemcpyDeviceToDevice, s), "plist0");
    if (!plan[0].ranges.empty())
      check(cudaMemcpyAsync(prep->ranges0.p, d_ranges[0], plan[0].ranges.size() * sizeof(PosRange),
                            cudaMemcpyDeviceToDevice, s), "ranges0");
    prep->ra = ra;
    if (domain) {
      const size_t n0 = size_t(lw[0]) * size_t(lh[0]), nf = size_t(lw[finest]) * size_t(lh[finest]);
      prep->owned = true;
      prep->lev0.reserve(n0);
      check(cudaMemcpyAsync(prep->lev0.p, lev[0].v, n0 * sizeof(float), cudaMemcpyDeviceToDevice, s), "lev0");
      prep->ra.lev0.v = prep->lev0.p;
      prep->ra.img.v = prep->lev0.p;
      if (finest) {
        prep->fine.reserve(nf);
        check(cudaMemcpyAsync(prep->fine.p, lev[finest].v, nf * sizeof(float), cudaMemcpyDeviceToDevice, s), "fine");
        prep->ra.img.v = prep->fine.p;
      }
      if (fine.pairs) {
        prep->pairs.reserve(nf);
        check(cudaMemcpyAsync(prep->pairs.p, fine.pairs, nf * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s),
              "pairs");
        prep->ra.img.pairs = prep->pairs.p;
      }
    }
    check(cudaStreamSynchronize(s), "sync");
    prep->ra.plist0 = prep->plist0.p;
    prep->ra.ranges0 = prep->ranges0.p;
    prep->geom = geom;
    prep->finest = int(finest);
    t_prof.collect();
    return out;
  }
  {
    Span sp(kStSelect, s, 2);
    check(launch_rects(ws.sorted.p, ws.aux.p, st, geom, cap, s), "rects");
    check(launch_select(se, s), "select");
  }
  // A round that accepts nothing (the candidates fail refinement or overlap)
  // makes the next speculative batch the widest (64) and doubles the rounds
  // queued per host check (up to 16): fewer host round trips while a quota
  // is far from met.  The matches do not depend on either: each candidate's
  // refinement is its own, the selection takes them in rank order, and the
  // rounds queued past the end of the selection return at once (done).
  int prepared = batch_limit;  // batch bound of the last select launched
  int accepted = 0;
  int ahead = 1;               // rounds queued per host check
  for (int round = 0; round < 100000; round += ahead) {
    for (int k = 0; k < ahead; ++k) {
      {
        Span sp(kStRefine, s);
        check(launch_refine(ra, prepared, s), "refine");
      }
      {
        Span sp(kStSelect, s);
        check(launch_select(se, s), "select");
      }
      prepared = se.batch_limit;
    }
    check(cudaMemcpyAsync(ws.h_state, st, sizeof(QueryState), cudaMemcpyDeviceToHost, s), "state");
    check(cudaStreamSynchronize(s), "find");
    if (ws.h_state->done || !ws.h_state->need) break;
    const bool none = ws.h_state->accepted == accepted;
    se.batch_limit = none ? 64 : batch_limit;
    ahead = none ? std::min(16, ahead * 2) : 1;
    accepted = ws.h_state->accepted;
  }
  const QueryState hs = *ws.h_state;
  t_prof.collect();
  t_prof.finds += 1;
  t_prof.work[kStTrack] += double(hs.track_macs);
  t_prof.work[kStTrackTc] += double(hs.tc_macs);
  t_prof.issued_tc += double(hs.tc_issued);
  t_prof.work[kStScore] += double(hs.count[slot]) * double(orig.n);
  if (t_batcher) t_batcher->add_work(double(hs.tc_macs), double(hs.tc_issued));
  // the device error flag first: after a failed kernel the later stages
  // read incomplete data (an overflow then is a consequence)
  if (hs.error) raise_device_error(hs.error);
  if (hs.overflow) raise(kLimitExceeded, "coarse candidate budget exceeded");
  std::vector<Cand> acc(size_t(hs.accepted));
  if (hs.accepted > 0) {
    check(cudaMemcpyAsync(acc.data(), ws.accepted.p, acc.size() * sizeof(Cand), cudaMemcpyDeviceToHost, s), "result");
    check(cudaStreamSynchronize(s), "result");
  }
  for (const Cand& c : acc) out.matches.push_back({c.row, c.col, c.angle, c.score});
  if (stage == -1) out.stage = out.matches;
  return out;
}

// ------------------------------------------------------------ FindNccModels
// Selection shared by all models (matching::Selection, src/matching/multi.hpp:14):
// -1 means "per model" (the control tuple held one value per model).
struct Selection {
  int64_t num_matches = -1;
  double max_overlap = -1;
};

struct Pt {
  double x, y;
};
using Quad = std::array<Pt, 4>;

// A pose's rotated template box (matching::box, src/matching/multi.hpp:50-55).
Quad pose_box(const RectGeom& g, double row, double col, double angle) {
  const double ca = std::cos(angle), sa = std::sin(angle);
  const Pt c[4] = {{g.left, g.top}, {g.right, g.top}, {g.right, g.bottom}, {g.left, g.bottom}};
  Quad q;
  for (int i = 0; i < 4; ++i) q[size_t(i)] = {col + ca * c[i].x + sa * c[i].y, row - sa * c[i].x + ca * c[i].y};
  return q;
}

struct Aabb {
  double top, bottom, left, right;
};
Aabb aabb_of(const Quad& q) {
  Aabb a{q[0].y, q[0].y, q[0].x, q[0].x};
  for (const Pt& p : q) {
    a.top = std::min(a.top, p.y);
    a.bottom = std::max(a.bottom, p.y);
    a.left = std::min(a.left, p.x);
    a.right = std::max(a.right, p.x);
  }
  return a;
}
bool apart(const Aabb& a, const Aabb& b) {
  return a.right < b.left || b.right < a.left || a.bottom < b.top || b.bottom < a.top;
}

double polygon_area(const Pt* p, size_t n) {
  double a = 0;
  for (size_t i = 0; i < n; ++i) {
    const Pt& u = p[i];
    const Pt& v = p[(i + 1) % n];
    a += u.x * v.y - v.x * u.y;
  }
  return std::abs(a) * .5;
}

// Intersection area of two boxes over the smaller box's area
// (matching::overlap, src/matching/multi.hpp:59-75): both boxes are moved to
// a's first corner, then a is clipped by each edge of b (Sutherland-Hodgman).
double box_overlap(Quad a, Quad b) {
  const Pt o = a[0];
  for (Pt& p : a) p = {p.x - o.x, p.y - o.y};
  for (Pt& p : b) p = {p.x - o.x, p.y - o.y};
  const double den = std::min(polygon_area(a.data(), 4), polygon_area(b.data(), 4));
  if (den <= 1e-12) return 0;
  std::array<Pt, 16> poly{}, next{};
  std::copy(a.begin(), a.end(), poly.begin());
  size_t n = 4;
  auto side = [](Pt u, Pt v, Pt p) { return (v.x - u.x) * (p.y - u.y) - (v.y - u.y) * (p.x - u.x); };
  for (int e = 0; e < 4 && n; ++e) {
    const Pt u = b[size_t(e)], v = b[size_t((e + 1) % 4)];
    size_t m = 0;
    for (size_t i = 0; i < n; ++i) {
      const Pt p = poly[i], q = poly[(i + 1) % n];
      const double dp = side(u, v, p), dq = side(u, v, q);
      if (dp >= 0) next[m++] = p;
      if ((dp >= 0) != (dq >= 0)) {
        const double t = dp / (dp - dq);
        next[m++] = {p.x + t * (q.x - p.x), p.y + t * (q.y - p.y)};
      }
    }
    poly = next;
    n = m;
  }
  return std::clamp(polygon_area(poly.data(), n) / den, 0., 1.);
}

struct MultiCand {
  Cand c;          // pose (refined once accepted)
  int model;       // index into the caller's model list
  int owner;       // model whose prepared query produced it
  int local;       // index in the owner's candidate list
};

bool ranks_before(const MultiCand& a, const MultiCand& b) {
  if (a.c.score != b.c.score) return a.c.score > b.c.score;
  if (a.model != b.model) return a.model < b.model;
  if (a.c.row != b.c.row) return a.c.row < b.c.row;
  if (a.c.col != b.c.col) return a.c.col < b.c.col;
  return a.c.angle < b.c.angle;
}

// Device refinement of host-chosen candidates, grouped by owner query, with
// the results memoised per (owner, candidate).
struct MultiRefiner {
  Workspace& ws;
  cudaStream_t s;
  std::vector<std::unique_ptr<Prepared>>& preps;
  std::vector<std::vector<Refined>> result;
  std::vector<std::vector<uint8_t>> done;
  DevBuf<Cand> d_cand;
  DevBuf<Refined> d_ref;
  DevBuf<int32_t> d_flag, d_iota;
  static constexpr int kMax = 64;

  MultiRefiner(Workspace& w, cudaStream_t st, std::vector<std::unique_ptr<Prepared>>& p)
      : ws(w), s(st), preps(p), result(p.size()), done(p.size()) {
    for (size_t i = 0; i < p.size(); ++i)
      if (p[i]) {
        result[i].resize(p[i]->cands.size());
        done[i].assign(p[i]->cands.size(), 0);
      }
    d_cand.reserve(kMax);
    d_ref.reserve(kMax);
    d_flag.reserve(kMax);
    d_iota.reserve(kMax);
    std::vector<int32_t> iota(kMax);
    for (int i = 0; i < kMax; ++i) iota[size_t(i)] = i;
    d_iota.upload(iota, s);
  }
  bool has(const MultiCand& m) const { return done[size_t(m.owner)][size_t(m.local)] != 0; }
  const Refined& get(const MultiCand& m) const { return result[size_t(m.owner)][size_t(m.local)]; }

  // refines `batch` (at most kMax, none refined yet) in one launch per owner
  void run(const std::vector<MultiCand>& batch) {
    std::vector<MultiCand> order(batch);
    std::stable_sort(order.begin(), order.end(), [](const MultiCand& a, const MultiCand& b) { return a.owner < b.owner; });
    const size_t n = order.size();
    std::vector<Cand> h(n);
    for (size_t i = 0; i < n; ++i) h[i] = preps[size_t(order[i].owner)]->cands[size_t(order[i].local)];
    check(cudaMemcpyAsync(d_cand.p, h.data(), n * sizeof(Cand), cudaMemcpyHostToDevice, s), "refine batch");
    for (size_t i = 0; i < n;) {
      size_t j = i;
      while (j < n && order[j].owner == order[i].owner) ++j;
      const Prepared& P = *preps[size_t(order[i].owner)];
      RefineArgs ra = P.ra;
      if (!P.owned && ra.img.pairs && ws.pairs_level != P.finest) ra.img.pairs = nullptr;  // another model's level
      ra.sorted = d_cand.p + i;
      ra.refined = d_ref.p + i;
      ra.refined_flag = d_flag.p + i;
      ra.batch = d_iota.p;
      ra.batch_count = int(j - i);
      {
        Span sp(kStRefine, s);
        check(launch_refine(ra, int(j - i), s), "refine");
      }
      i = j;
    }
    std::vector<Refined> r(n);
    check(cudaMemcpyAsync(r.data(), d_ref.p, n * sizeof(Refined), cudaMemcpyDeviceToHost, s), "refined");
    check(cudaStreamSynchronize(s), "refine");
    for (size_t i = 0; i < n; ++i) {
      result[size_t(order[i].owner)][size_t(order[i].local)] = r[i];
      done[size_t(order[i].owner)][size_t(order[i].local)] = 1;
    }
  }
};

// matching::select_refined (src/matching/multi.hpp:79-119) over the pooled,
// ranked candidates: per-model or shared quota and overlap threshold, an
// overlap test before and after refinement (refinement may move the pose),
// and the final ranking.  Refinement runs in speculative device batches: the
// next candidates that would be refined next if no earlier one were
// accepted.
std::vector<MultiCand> select_models(std::vector<MultiCand> cands, const std::vector<FindParams>& opts,
                                     const std::vector<RectGeom>& geoms, Selection sel, MultiRefiner* refiner) {
  std::sort(cands.begin(), cands.end(), ranks_before);
  std::vector<MultiCand> out;
  std::vector<Quad> boxes;
  std::vector<Aabb> bounds;
  std::vector<size_t> counts(opts.size(), 0);
  auto quota_full = [&](int m) {
    const int64_t limit = sel.num_matches >= 0 ? sel.num_matches : opts[size_t(m)].num_matches;
    return sel.num_matches < 0 && limit && counts[size_t(m)] >= uint64_t(limit);
  };
  auto threshold = [&](int m) { return sel.max_overlap >= 0 ? sel.max_overlap : opts[size_t(m)].max_overlap; };
  auto suppressed = [&](int m, const Quad& q, const Aabb& a) {
    const double thr = threshold(m) + 1e-12;
    for (size_t i = 0; i < out.size(); ++i) {
      if (sel.max_overlap < 0 && out[i].model != m) continue;
      if (apart(a, bounds[i])) continue;
      if (box_overlap(q, boxes[i]) > thr) return true;
    }
    return false;
  };
  for (size_t k = 0; k < cands.size(); ++k) {
    MultiCand c = cands[k];
    if (quota_full(c.model)) continue;
    const RectGeom& g = geoms[size_t(c.model)];
    Quad q = pose_box(g, c.c.row, c.c.col, c.c.angle);
    Aabb a = aabb_of(q);
    if (suppressed(c.model, q, a)) continue;
    if (refiner) {
      if (!refiner->has(c)) {
        // speculative batch: this candidate and the next ones that pass the
        // same tests now and are not mostly covered by one already queued
        std::vector<MultiCand> batch{c};
        std::vector<Aabb> queued{a};
        const size_t want = sel.num_matches > 0 ? size_t(std::max<int64_t>(1, sel.num_matches - int64_t(out.size())))
                                                : size_t(32);
        for (size_t j = k + 1; j < cands.size() && batch.size() < std::min<size_t>(want, MultiRefiner::kMax); ++j) {
          const MultiCand& o = cands[j];
          if (refiner->has(o) || quota_full(o.model)) continue;
          bool dup = false;
          for (const MultiCand& b : batch) dup = dup || (b.owner == o.owner && b.local == o.local);
          if (dup) continue;
          const Quad oq = pose_box(geoms[size_t(o.model)], o.c.row, o.c.col, o.c.angle);
          const Aabb oa = aabb_of(oq);
          if (suppressed(o.model, oq, oa)) continue;
          for (const Aabb& qa : queued) {
            const double ix = std::min(oa.right, qa.right) - std::max(oa.left, qa.left);
            const double iy = std::min(oa.bottom, qa.bottom) - std::max(oa.top, qa.top);
            const double ao = (oa.right - oa.left) * (oa.bottom - oa.top), aq = (qa.right - qa.left) * (qa.bottom - qa.top);
            if (ix > 0 && iy > 0 && ix * iy > .5 * std::min(ao, aq)) dup = true;
          }
          if (dup) continue;
          batch.push_back(o);
          queued.push_back(oa);
        }
        refiner->run(batch);
      }
      const Refined& r = refiner->get(c);
      if (!r.ok) continue;
      c.c.row = r.row;
      c.c.col = r.col;
      c.c.angle = r.angle;
      c.c.score = r.score;
      q = pose_box(g, c.c.row, c.c.col, c.c.angle);
      a = aabb_of(q);
      if (suppressed(c.model, q, a)) continue;
    }
    out.push_back(c);
    boxes.push_back(q);
    bounds.push_back(a);
    ++counts[size_t(c.model)];
    if (sel.num_matches > 0 && out.size() >= uint64_t(sel.num_matches)) break;
  }
  std::sort(out.begin(), out.end(), ranks_before);
  return out;
}

// find_models (src/ncc_matching/matcher.cpp:1077-1124) with HALCON's quota
// rule (per_model_quota_before_overlap = true, as mv_find_ncc_models calls
// it): one prepared query per distinct (model, options), the candidates
// pooled, selected and refined on the device.
std::vector<MultiCand> run_find_models(const std::vector<mvg_ncc_model_s*>& models, const void* pixels, int type,
                                       int64_t W, int64_t H, int64_t stride, int location, const uint8_t* domain,
                                       const std::vector<FindParams>& opts, Selection sel, cudaStream_t user_stream) {
  Workspace& ws = workspace();
  cudaStream_t s = user_stream ? user_stream : ws.own_stream;
  if (type != 0 && type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
  if (!pixels) raise(kInvalidArgument, "image pixels must not be null");
  const int64_t bpp = type == 1 ? 2 : 1;
  if (W <= 0 || H <= 0 || W > std::numeric_limits<int>::max() || H > std::numeric_limits<int>::max() ||
      H > thread_budgets().pixels / W)
    raise(kLimitExceeded, "search image exceeds pixel budget");
  if (stride < W * bpp || stride % bpp) raise(kInvalidArgument, "invalid row stride");
  // one upload of a host image for all models
  const void* dev = pixels;
  if (location == MVG_MEMORY_HOST) {
    const size_t bytes = size_t(stride) * size_t(H - 1) + size_t(W * bpp);
    ws.image.reserve(bytes);
    Span sp(kStUpload, s, 0);
    check(cudaMemcpyAsync(ws.image.p, pixels, bytes, cudaMemcpyHostToDevice, s), "image upload");
    dev = ws.image.p;
  }
  const size_t n = models.size();
  std::vector<int> owner(n);
  std::vector<std::unique_ptr<Prepared>> preps(n);
  auto same = [](const FindParams& a, const FindParams& b) {
    return a.angle_start == b.angle_start && a.angle_extent == b.angle_extent && a.min_score == b.min_score &&
           a.max_overlap == b.max_overlap && a.num_matches == b.num_matches && a.subpixel == b.subpixel &&
           a.highest == b.highest && a.lowest == b.lowest;
  };
  std::vector<RectGeom> geoms(n);
  for (size_t i = 0; i < n; ++i) {
    const ModelLevel& b = models[i]->host.levels.front();
    geoms[i] = RectGeom{-b.ocol - .5, double(b.width) - b.ocol - .5, -b.orow - .5, double(b.height) - b.orow - .5,
                        double(b.width) * double(b.height)};
    owner[i] = int(i);
    for (size_t j = 0; j < i; ++j)
      if (models[i] == models[j] && same(opts[i], opts[j])) {
        owner[i] = owner[j];
        break;
      }
    if (owner[i] != int(i)) continue;
    preps[i] = std::make_unique<Prepared>();
    run_find(*models[i], dev, type, W, H, stride, MVG_MEMORY_DEVICE, domain, opts[i], s, -3, preps[i].get());
  }
  std::vector<MultiCand> pool;
  for (size_t i = 0; i < n; ++i) {
    const Prepared& P = *preps[size_t(owner[i])];
    for (size_t k = 0; k < P.cands.size(); ++k)
      if (std::isfinite(P.cands[k].score)) pool.push_back({P.cands[k], int(i), owner[i], int(k)});
  }
  MultiRefiner refiner(ws, s, preps);
  const bool independent = sel.num_matches < 0 && sel.max_overlap >= 0 &&
                           std::any_of(opts.begin(), opts.end(), [](const FindParams& q) { return q.num_matches > 0; });
  std::vector<MultiCand> out = select_models(std::move(pool), opts, geoms, independent ? Selection{} : sel, &refiner);
  if (independent) out = select_models(std::move(out), opts, geoms, sel, nullptr);
  t_prof.collect();
  t_prof.finds += 1;
  return out;
}

template <class Fn> int32_t guarded(Fn&& fn) {
  try {
    fn();
    g_last_error.clear();
    return kOk;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_last_error = "out of memory";
    return kOutOfMemory;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return kInternal;
  } catch (...) {
    g_last_error = "unknown failure";
    return kInternal;
  }
}

// Controls of a single-model find, checked as NccControls checks them
// (src/c_api/ncc_matching_api.cpp:140-157): AngleExtent within [0, 2 pi],
// lowest level 0 read as 1.
FindParams make_params(double angle_start, double angle_extent, double min_score, int64_t num_matches,
                       double max_overlap, int32_t subpixel, int32_t highest, int32_t lowest) {
  auto number = [](double x, double lo, double hi, const char* name) {
    if (!std::isfinite(x) || x < lo || x > hi)
      raise(kInvalidArgument, std::string(name) + ": numeric control outside allowed range");
  };
  number(angle_start, -std::numeric_limits<double>::max(), std::numeric_limits<double>::max(), "AngleStart");
  number(angle_extent, 0, 6.28318530717958647692, "AngleExtent");
  number(min_score, 0, 1, "MinScore");
  number(max_overlap, 0, 1, "MaxOverlap");
  if (num_matches < 0) raise(kInvalidArgument, "NumMatches: match count must be nonnegative");
  if (subpixel != 0 && subpixel != 1) raise(kInvalidArgument, "SubPixel: expected true or false");
  if (highest < 0 || lowest < 0) raise(kInvalidArgument, "NumLevels: invalid highest/lowest level pair");
  FindParams p;
  p.angle_start = angle_start;
  p.angle_extent = angle_extent;
  p.min_score = min_score;
  p.num_matches = num_matches;
  p.max_overlap = max_overlap;
  p.subpixel = subpixel != 0;
  p.highest = highest;
  p.lowest = std::max<int32_t>(1, lowest);
  return p;
}

// Model handles and control tuples of a FindNccModels call, checked as
// ncc_models and NccControls do (src/c_api/ncc_matching_api.cpp:112-162).
struct MultiControls {
  std::vector<mvg_ncc_model_s*> models;
  std::vector<FindParams> opts;
  Selection sel;
};

MultiControls multi_controls(const mvg_ncc_model* model_ids, int64_t num_models, const double* angle_start,
                             int64_t n_angle_start, const double* angle_extent, int64_t n_angle_extent,
                             const double* min_score, int64_t n_min_score, const int64_t* num_matches,
                             int64_t n_num_matches, const double* max_overlap, int64_t n_max_overlap,
                             const int32_t* subpixel, int64_t n_subpixel, const int32_t* num_levels,
                             int64_t n_num_levels) {
  if (!model_ids || num_models <= 0 || num_models > 4096)
    raise(kInvalidArgument, "one model or a nonempty model array (maximum 4096) required");
  const size_t n = size_t(num_models);
  MultiControls mc;
  std::vector<mvg_ncc_model_s*>& models = mc.models;
  models.resize(n);
  for (size_t i = 0; i < n; ++i) {
    if (!model_ids[i]) raise(kTypeMismatch, "control handle is not an NCC model");
    models[i] = model_ids[i];
  }
  auto card = [&](const void* p, int64_t k, const char* name) {
    if (!p || (k != 1 && k != num_models))
      raise(kInvalidArgument, std::string(name) + ": one value or one value per model required");
  };
  card(angle_start, n_angle_start, "AngleStart");
  card(angle_extent, n_angle_extent, "AngleExtent");
  card(min_score, n_min_score, "MinScore");
  card(num_matches, n_num_matches, "NumMatches");
  card(max_overlap, n_max_overlap, "MaxOverlap");
  card(subpixel, n_subpixel, "SubPixel");
  if (!num_levels ||
      (n_num_levels != 1 && n_num_levels != 2 && n_num_levels != num_models && n_num_levels != 2 * num_models))
    raise(kInvalidArgument, "NumLevels: highest level or shared/per-model level pairs required");
  auto number = [&](const double* v, int64_t k, size_t i, double lo, double hi, const char* name) {
    const double x = v[k == 1 ? 0 : i];
    if (!std::isfinite(x) || x < lo || x > hi)
      raise(kInvalidArgument, std::string(name) + ": numeric control outside allowed range");
    return x;
  };
  std::vector<FindParams>& opts = mc.opts;
  opts.resize(n);
  for (size_t i = 0; i < n; ++i) {
    FindParams& q = opts[i];
    q.angle_start = number(angle_start, n_angle_start, i, -std::numeric_limits<double>::max(),
                           std::numeric_limits<double>::max(), "AngleStart");
    q.angle_extent = number(angle_extent, n_angle_extent, i, 0, 6.28318530717958647692, "AngleExtent");
    q.min_score = number(min_score, n_min_score, i, 0, 1, "MinScore");
    q.max_overlap = number(max_overlap, n_max_overlap, i, 0, 1, "MaxOverlap");
    const int64_t quota = num_matches[n_num_matches == 1 ? 0 : i];
    if (quota < 0) raise(kInvalidArgument, "NumMatches: match count must be nonnegative");
    q.num_matches = quota;
    const int32_t sp = subpixel[n_subpixel == 1 ? 0 : i];
    if (sp != 0 && sp != 1) raise(kInvalidArgument, "SubPixel: expected true or false");
    q.subpixel = sp != 0;
    size_t hi_at = 0, lo_at = 0;
    bool pair = false;
    if (n_num_levels == num_models && num_models > 1) {
      hi_at = i;
    } else if (n_num_levels == 2 * num_models) {
      hi_at = 2 * i;
      lo_at = hi_at + 1;
      pair = true;
    } else if (n_num_levels == 2) {
      lo_at = 1;
      pair = true;
    }
    const int64_t highest = num_levels[hi_at], lowest = pair ? num_levels[lo_at] : 1;
    if (highest < 0 || lowest < 0) raise(kInvalidArgument, "NumLevels: invalid highest/lowest level pair");
    q.highest = int(highest);
    q.lowest = int(std::max<int64_t>(1, lowest));
  }
  Selection& sel = mc.sel;
  sel.num_matches = n_num_matches == 1 ? opts.front().num_matches : -1;
  sel.max_overlap = n_max_overlap == 1 ? opts.front().max_overlap : -1;
  return mc;
}

// Host threads of the batched find.  They live as long as the process, so
// each keeps its workspace, stream and device buffers from one batch to the
// next (a thread of its own per find in flight, as the finds share nothing
// but the read-only models).  One batch runs at a time.
class FindPool {
 public:
  // Runs job(worker) on `workers` pool threads and returns when all are done.
  template <class Job> void run(int workers, Job& job) {
    std::lock_guard<std::mutex> one_batch(batch_);
    std::unique_lock<std::mutex> lk(m_);
    while (int(threads_.size()) < workers) {
      const int id = int(threads_.size());
      threads_.emplace_back([this, id] { loop(id); });
      threads_.back().detach();
    }
    call_ = [](void* j, int w) { (*static_cast<Job*>(j))(w); };
    job_ = &job;
    want_ = workers;
    done_ = 0;
    ++generation_;
    wake_.notify_all();
    finished_.wait(lk, [&] { return done_ == want_; });
    job_ = nullptr;
  }

 private:
  void loop(int id) {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(m_);
    for (;;) {
      wake_.wait(lk, [&] { return generation_ != seen; });
      seen = generation_;
      if (id >= want_) continue;
      void (*call)(void*, int) = call_;
      void* job = job_;
      lk.unlock();
      try {
        call(job, id);
      } catch (...) {
      }
      lk.lock();
      if (++done_ == want_) finished_.notify_all();
    }
  }

  std::mutex batch_, m_;
  std::condition_variable wake_, finished_;
  std::vector<std::thread> threads_;
  void (*call_)(void*, int) = nullptr;
  void* job_ = nullptr;
  int want_ = 0, done_ = 0;
  uint64_t generation_ = 0;
};

FindPool& find_pool() {
  static FindPool* pool = new FindPool;  // never destroyed: its threads outlive static destruction
  return *pool;
}

// One image of a batch: its matches, or the status and message of its failure.
struct BatchImage {
  std::vector<MultiCand> matches;
  int32_t status = 0;
  std::string message;
};

}  // namespace

// Thread-local error message shared by every entry point of the library.
void set_last_error(const char* message) { g_last_error = message ? message : ""; }

}  // namespace mvg

using namespace mvg;

extern "C" {

int32_t mvg_create_ncc_model(const void* pixels, int32_t pixel_type, int64_t width, int64_t height, int64_t row_stride,
                             const uint8_t* domain, int32_t num_levels, double angle_start, double angle_extent,
                             double angle_step, int32_t metric, mvg_ncc_model* model_id) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "ModelID must not be null");
    *model_id = nullptr;
    if (metric != MVG_METRIC_USE_POLARITY && metric != MVG_METRIC_IGNORE_GLOBAL_POLARITY)
      raise(kInvalidArgument, "unsupported NCC metric");
    if (num_levels > 16) raise(kInvalidArgument, "levels must be 0..16 or auto");
    if (angle_step > 3.14159265358979323846 / 16) raise(kInvalidArgument, "angle step must be in [0,pi/16] or auto");
    CreateParams p;
    p.levels = std::max(0, num_levels);
    p.ignore_polarity = metric == MVG_METRIC_IGNORE_GLOBAL_POLARITY;
    p.angle_start = angle_start;
    p.angle_extent = angle_extent;
    p.angle_step = angle_step > 0 ? angle_step : 0.;
    auto m = std::make_unique<mvg_ncc_model_s>();
    m->host = create_model(pixels, pixel_type, width, height, row_stride, domain, p, false);
    finish_model(*m);
    *model_id = m.release();
  });
}

int32_t mvg_test_withhold_tensor_weights(int32_t on) {
  return guarded([&] { t_withhold_weights = on != 0; });
}

int32_t mvg_set_model_build(int32_t where) {
  return guarded([&] {
    if (where != 0 && where != 1) raise(kInvalidArgument, "model build must be 0 (device) or 1 (host)");
    g_model_build.store(where);
  });
}

int32_t mvg_ncc_model_tables_digest(mvg_ncc_model model_id, uint64_t* digest) {
  return guarded([&] {
    if (!model_id || !digest) raise(kInvalidArgument, "model and digest must not be null");
    std::unique_lock<std::mutex> lock(model_id->mutex);
    ensure_device(*model_id);
    uint64_t h = 14695981039346656037ULL;
    auto mix = [&](const void* p, size_t n) {
      const unsigned char* b = static_cast<const unsigned char*>(p);
      for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ULL;
      }
    };
    for (const auto& L : model_id->levels) {
      const size_t np = L->model_patches;
      mix(L->desc.data(), np * sizeof(PatchDesc));
      mix(L->angles.data(), np * sizeof(double));
      const size_t ns = np ? size_t(L->desc[np - 1].sample_off + L->desc[np - 1].n) : 0;
      const size_t nr = np ? size_t(L->desc[np - 1].run_off + L->desc[np - 1].nruns) : 0;
      mix(L->offs.data(), ns * sizeof(int32_t));
      mix(L->w.data(), ns * sizeof(float));
      mix(L->sw.data(), ns * sizeof(int2));
      mix(L->lw.data(), ns * sizeof(int2));
      mix(L->runs.data(), nr * sizeof(int32_t));
      mix(L->runs_end.data(), nr * sizeof(int32_t));
    }
    *digest = h;
  });
}

int32_t mvg_write_ncc_model(mvg_ncc_model model_id, const char* file_name) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (!file_name || !*file_name) raise(kInvalidArgument, "nonempty file name without NUL required");
    write_model_file(model_id->host, file_name);
  });
}

int32_t mvg_read_ncc_model(const char* file_name, mvg_ncc_model* model_id) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "ModelID must not be null");
    *model_id = nullptr;
    if (!file_name || !*file_name) raise(kInvalidArgument, "nonempty file name without NUL required");
    auto m = std::make_unique<mvg_ncc_model_s>();
    m->host = read_model_file(file_name, false);
    try {
      finish_model(*m);
    } catch (const Error& e) {
      // persist.cpp:73-76: a model whose rasters cannot be built
      raise(e.status == kLimitExceeded ? kLimitExceeded : kDecodeError, "invalid prepared NCC model");
    }
    *model_id = m.release();
  });
}

int32_t mvg_serialize_ncc_model(mvg_ncc_model model_id, char* buffer, int64_t capacity, int64_t* size) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (!size) raise(kInvalidArgument, "size must not be null");
    const std::string bytes = serialize_model(model_id->host);
    *size = int64_t(bytes.size());
    if (buffer && capacity > 0) std::memcpy(buffer, bytes.data(), size_t(std::min<int64_t>(capacity, *size)));
  });
}

int32_t mvg_deserialize_ncc_model(const char* bytes, int64_t size, mvg_ncc_model* model_id) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "ModelID must not be null");
    *model_id = nullptr;
    if (size < 0 || (!bytes && size > 0)) raise(kInvalidArgument, "invalid model bytes");
    auto m = std::make_unique<mvg_ncc_model_s>();
    m->host = deserialize_model(std::string_view(bytes ? bytes : "", size_t(size)), false);
    try {
      finish_model(*m);
    } catch (const Error& e) {
      // persist.cpp:73-76: a model whose rasters cannot be built
      raise(e.status == kLimitExceeded ? kLimitExceeded : kDecodeError, "invalid prepared NCC model");
    }
    *model_id = m.release();
  });
}

int32_t mvg_get_ncc_model_params(mvg_ncc_model model_id, int32_t* num_levels, double* angle_start,
                                 double* angle_extent, double* angle_step, int32_t* metric) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    const HostModel& h = model_id->host;
    if (num_levels) *num_levels = int32_t(h.levels.size());
    if (angle_start) *angle_start = h.params.angle_start;
    if (angle_extent) *angle_extent = h.params.angle_extent;
    if (angle_step) *angle_step = h.params.angle_extent == 0 ? 0. : h.params.angle_step;
    if (metric) *metric = h.params.ignore_polarity ? MVG_METRIC_IGNORE_GLOBAL_POLARITY : MVG_METRIC_USE_POLARITY;
  });
}

int32_t mvg_ncc_model_raster(mvg_ncc_model model_id, int32_t level, int32_t index, int32_t* rows, int32_t* cols,
                             double* weights, int64_t capacity, double* meta, int64_t* count) {
  return guarded([&] {
    if (!model_id || !count) raise(kInvalidArgument, "model and count must not be null");
    *count = 0;
    std::unique_lock<std::mutex> lock(model_id->mutex);
    HostModel& h = model_id->host;
    const Raster* r = nullptr;
    if (level < 0) {
      r = &h.original;
    } else {
      if (size_t(level) >= h.levels.size()) raise(kInvalidArgument, "level out of range");
      // a model whose rasters were built on the device gets host copies here
      if (!h.rasters) {
        build_rasters(h);
        h.rasters = true;
      }
      const auto& ps = h.levels[size_t(level)].patches;
      if (index < 0 || size_t(index) >= ps.size()) raise(kInvalidArgument, "raster index out of range");
      r = &ps[size_t(index)];
    }
    if (meta) {
      meta[0] = r->angle;
      meta[1] = r->orow;
      meta[2] = r->ocol;
      meta[3] = r->wsum;
    }
    const int64_t n = int64_t(r->size());
    *count = n;
    if (n > capacity || !rows || !cols || !weights) return;
    std::copy(r->rows.begin(), r->rows.end(), rows);
    std::copy(r->cols.begin(), r->cols.end(), cols);
    std::copy(r->w.begin(), r->w.end(), weights);
  });
}

int32_t mvg_clear_ncc_model(mvg_ncc_model model_id) {
  return guarded([&] { delete model_id; });
}

int32_t mvg_find_ncc_model(const void* pixels, int32_t pixel_type, int64_t width, int64_t height, int64_t row_stride,
                           int32_t location, const uint8_t* domain, mvg_ncc_model model_id, double angle_start,
                           double angle_extent,
                           double min_score, int64_t num_matches, double max_overlap, int32_t subpixel,
                           int32_t highest_level, int32_t lowest_level, double* row, double* column, double* angle,
                           double* score, int64_t capacity, int64_t* count, void* stream) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (!count) raise(kInvalidArgument, "count must not be null");
    *count = 0;
    const auto p = make_params(angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel,
                               highest_level, lowest_level);
    const FindOutput r = run_find(*model_id, pixels, pixel_type, width, height, row_stride, location, domain, p,
                                  static_cast<cudaStream_t>(stream), -2);
    *count = int64_t(r.matches.size());
    for (size_t i = 0; i < r.matches.size() && int64_t(i) < capacity; ++i) {
      // edge-centred pose convention (src/c_api/ncc_matching_api.cpp:171-176)
      const Match& mt = r.matches[i];
      const double c = std::cos(mt.angle), s = std::sin(mt.angle);
      if (row) row[i] = mt.row + .5 * (1 - c + s);
      if (column) column[i] = mt.col + .5 * (1 - c - s);
      if (angle) angle[i] = mt.angle;
      if (score) score[i] = mt.score;
    }
  });
}

int32_t mvg_find_ncc_models(const void* pixels, int32_t pixel_type, int64_t width, int64_t height, int64_t row_stride,
                            int32_t location, const uint8_t* domain, const mvg_ncc_model* model_ids,
                            int64_t num_models,
                            const double* angle_start, int64_t n_angle_start, const double* angle_extent,
                            int64_t n_angle_extent, const double* min_score, int64_t n_min_score,
                            const int64_t* num_matches, int64_t n_num_matches, const double* max_overlap,
                            int64_t n_max_overlap, const int32_t* subpixel, int64_t n_subpixel,
                            const int32_t* num_levels, int64_t n_num_levels, double* row, double* column,
                            double* angle, double* score, int64_t* model, int64_t capacity, int64_t* count,
                            void* stream) {
  return guarded([&] {
    if (!count) raise(kInvalidArgument, "count must not be null");
    *count = 0;
    const MultiControls mc = multi_controls(model_ids, num_models, angle_start, n_angle_start, angle_extent,
                                            n_angle_extent, min_score, n_min_score, num_matches, n_num_matches,
                                            max_overlap, n_max_overlap, subpixel, n_subpixel, num_levels,
                                            n_num_levels);
    const std::vector<mvg_ncc_model_s*>& models = mc.models;
    const std::vector<FindParams>& opts = mc.opts;
    const Selection& sel = mc.sel;
    const std::vector<MultiCand> r = run_find_models(models, pixels, pixel_type, width, height, row_stride, location,
                                                     domain, opts, sel, static_cast<cudaStream_t>(stream));
    *count = int64_t(r.size());
    for (size_t i = 0; i < r.size() && int64_t(i) < capacity; ++i) {
      // edge-centred pose convention (src/c_api/ncc_matching_api.cpp:171-176)
      const Cand& c = r[i].c;
      const double cs = std::cos(c.angle), sn = std::sin(c.angle);
      if (row) row[i] = c.row + .5 * (1 - cs + sn);
      if (column) column[i] = c.col + .5 * (1 - cs - sn);
      if (angle) angle[i] = c.angle;
      if (score) score[i] = c.score;
      if (model) model[i] = r[i].model;
    }
  });
}

int32_t mvg_find_ncc_models_batch(const void* const* images, const int32_t* pixel_types, const int64_t* widths,
                                  const int64_t* heights, const int64_t* row_strides, int64_t num_images,
                                  int32_t location, const uint8_t* const* domains, const mvg_ncc_model* model_ids,
                                  int64_t num_models, const double* angle_start, int64_t n_angle_start,
                                  const double* angle_extent, int64_t n_angle_extent, const double* min_score,
                                  int64_t n_min_score, const int64_t* num_matches, int64_t n_num_matches,
                                  const double* max_overlap, int64_t n_max_overlap, const int32_t* subpixel,
                                  int64_t n_subpixel, const int32_t* num_levels, int64_t n_num_levels,
                                  int32_t workers, double* row, double* column, double* angle, double* score,
                                  int64_t* model, int64_t capacity, int64_t* image_offsets, int32_t* statuses,
                                  int64_t* count) {
  std::string first_failure;
  int32_t first_status = kOk;
  const int32_t st = guarded([&] {
    if (!count || !image_offsets || !statuses) raise(kInvalidArgument, "count, offsets and statuses required");
    *count = 0;
    if (num_images < 0 || num_images > (int64_t(1) << 24)) raise(kInvalidArgument, "invalid image count");
    image_offsets[0] = 0;
    if (num_images == 0) return;
    if (!images || !pixel_types || !widths || !heights || !row_strides)
      raise(kInvalidArgument, "image arrays must not be null");
    if (workers < 1 || workers > 256) raise(kInvalidArgument, "workers must be 1..256");
    const MultiControls mc = multi_controls(model_ids, num_models, angle_start, n_angle_start, angle_extent,
                                            n_angle_extent, min_score, n_min_score, num_matches, n_num_matches,
                                            max_overlap, n_max_overlap, subpixel, n_subpixel, num_levels,
                                            n_num_levels);
    int device = 0;
    check(cudaGetDevice(&device), "batch");
    const int path = t_path, lookahead = t_tc_lookahead;
    const Budgets budgets = thread_budgets();
    std::vector<BatchImage> done(static_cast<size_t>(num_images));
    std::atomic<int64_t> next{0};
    const int nworkers = int(std::min<int64_t>(workers, num_images));
    // the workers' tensor-core launches are merged (one launch per step for
    // all finds in flight) unless the calling thread asked for separate ones
    const int cohorts = path == 0 ? std::min(t_merge_tc, nworkers) : 0;
    // batched calls run one after the other (the pool and the batchers serve one)
    static std::mutex one_call;
    std::lock_guard<std::mutex> serial(one_call);
    if (cohorts > 0) {
      int sms = 0;
      check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attribute");
      for (int c = 0; c < cohorts; ++c) tc_batcher(c).begin(nworkers / cohorts + (c < nworkers % cohorts), device, sms);
    }
    auto job = [&](int w) {
      TcBatcher* batcher = cohorts > 0 ? &tc_batcher(w % cohorts) : nullptr;
      struct Member {
        TcBatcher* b;
        ~Member() {
          t_batcher = nullptr;
          if (b) b->leave();
        }
      } member{batcher};
      if (cudaSetDevice(device) != cudaSuccess) return;
      t_path = path;
      t_tc_lookahead = lookahead;
      thread_budgets() = budgets;
      t_batcher = batcher;
      for (int64_t i; (i = next.fetch_add(1)) < num_images;) {
        BatchImage& b = done[size_t(i)];
        b.status = guarded([&] {
          // an empty image finds nothing (the operator commits empty outputs,
          // src/c_api/ncc_matching_api.cpp:178-190)
          if (widths[i] == 0 || heights[i] == 0) return;
          const uint8_t* dom = domains ? domains[i] : nullptr;
          if (mc.models.size() > 1) {
            b.matches = run_find_models(mc.models, images[i], pixel_types[i], widths[i], heights[i],
                                        row_strides[i], location, dom, mc.opts, mc.sel, nullptr);
            return;
          }
          // one model: find_models reduces to find (same quota and overlap
          // rule), whose selection and refinement stay on the device
          const FindOutput r = run_find(*mc.models[0], images[i], pixel_types[i], widths[i], heights[i],
                                        row_strides[i], location, dom, mc.opts[0], nullptr, -2);
          for (const Match& mt : r.matches) {
            MultiCand m{};
            m.c.row = mt.row;
            m.c.col = mt.col;
            m.c.angle = mt.angle;
            m.c.score = mt.score;
            b.matches.push_back(m);
          }
        });
        if (b.status != kOk) b.message = g_last_error;
      }
    };
    find_pool().run(nworkers, job);
    if (next.load() < num_images) raise(kInternal, "batch worker could not select the device");
    int64_t at = 0;
    for (int64_t i = 0; i < num_images; ++i) {
      const BatchImage& b = done[size_t(i)];
      statuses[i] = b.status;
      if (b.status != kOk && first_status == kOk) {
        first_status = b.status;
        first_failure = "image " + std::to_string(i) + ": " + b.message;
      }
      for (const MultiCand& m : b.matches) {
        if (at < capacity) {
          // edge-centred pose convention (src/c_api/ncc_matching_api.cpp:171-176)
          const Cand& c = m.c;
          const double cs = std::cos(c.angle), sn = std::sin(c.angle);
          if (row) row[at] = c.row + .5 * (1 - cs + sn);
          if (column) column[at] = c.col + .5 * (1 - cs - sn);
          if (angle) angle[at] = c.angle;
          if (score) score[at] = c.score;
          if (model) model[at] = m.model;
        }
        ++at;
      }
      image_offsets[i + 1] = at;
    }
    *count = at;
  });
  if (st != kOk || first_status == kOk) return st;
  g_last_error = first_failure;
  return first_status;
}

int32_t mvg_ncc_score_gradient(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                               int64_t row_stride, int32_t location, mvg_ncc_model model_id, const double* poses,
                               int64_t count, double* score, double* gradient, void* stream) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (pixel_type != 0 && pixel_type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
    if (!pixels) raise(kInvalidArgument, "image pixels must not be null");
    if (count < 0 || (count > 0 && (!poses || !score || !gradient)))
      raise(kInvalidArgument, "poses, score and gradient arrays required");
    if (width <= 0 || height <= 0 || width > std::numeric_limits<int>::max() ||
        height > std::numeric_limits<int>::max() || height > thread_budgets().pixels / width)
      raise(kLimitExceeded, "search image exceeds pixel budget");
    const int64_t bpp = pixel_type == 1 ? 2 : 1;
    if (row_stride < width * bpp || row_stride % bpp) raise(kInvalidArgument, "invalid row stride");
    for (int64_t i = 0; i < 4 * count; ++i)
      if (!std::isfinite(poses[i])) raise(kInvalidArgument, "poses must be finite");
    if (count == 0) return;
    Workspace& ws = workspace();
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ws.own_stream;
    OriginalView orig;
    {
      std::unique_lock<std::mutex> lock(model_id->mutex);
      ensure_device(*model_id);
      orig = model_id->original.view();
    }
    const void* dev = pixels;
    if (location == MVG_MEMORY_HOST) {
      const size_t bytes = size_t(row_stride) * size_t(height - 1) + size_t(width * bpp);
      ws.image.reserve(bytes);
      check(cudaMemcpyAsync(ws.image.p, pixels, bytes, cudaMemcpyHostToDevice, s), "image upload");
      dev = ws.image.p;
    }
    init_state(ws, s, kMaxCandidates);
    LevelImage lev0{};
    ws.lev_v[0].reserve(size_t(width) * size_t(height));
    lev0.v = ws.lev_v[0].p;
    lev0.w = int(width);
    lev0.h = int(height);
    check(launch_pyramid0(dev, pixel_type, row_stride / bpp, 0, 0, lev0, &ws.state.p->error, s), "pyramid0");
    const size_t n = size_t(count);
    ws.adj_poses.reserve(4 * n);
    ws.adj_score.reserve(n);
    ws.adj_grad.reserve(4 * n);
    check(cudaMemcpyAsync(ws.adj_poses.p, poses, 4 * n * sizeof(double), cudaMemcpyHostToDevice, s), "poses");
    AdjointArgs aa;
    aa.img = ImageView{lev0.v, lev0.w, lev0.h, nullptr};
    aa.orig = orig;
    aa.poses = ws.adj_poses.p;
    aa.n = int(count);
    aa.score = ws.adj_score.p;
    aa.grad = ws.adj_grad.p;
    aa.absolute = model_id->host.params.ignore_polarity;
    check(launch_adjoint(aa, s), "adjoint");
    check(cudaMemcpyAsync(score, ws.adj_score.p, n * sizeof(double), cudaMemcpyDeviceToHost, s), "score");
    check(cudaMemcpyAsync(gradient, ws.adj_grad.p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s), "gradient");
    check(cudaStreamSynchronize(s), "adjoint");
  });
}

int32_t mvg_ncc_refine_similarity(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                  int64_t row_stride, int32_t location, mvg_ncc_model model_id, double* poses,
                                  int64_t count, int32_t iterations, double* score, void* stream) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (pixel_type != 0 && pixel_type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
    if (!pixels) raise(kInvalidArgument, "image pixels must not be null");
    if (count < 0 || (count > 0 && (!poses || !score))) raise(kInvalidArgument, "poses and score arrays required");
    if (iterations < 0 || iterations > 100) raise(kInvalidArgument, "iterations must be in [0, 100]");
    if (width <= 0 || height <= 0 || width > std::numeric_limits<int>::max() ||
        height > std::numeric_limits<int>::max() || height > thread_budgets().pixels / width)
      raise(kLimitExceeded, "search image exceeds pixel budget");
    const int64_t bpp = pixel_type == 1 ? 2 : 1;
    if (row_stride < width * bpp || row_stride % bpp) raise(kInvalidArgument, "invalid row stride");
    for (int64_t i = 0; i < 4 * count; ++i)
      if (!std::isfinite(poses[i])) raise(kInvalidArgument, "poses must be finite");
    if (count == 0) return;
    Workspace& ws = workspace();
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ws.own_stream;
    OriginalView orig;
    {
      std::unique_lock<std::mutex> lock(model_id->mutex);
      ensure_device(*model_id);
      orig = model_id->original.view();
    }
    const void* dev = pixels;
    if (location == MVG_MEMORY_HOST) {
      const size_t bytes = size_t(row_stride) * size_t(height - 1) + size_t(width * bpp);
      ws.image.reserve(bytes);
      check(cudaMemcpyAsync(ws.image.p, pixels, bytes, cudaMemcpyHostToDevice, s), "image upload");
      dev = ws.image.p;
    }
    init_state(ws, s, kMaxCandidates);
    LevelImage lev0{};
    ws.lev_v[0].reserve(size_t(width) * size_t(height));
    lev0.v = ws.lev_v[0].p;
    lev0.w = int(width);
    lev0.h = int(height);
    check(launch_pyramid0(dev, pixel_type, row_stride / bpp, 0, 0, lev0, &ws.state.p->error, s), "pyramid0");
    const size_t n = size_t(count);
    ws.adj_poses.reserve(4 * n);
    ws.adj_score.reserve(n);
    check(cudaMemcpyAsync(ws.adj_poses.p, poses, 4 * n * sizeof(double), cudaMemcpyHostToDevice, s), "poses");
    const HostModel& hm = model_id->host;
    Refine4Args ra;
    ra.img = ImageView{lev0.v, lev0.w, lev0.h, nullptr};
    ra.orig = orig;
    ra.poses = ws.adj_poses.p;
    ra.score = ws.adj_score.p;
    ra.n = int(count);
    ra.iterations = iterations;
    ra.absolute = hm.params.ignore_polarity;
    ra.max_shift = .75;  // as the reference's step limit (matcher.cpp:931)
    ra.max_angle = hm.params.angle_extent > 0 ? hm.params.angle_step : .01;
    ra.max_scale = .01;
    check(launch_refine4(ra, s), "refine4");
    check(cudaMemcpyAsync(poses, ws.adj_poses.p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s), "poses");
    check(cudaMemcpyAsync(score, ws.adj_score.p, n * sizeof(double), cudaMemcpyDeviceToHost, s), "score");
    check(cudaStreamSynchronize(s), "refine4");
  });
}

int32_t mvg_find_ncc_model_stage(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                                 int64_t row_stride, int32_t location, const uint8_t* domain, mvg_ncc_model model_id,
                                 double angle_start,
                                 double angle_extent, double min_score, int64_t num_matches, double max_overlap,
                                 int32_t subpixel, int32_t highest_level, int32_t lowest_level, int32_t stage,
                                 double* out, int64_t capacity, int64_t* count) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (!count) raise(kInvalidArgument, "count must not be null");
    *count = 0;
    const auto p = make_params(angle_start, angle_extent, min_score, num_matches, max_overlap, subpixel,
                               highest_level, lowest_level);
    const FindOutput r = run_find(*model_id, pixels, pixel_type, width, height, row_stride, location, domain, p,
                                  nullptr,
                                  stage);
    *count = int64_t(r.stage.size());
    for (size_t i = 0; i < r.stage.size() && int64_t(i) < capacity; ++i) {
      out[4 * i + 0] = r.stage[i].row;
      out[4 * i + 1] = r.stage[i].col;
      out[4 * i + 2] = r.stage[i].angle;
      out[4 * i + 3] = r.stage[i].score;
    }
  });
}

int32_t mvg_ncc_pyramid_level(const void* pixels, int32_t pixel_type, int64_t width, int64_t height,
                              int64_t row_stride, mvg_ncc_model model_id, int32_t highest_level, int32_t level,
                              float* out, int64_t capacity, double* geom) {
  return guarded([&] {
    if (!model_id) raise(kInvalidArgument, "control handle is not an NCC model");
    if (pixel_type != 0 && pixel_type != 1) raise(kTypeMismatch, "one byte or uint2 channel required");
    const HostModel& hm = model_id->host;
    const size_t level_count = highest_level ? std::min(hm.levels.size(), size_t(highest_level)) : hm.levels.size();
    if (level < 0 || size_t(level) >= level_count) raise(kInvalidArgument, "level out of range");
    const ModelLevel& base = hm.levels.front();
    const double radius = std::hypot(std::max(base.orow, double(base.height - 1) - base.orow),
                                     std::max(base.ocol, double(base.width - 1) - base.ocol));
    const int64_t lattice = int64_t(size_t{1} << (level_count - 1));
    const int64_t halo = int64_t(std::ceil(radius)) + 4 * lattice;
    const int64_t crop_bottom = std::min<int64_t>(height, ((height - 1 + halo) / lattice + 1) * lattice);
    const int64_t crop_right = std::min<int64_t>(width, ((width - 1 + halo) / lattice + 1) * lattice);
    Workspace& ws = workspace();
    cudaStream_t s = ws.own_stream;
    const int64_t bpp = pixel_type == 1 ? 2 : 1;
    const size_t bytes = size_t(row_stride) * size_t(height - 1) + size_t(width * bpp);
    ws.image.reserve(bytes);
    check(cudaMemcpyAsync(ws.image.p, pixels, bytes, cudaMemcpyHostToDevice, s), "image upload");
    init_state(ws, s, kMaxCandidates);
    LevelImage lev[kMaxLevels];
    int w = int(crop_right), h = int(crop_bottom);
    for (int l = 0; l <= level; ++l) {
      if (l) {
        w = std::max(1, w / 2);
        h = std::max(1, h / 2);
      }
      ws.lev_v[l].reserve(size_t(w) * size_t(h));
      lev[l].v = ws.lev_v[l].p;
      lev[l].w = w;
      lev[l].h = h;
      if (l == 0)
        check(launch_pyramid0(ws.image.p, pixel_type, row_stride / bpp, 0, 0, lev[0], &ws.state.p->error, s), "pyramid0");
      else
        check(launch_pyramid(lev[l - 1], lev[l], &ws.state.p->error, s), "pyramid");
    }
    if (int64_t(w) * h > capacity) raise(kInvalidArgument, "output capacity too small");
    check(cudaMemcpyAsync(out, lev[level].v, size_t(w) * size_t(h) * sizeof(float), cudaMemcpyDeviceToHost, s), "copy");
    check(cudaMemcpyAsync(ws.h_state, ws.state.p, sizeof(QueryState), cudaMemcpyDeviceToHost, s), "state");
    check(cudaStreamSynchronize(s), "sync");
    if (ws.h_state->error) raise_device_error(ws.h_state->error);
    const uint8_t* px = static_cast<const uint8_t*>(pixels);
    geom[0] = w;
    geom[1] = h;
    geom[2] = 0;
    geom[3] = 0;
    geom[4] = pixel_type == 1 ? double(*reinterpret_cast<const uint16_t*>(px)) : double(px[0]);
  });
}

const char* mvg_last_error(void) { return g_last_error.c_str(); }

int32_t mvg_set_correlation_path(int32_t path) {
  return guarded([&] {
    if (path != 0 && path != 1) raise(kInvalidArgument, "path must be 0 (tensor cores) or 1 (CUDA cores)");
    t_path = path;
  });
}

int32_t mvg_set_tc_weight_lookahead(int32_t rows) {
  return guarded([&] {
    if (rows < 1 || rows > 64) raise(kInvalidArgument, "weight lookahead must be 1..64 grid rows");
    t_tc_lookahead = rows;
  });
}

int32_t mvg_profile_enable(int32_t on) {
  return guarded([&] { t_prof.on = on != 0; });
}

int32_t mvg_profile_reset(void) {
  return guarded([&] { t_prof.reset(); });
}

int32_t mvg_profile_read(int32_t stage, const char** name, double* ms, int64_t* launches, double* work,
                         int64_t* finds) {
  return guarded([&] {
    if (stage < 0 || stage >= kStages) raise(kInvalidArgument, "stage out of range");
    if (name) *name = kStageNames[stage];
    if (ms) *ms = t_prof.ms[stage];
    if (launches) *launches = t_prof.launches[stage];
    if (work) *work = t_prof.work[stage];
    if (finds) *finds = t_prof.finds;
  });
}

int32_t mvg_set_budgets(int64_t samples, int64_t pixels, int32_t candidates) {
  return guarded([&] {
    if (samples < 0 || samples > int64_t(INT32_MAX) || pixels < 0 || pixels > (int64_t(1) << 30) || candidates < 0 ||
        candidates > kMaxCandidatesExt)
      raise(kInvalidArgument, "budgets: samples 0..2^31-1, pixels 0..2^30, candidates 0..2097152 (0 = default)");
    Budgets& b = thread_budgets();
    b.samples = samples ? size_t(samples) : kModelSampleBudget;
    b.pixels = pixels ? pixels : 32000000;
    b.candidates = candidates ? candidates : kMaxCandidates;
  });
}

int32_t mvg_get_budgets(int64_t* samples, int64_t* pixels, int32_t* candidates) {
  const Budgets& b = thread_budgets();
  if (samples) *samples = int64_t(b.samples);
  if (pixels) *pixels = b.pixels;
  if (candidates) *candidates = b.candidates;
  return kOk;
}

int32_t mvg_set_batch_merge(int32_t cohorts) {
  if (cohorts < 0 || cohorts > kMaxCohorts) {
    g_last_error = "cohorts must be 0..16";
    return kInvalidArgument;
  }
  t_merge_tc = cohorts;
  return kOk;
}

int32_t mvg_batch_profile_reset(void) {
  return guarded([&] {
    for (int c = 0; c < kMaxCohorts; ++c) tc_batcher(c).reset_stats();
  });
}

int32_t mvg_batch_profile_read(double* ms, int64_t* launches, int64_t* jobs, double* macs, double* issued) {
  return guarded([&] {
    TcBatcher::Stats sum;
    for (int c = 0; c < kMaxCohorts; ++c) {
      const TcBatcher::Stats st = tc_batcher(c).stats();
      sum.ms += st.ms;
      sum.launches += st.launches;
      sum.jobs += st.jobs;
      sum.macs += st.macs;
      sum.issued += st.issued;
    }
    if (ms) *ms = sum.ms;
    if (launches) *launches = sum.launches;
    if (jobs) *jobs = sum.jobs;
    if (macs) *macs = sum.macs;
    if (issued) *issued = sum.issued;
  });
}

int32_t mvg_profile_tensor_issued(double* macs) {
  return guarded([&] {
    if (!macs) raise(kInvalidArgument, "macs must not be null");
    *macs = t_prof.issued_tc;
  });
}

int32_t mvg_host_alloc(size_t bytes, void** ptr) {
  return guarded([&] { check(cudaMallocHost(ptr, bytes), "cudaMallocHost"); });
}
int32_t mvg_host_free(void* ptr) {
  return guarded([&] { check(cudaFreeHost(ptr), "cudaFreeHost"); });
}
int32_t mvg_device_alloc(size_t bytes, void** ptr) {
  return guarded([&] { check(cudaMalloc(ptr, bytes), "cudaMalloc"); });
}
int32_t mvg_device_free(void* ptr) {
  return guarded([&] { check(cudaFree(ptr), "cudaFree"); });
}
int32_t mvg_copy_to_device(void* dst, const void* src, size_t bytes) {
  return guarded([&] { check(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy"); });
}

}  // extern "C"
