// CreateNccModel's rotated rasters on the device (src/ncc_matching/model.cpp:
// 38-98, 225-241): for every level and trained angle, bilinear samples of the
// level raster at the rotated integer offsets, normalised to zero mean and
// unit energy, packed straight into the find kernels' sample and run tables.
//
// The weights must equal the host FP64 build bit for bit, so every
// expression keeps the reference's operation order with explicit
// round-to-nearest intrinsics (no contraction), cos/sin come from the host,
// and the order-dependent sums (the incremental mean, the energy, the weight
// sum) run serially in sample order, one thread per raster.  The rest is
// parallel: sampling one block per raster, ordered compaction by block scans,
// table packing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ncc_build.h"

namespace mvg {
namespace {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

struct LevelData {
  const double* gray;
  const uint8_t* mask;
  int w, h;
  double orow, ocol;
  int lin_pitch;
};

struct RasterJob {
  int level;
  int unrotated;
  double ca, sa;
  int r0, c0, rows, cols;  // offset box (unrotated: the level's pixels)
  long long pos_off;       // first dense position (chunk-relative)
  long long sample_off;    // first compacted sample (chunk-relative)
  long long table_off;     // first sample in the model's table arrays
  int run_off;             // first run in the model's run arrays
  int known;               // moments given (the unrotated level-0 raster)
  double mean, energy;
};

constexpr int kBuildThreads = 256;

// Dense sample values and validity over each raster's offset box
// (model.cpp:81-95; unrotated: model.cpp:70-76).
__global__ void __launch_bounds__(kBuildThreads) raster_sample_kernel(const RasterJob* jobs, const LevelData* levels,
                                                                      double* val, uint8_t* ok) {
  const RasterJob job = jobs[blockIdx.x];
  const LevelData L = levels[job.level];
  const long long n = (long long)job.rows * job.cols;
  for (long long p = threadIdx.x; p < n; p += blockDim.x) {
    const int r = job.r0 + int(p / job.cols), c = job.c0 + int(p % job.cols);
    double v = 0;
    uint8_t good = 0;
    if (job.unrotated) {
      const size_t i = size_t(r) * L.w + c;
      good = L.mask[i] != 0;
      v = L.gray[i];
    } else {
      // source position of the rotated offset (r, c) in the level raster
      const double y = dadd(dadd(dmul(job.ca, double(r)), dmul(job.sa, double(c))), L.orow);
      const double x = dadd(dadd(dmul(-job.sa, double(r)), dmul(job.ca, double(c))), L.ocol);
      if (!(y < 0 || x < 0 || y > double(L.h - 1) || x > double(L.w - 1))) {
        const size_t y0 = size_t(y), x0 = size_t(x);
        const size_t y1 = min(y0 + 1, size_t(L.h - 1)), x1 = min(x0 + 1, size_t(L.w - 1));
        const size_t i00 = y0 * L.w + x0, i01 = y0 * L.w + x1, i10 = y1 * L.w + x0, i11 = y1 * L.w + x1;
        if (L.mask[i00] && L.mask[i01] && L.mask[i10] && L.mask[i11]) {
          const double fy = dsub(y, double(y0)), fx = dsub(x, double(x0));
          const double gx = dsub(1., fx);
          const double top = dadd(dmul(gx, L.gray[i00]), dmul(fx, L.gray[i01]));
          const double bottom = dadd(dmul(gx, L.gray[i10]), dmul(fx, L.gray[i11]));
          v = dadd(dmul(dsub(1., fy), top), dmul(fy, bottom));
          good = 1;
        }
      }
    }
    val[job.pos_off + p] = v;
    ok[job.pos_off + p] = good;
  }
}

// Block-wide inclusive scan of one int per thread (kBuildThreads threads);
// returns the inclusive prefix, *total gets the block total.
__device__ int block_scan(int x, int* total) {
  __shared__ int warp_sum[kBuildThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int v = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sum[warp] = v;
  __syncthreads();
  int base = 0, all = 0;
  for (int k = 0; k < kBuildThreads / 32; ++k) {
    if (k < warp) base += warp_sum[k];
    all += warp_sum[k];
  }
  __syncthreads();
  *total = all;
  return base + v;
}

// Samples and runs per raster: a run starts at a valid position whose left
// neighbour in the box is not valid (samples are in row-major order).
__global__ void __launch_bounds__(kBuildThreads) raster_count_kernel(const RasterJob* jobs, const uint8_t* ok,
                                                                     int* samples, int* runs) {
  const RasterJob job = jobs[blockIdx.x];
  const long long n = (long long)job.rows * job.cols;
  int ns = 0, nr = 0;
  for (long long p = threadIdx.x; p < n; p += blockDim.x) {
    const uint8_t* o = ok + job.pos_off;
    if (o[p]) {
      ++ns;
      if (p % job.cols == 0 || !o[p - 1]) ++nr;
    }
  }
  int ts = 0, tr = 0;
  block_scan(ns, &ts);
  block_scan(nr, &tr);
  if (threadIdx.x == 0) {
    samples[blockIdx.x] = ts;
    runs[blockIdx.x] = tr;
  }
}

// Ordered compaction of the valid positions: (row, column, value) per sample.
__global__ void __launch_bounds__(kBuildThreads) raster_compact_kernel(const RasterJob* jobs, const double* val,
                                                                       const uint8_t* ok, int2* rc, double* v) {
  const RasterJob job = jobs[blockIdx.x];
  const long long n = (long long)job.rows * job.cols;
  long long base = job.sample_off;
  for (long long t0 = 0; t0 < n; t0 += blockDim.x) {
    const long long p = t0 + threadIdx.x;
    const int good = p < n && ok[job.pos_off + p];
    int total = 0;
    const int incl = block_scan(good, &total);
    if (good) {
      const long long k = base + incl - 1;
      rc[k] = make_int2(job.r0 + int(p / job.cols), job.c0 + int(p % job.cols));
      v[k] = val[job.pos_off + p];
    }
    base += total;
  }
}

// finish_raster of the host build (model.cpp:38-65), one thread per raster,
// in sample order: incremental mean (or the given one), centring and energy,
// 1/sqrt(energy), weights, the float weight sum and the bounds.  flag: 1 =
// degenerate (fewer than 4 samples, or no finite positive energy).
__global__ void raster_moments_kernel(const RasterJob* jobs, int njobs, const int* samples, const int2* rc,
                                      double* v, int* flag, float* fwsum, int4* bounds) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  const RasterJob job = jobs[j];
  const int n = samples[j];
  double* x = v + job.sample_off;
  const int2* p = rc + job.sample_off;
  flag[j] = 1;
  if (n < 4) return;
  double mean = 0, energy = 0;
  if (job.known) {
    mean = job.mean;
    energy = job.energy;
    for (int i = 0; i < n; ++i) x[i] = dsub(x[i], mean);
  } else {
    for (int i = 0; i < n; ++i) mean = dadd(mean, __ddiv_rn(dsub(x[i], mean), double(i + 1)));
    for (int i = 0; i < n; ++i) {
      const double d = dsub(x[i], mean);
      x[i] = d;
      energy = dadd(energy, dmul(d, d));
    }
  }
  if (!(energy > 0) || !isfinite(energy)) return;
  const double k = __ddiv_rn(1., __dsqrt_rn(energy));
  double fsum = 0;
  int4 b = make_int4(p[0].x, p[0].x, p[0].y, p[0].y);
  for (int i = 0; i < n; ++i) {
    const double w = dmul(x[i], k);
    x[i] = w;
    fsum = dadd(fsum, double(__double2float_rn(w)));
    b.x = min(b.x, p[i].x);
    b.y = max(b.y, p[i].x);
    b.z = min(b.z, p[i].y);
    b.w = max(b.w, p[i].y);
  }
  fwsum[j] = __double2float_rn(fsum);
  bounds[j] = b;
  flag[j] = 0;
}

// Packs one raster's samples into the level tables (the layout DevLevel
// builds on the host): packed int16 (row, column), float weight,
// interleaved {offset, weight bits} and {row * lin_pitch + column, weight
// bits}, and the row runs (packed row and begin; end).
__global__ void __launch_bounds__(kBuildThreads) raster_tables_kernel(const RasterJob* jobs, const LevelData* levels,
                                                                      const int* samples, const int2* rc,
                                                                      const double* v, int32_t* offs, float* w,
                                                                      int2* sw, int2* lw, int32_t* runs,
                                                                      int32_t* runs_end) {
  const RasterJob job = jobs[blockIdx.x];
  const int n = samples[blockIdx.x];
  const int pitch = levels[job.level].lin_pitch;
  const int2* p = rc + job.sample_off;
  int run_base = job.run_off;
  for (int t0 = 0; t0 < n; t0 += blockDim.x) {
    const int i = t0 + threadIdx.x;
    int starts = 0;
    int2 q = make_int2(0, 0);
    if (i < n) {
      q = p[i];
      starts = i == 0 || p[i - 1].x != q.x || p[i - 1].y + 1 != q.y;
    }
    int total = 0;
    const int incl = block_scan(starts, &total);
    if (i < n) {
      const long long g = job.table_off + i;
      const int32_t o = int32_t((uint32_t(uint16_t(int16_t(q.x))) << 16) | uint16_t(int16_t(q.y)));
      const float wf = __double2float_rn(v[job.sample_off + i]);
      offs[g] = o;
      w[g] = wf;
      sw[g] = make_int2(o, __float_as_int(wf));
      lw[g] = make_int2(q.x * pitch + q.y, __float_as_int(wf));
      const int run = run_base + incl - 1;
      if (starts) runs[run] = o;
      const bool last = i + 1 == n || p[i + 1].x != q.x || p[i + 1].y != q.y + 1;
      if (last) runs_end[run] = q.y;
    }
    run_base += total;
  }
}

}  // namespace
}  // namespace mvg

namespace mvg {
namespace {

void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) raise(kInternal, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T> struct Buf {
  T* p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() {
    if (p) cudaFree(p);
  }
  T* get(size_t count) {
    if (count > n || !p) {
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
      cuda_ok(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), "cudaMalloc");
      n = std::max<size_t>(count, 1);
    }
    return p;
  }
};

template <class T> void to_host(std::vector<T>& dst, const T* src, size_t n, cudaStream_t s) {
  const size_t at = dst.size();
  dst.resize(at + n);
  if (n) cuda_ok(cudaMemcpyAsync(dst.data() + at, src, n * sizeof(T), cudaMemcpyDeviceToHost, s), "copy");
}

constexpr long long kChunkPositions = 16ll << 20;  // dense positions per chunk of rasters

}  // namespace

void build_tables_device(const HostModel& m, const std::vector<int32_t>& lin_pitch, std::vector<LevelTables>& out,
                         cudaStream_t s) {
  const size_t nl = m.levels.size();
  out.assign(nl, LevelTables{});
  // level rasters on the device
  std::vector<std::unique_ptr<Buf<double>>> gray(nl);
  std::vector<std::unique_ptr<Buf<uint8_t>>> mask(nl);
  std::vector<LevelData> ld(nl);
  for (size_t l = 0; l < nl; ++l) {
    const ModelLevel& L = m.levels[l];
    gray[l] = std::make_unique<Buf<double>>();
    mask[l] = std::make_unique<Buf<uint8_t>>();
    const size_t px = L.width * L.height;
    cuda_ok(cudaMemcpyAsync(gray[l]->get(px), L.gray.data(), px * sizeof(double), cudaMemcpyHostToDevice, s), "gray");
    cuda_ok(cudaMemcpyAsync(mask[l]->get(px), L.mask.data(), px, cudaMemcpyHostToDevice, s), "mask");
    ld[l] = LevelData{gray[l]->p, mask[l]->p, int(L.width), int(L.height), L.orow, L.ocol, lin_pitch[l]};
  }
  Buf<LevelData> d_levels;
  cuda_ok(cudaMemcpyAsync(d_levels.get(nl), ld.data(), nl * sizeof(LevelData), cudaMemcpyHostToDevice, s), "levels");

  // every raster in the reference's order; the first box over budget ends
  // the list (its error comes after the earlier rasters' own)
  std::vector<RasterJob> all;
  std::vector<RasterBox> boxes;
  bool box_error = false;
  for (size_t l = 0; l < nl && !box_error; ++l)
    for (const double angle : m.angles) {
      const RasterBox b = raster_box(m.levels[l], angle);
      if (b.too_large) {
        box_error = true;
        break;
      }
      RasterJob j{};
      j.level = int(l);
      j.unrotated = b.unrotated;
      j.ca = b.ca;
      j.sa = b.sa;
      j.r0 = b.r0;
      j.c0 = b.c0;
      j.rows = b.r1 - b.r0 + 1;
      j.cols = b.c1 - b.c0 + 1;
      j.known = l == 0 && b.unrotated;
      j.mean = m.level0_mean;
      j.energy = m.level0_energy;
      all.push_back(j);
      boxes.push_back(b);
    }

  Buf<RasterJob> d_jobs;
  Buf<double> d_val, d_v;
  Buf<uint8_t> d_ok;
  Buf<int> d_samples, d_runs, d_flag;
  Buf<int2> d_rc;
  Buf<float> d_fwsum;
  Buf<int4> d_bounds;
  Buf<int32_t> d_offs, d_runsv, d_runs_end;
  Buf<float> d_w;
  Buf<int2> d_sw, d_lw;
  size_t total = 0;  // samples of the rasters accepted so far (budget)
  for (size_t first = 0; first < all.size();) {
    // one chunk of consecutive rasters
    size_t last = first;
    long long pos = 0;
    while (last < all.size()) {
      const long long np = (long long)all[last].rows * all[last].cols;
      if (last > first && pos + np > kChunkPositions) break;
      all[last].pos_off = pos;
      pos += np;
      ++last;
    }
    const int nj = int(last - first);
    RasterJob* jobs = all.data() + first;
    cuda_ok(cudaMemcpyAsync(d_jobs.get(size_t(nj)), jobs, size_t(nj) * sizeof(RasterJob), cudaMemcpyHostToDevice, s),
            "jobs");
    raster_sample_kernel<<<nj, kBuildThreads, 0, s>>>(d_jobs.p, d_levels.p, d_val.get(size_t(pos)), d_ok.get(size_t(pos)));
    raster_count_kernel<<<nj, kBuildThreads, 0, s>>>(d_jobs.p, d_ok.p, d_samples.get(size_t(nj)), d_runs.get(size_t(nj)));
    cuda_ok(cudaGetLastError(), "raster count");
    std::vector<int> ns, nr;
    to_host(ns, d_samples.p, size_t(nj), s);
    to_host(nr, d_runs.p, size_t(nj), s);
    cuda_ok(cudaStreamSynchronize(s), "raster count");
    long long samples = 0, runs = 0;
    for (int k = 0; k < nj; ++k) {
      jobs[k].sample_off = samples;
      jobs[k].table_off = samples;
      jobs[k].run_off = int(runs);
      samples += ns[size_t(k)];
      runs += nr[size_t(k)];
    }
    cuda_ok(cudaMemcpyAsync(d_jobs.p, jobs, size_t(nj) * sizeof(RasterJob), cudaMemcpyHostToDevice, s), "jobs");
    raster_compact_kernel<<<nj, kBuildThreads, 0, s>>>(d_jobs.p, d_val.p, d_ok.p, d_rc.get(size_t(samples)),
                                                       d_v.get(size_t(samples)));
    raster_moments_kernel<<<(nj + 31) / 32, 32, 0, s>>>(d_jobs.p, nj, d_samples.p, d_rc.p, d_v.p,
                                                        d_flag.get(size_t(nj)), d_fwsum.get(size_t(nj)),
                                                        d_bounds.get(size_t(nj)));
    cuda_ok(cudaGetLastError(), "raster moments");
    std::vector<int> flag;
    std::vector<float> fwsum;
    std::vector<int4> bounds;
    to_host(flag, d_flag.p, size_t(nj), s);
    to_host(fwsum, d_fwsum.p, size_t(nj), s);
    to_host(bounds, d_bounds.p, size_t(nj), s);
    cuda_ok(cudaStreamSynchronize(s), "raster moments");
    // the reference's checks, raster by raster (model.cpp:235-238)
    for (int k = 0; k < nj; ++k) {
      if (flag[size_t(k)]) raise(kInvalidArgument, "rotation produces a degenerate template");
      if (size_t(ns[size_t(k)]) > m.sample_budget - total) raise(kLimitExceeded, "model raster budget exceeded");
      total += size_t(ns[size_t(k)]);
    }
    raster_tables_kernel<<<nj, kBuildThreads, 0, s>>>(
        d_jobs.p, d_levels.p, d_samples.p, d_rc.p, d_v.p, d_offs.get(size_t(samples)), d_w.get(size_t(samples)),
        d_sw.get(size_t(samples)), d_lw.get(size_t(samples)), d_runsv.get(size_t(runs)), d_runs_end.get(size_t(runs)));
    cuda_ok(cudaGetLastError(), "raster tables");
    // level tables on the host, raster by raster (a chunk may span levels)
    for (int k = 0; k < nj;) {
      const int level = jobs[k].level;
      int e = k;
      while (e < nj && jobs[e].level == level) ++e;
      LevelTables& T = out[size_t(level)];
      const long long s0 = jobs[k].table_off, r0 = jobs[k].run_off;
      const long long s1 = e < nj ? jobs[e].table_off : samples, r1 = e < nj ? jobs[e].run_off : runs;
      const int32_t base_s = int32_t(T.offs.size()), base_r = int32_t(T.runs.size());
      for (int q = k; q < e; ++q) {
        const RasterBox& b = boxes[first + size_t(q)];
        const ModelLevel& L = m.levels[size_t(level)];
        PatchDesc d{};
        d.angle = b.angle;
        d.orow = b.unrotated ? L.orow : 0.;
        d.ocol = b.unrotated ? L.ocol : 0.;
        d.rmin = bounds[size_t(q)].x;
        d.rmax = bounds[size_t(q)].y;
        d.cmin = bounds[size_t(q)].z;
        d.cmax = bounds[size_t(q)].w;
        d.n = ns[size_t(q)];
        d.sample_off = base_s + int32_t(jobs[q].table_off - s0);
        d.nruns = nr[size_t(q)];
        d.run_off = base_r + int32_t(jobs[q].run_off - r0);
        d.wsum = fwsum[size_t(q)];
        T.desc.push_back(d);
        T.angles.push_back(b.angle);
      }
      to_host(T.offs, d_offs.p + s0, size_t(s1 - s0), s);
      to_host(T.w, d_w.p + s0, size_t(s1 - s0), s);
      to_host(T.sw, d_sw.p + s0, size_t(s1 - s0), s);
      to_host(T.lw, d_lw.p + s0, size_t(s1 - s0), s);
      to_host(T.runs, d_runsv.p + r0, size_t(r1 - r0), s);
      to_host(T.runs_end, d_runs_end.p + r0, size_t(r1 - r0), s);
      k = e;
    }
    cuda_ok(cudaStreamSynchronize(s), "raster tables");
    first = last;
  }
  if (box_error) raise(kLimitExceeded, "rotated bounding box exceeds budget");
}

}  // namespace mvg
