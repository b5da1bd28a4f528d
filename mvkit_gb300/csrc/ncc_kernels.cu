// CUDA kernels of the GB300 NCC find path (sm_103a).
//
// Numerics.  Every pyramid value is an integer sum of 4^k input pixels, held
// exactly in float.  Window moments (sum S, sum S^2) come from int64 row
// prefix sums, so the variance numerator n*sum(S^2) - (sum S)^2 is exact and
// the "variance <= 0 -> no score" rule of the reference is decided exactly.
// The template dot product sum(w * (S - S_first)) runs in FP32 on the CUDA
// cores.  The full-resolution score and the Gauss-Newton moments accumulate
// in FP32 per thread and combine as FP32 (hi, lo) two-sum pairs; the 3x3
// normal equations are solved in FP64 on one thread.
//
// sm_103 issues FP64 at a small fraction of the FP32 rate, so FP64 appears
// only where the reference's decisions need it: pose lattice arithmetic (or
// an FP32 form the host proved exact), the normal-equation solve, and the
// rectangle overlap of the MaxOverlap rule.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "ncc_kernels.h"

namespace mvg {
namespace {

__device__ __forceinline__ int off_row(int32_t o) { return o >> 16; }
__device__ __forceinline__ int off_col(int32_t o) { return int(int16_t(o & 0xffff)); }
__device__ __forceinline__ int run_row(int32_t o) { return o >> 16; }
__device__ __forceinline__ int run_begin(int32_t o) { return int(int16_t(o & 0xffff)); }

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// pose coordinate of integer position r on a level: crop + step*(r + o) + off
// (src/ncc_matching/matcher.cpp:558,592,687)
__device__ __forceinline__ double lattice_pose(double crop, double step, int r, double o, double off) {
  return dadd(dadd(crop, dmul(step, dadd(double(r), o))), off);
}
__device__ __forceinline__ float lattice_pose32(float crop, float step, int r, float o, float off) {
  return __fadd_rn(__fadd_rn(crop, __fmul_rn(step, __fadd_rn(float(r), o))), off);
}

// ------------------------------------------------------------ search domain
// domain_contains (src/ncc_matching/matcher.cpp:249-251): the pixel nearest
// to the pose lies in the domain.
__device__ __forceinline__ bool domain_contains(const DomainView& d, double row, double col) {
  const double rr = floor(row + .5), cc = floor(col + .5);
  if (!(rr >= 0 && cc >= 0 && rr < d.h && cc < d.w)) return false;
  return !d.mask || d.mask[size_t(rr) * d.w + size_t(cc)] != 0;
}

// may_contain (matcher.cpp:507-534) for a reduced domain, beyond the bounding
// box that the position ranges encode: spacing 1 tests the nearest pixel; a
// coarser spacing s accepts a pose with a domain pixel within 2s rows and
// columns (a run [b, e] of row y meets |y - row| <= 2s, b <= col + 2s,
// e >= col - 2s exactly when the mask has a pixel in the integer rectangle
// [ceil(row - 2s), floor(row + 2s)] x [ceil(col - 2s), floor(col + 2s)]),
// counted from the mask's 2-D prefix counts.  The full image (mask null)
// passes.
__device__ bool may_contain(const DomainView& d, double row, double col, double spacing) {
  if (!d.mask) return true;
  if (spacing == 1) return domain_contains(d, row, col);
  const double m = 2 * spacing;
  if (row < d.rmin - m || row > d.rmax + m || col < d.cmin - m || col > d.cmax + m) return false;
  if (!d.sparse) return true;
  const int r0 = max(0, int(ceil(dsub(row, m)))), r1 = min(d.h - 1, int(floor(dadd(row, m))));
  const int c0 = max(0, int(ceil(dsub(col, m)))), c1 = min(d.w - 1, int(floor(dadd(col, m))));
  if (r0 > r1 || c0 > c1) return false;
  const size_t pitch = size_t(d.w) + 1;
  const int32_t n = d.count[size_t(r1 + 1) * pitch + c1 + 1] - d.count[size_t(r0) * pitch + c1 + 1] -
                    d.count[size_t(r1 + 1) * pitch + c0] + d.count[size_t(r0) * pitch + c0];
  return n > 0;
}

// ------------------------------------------------------- FP32 pair arithmetic
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 f2(float x) { return F2{x, 0.f}; }
__device__ __forceinline__ F2 f2_add(F2 x, F2 y) {
  const float s = __fadd_rn(x.hi, y.hi);
  const float bb = __fsub_rn(s, x.hi);
  const float e = __fadd_rn(__fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb)), __fadd_rn(x.lo, y.lo));
  const float h = __fadd_rn(s, e);
  return F2{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ F2 f2_neg(F2 x) { return F2{-x.hi, -x.lo}; }
__device__ __forceinline__ F2 f2_sub(F2 x, F2 y) { return f2_add(x, f2_neg(y)); }
__device__ __forceinline__ F2 f2_mul(F2 x, F2 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  const float h = __fadd_rn(p, e);
  return F2{h, __fsub_rn(e, __fsub_rn(h, p))};
}
__device__ __forceinline__ F2 f2_div(F2 x, F2 y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const F2 r = f2_sub(x, f2_mul(f2(q1), y));
  const float q2 = __fdiv_rn(r.hi, y.hi);
  const float h = __fadd_rn(q1, q2);
  return F2{h, __fsub_rn(q2, __fsub_rn(h, q1))};
}
__device__ __forceinline__ float f2_val(F2 x) { return x.hi + x.lo; }
__device__ __forceinline__ double f2_dbl(F2 x) { return double(x.hi) + double(x.lo); }

// Score of one window from the FP32 template dot and exact integer moments.
// D = sum w (S - S0) relates to the reference's sum w q by a 4^k factor that
// cancels against the variance, giving score = D / sqrt(V / n) with
// V = n sum S^2 - (sum S)^2 (src/ncc_matching/matcher.cpp:97-105).
__device__ __forceinline__ float window_score(float dot, long long s1, long long s2, int n, int absolute) {
  const __int128 v = (__int128)n * s2 - (__int128)s1 * s1;
  if (v <= 0) return -INFINITY;
  const long long hi = (long long)(v >> 62);
  const float vf = hi ? __ll2float_rn(hi) * 4.611686018427387904e18f +
                            __ull2float_rn((unsigned long long)(v & ((((__int128)1) << 62) - 1)))
                      : __ll2float_rn((long long)v);
  float s = dot * rsqrtf(vf / float(n));
  s = fminf(1.f, fmaxf(-1.f, s));
  return absolute ? fabsf(s) : s;
}

// Window moments {sum S, sum S^2} of a patch at (r, c) from the level's row
// prefixes: runs first, first + step, ... (step > 1 splits the runs over
// threads; the caller adds the parts).
__device__ __forceinline__ void window_moments(const LevelImage& lev, int pitch, int r, int c,
                                               const int2* __restrict__ runs, int nruns, long long& s1, long long& s2,
                                               int first = 0, int step = 1) {
  s1 = 0;
  s2 = 0;
  if (lev.prefix32) {
    // four runs per step, all eight prefix loads issued before the sums
    const uint2* __restrict__ P = lev.prefix32;
    int j = first;
    for (; j + 3 * step < nruns; j += 4 * step) {
      int2 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) q[u] = __ldg(runs + j + u * step);
      uint2 hi[4], lo[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const size_t base = size_t(r + run_row(q[u].x)) * pitch + c;
        hi[u] = P[base + q[u].y + 1];
        lo[u] = P[base + run_begin(q[u].x)];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        s1 += (long long)(hi[u].x - lo[u].x);
        s2 += (long long)(hi[u].y - lo[u].y);
      }
    }
    for (; j < nruns; j += step) {
      const int2 q = __ldg(runs + j);
      const size_t base = size_t(r + run_row(q.x)) * pitch + c;
      const uint2 hi = P[base + q.y + 1];
      const uint2 lo = P[base + run_begin(q.x)];
      s1 += (long long)(hi.x - lo.x);
      s2 += (long long)(hi.y - lo.y);
    }
    return;
  }
  const longlong2* __restrict__ P = lev.prefix;
  int j = first;
  for (; j + step < nruns; j += 2 * step) {
    const int2 q0 = __ldg(runs + j), q1 = __ldg(runs + j + step);
    const size_t b0 = size_t(r + run_row(q0.x)) * pitch + c, b1 = size_t(r + run_row(q1.x)) * pitch + c;
    const longlong2 h0 = P[b0 + q0.y + 1], l0 = P[b0 + run_begin(q0.x)];
    const longlong2 h1 = P[b1 + q1.y + 1], l1 = P[b1 + run_begin(q1.x)];
    s1 += (h0.x - l0.x) + (h1.x - l1.x);
    s2 += (h0.y - l0.y) + (h1.y - l1.y);
  }
  for (; j < nruns; j += step) {
    const int2 q = __ldg(runs + j);
    const size_t base = size_t(r + run_row(q.x)) * pitch + c;
    const longlong2 hi = P[base + q.y + 1];
    const longlong2 lo = P[base + run_begin(q.x)];
    s1 += hi.x - lo.x;
    s2 += hi.y - lo.y;
  }
}

// (score, order) with the first strict maximum in iteration order winning
__device__ __forceinline__ bool better(float s, int o, float bs, int bo) {
  return s > bs || (s == bs && o < bo);
}

// ------------------------------------------------------------------ pyramid
// Level 0: the crop as float; with `pairs`, also the fp16 pairs (v[x],
// v[x+1]) of pairs_kernel (last column repeated) for an fp16-exact level 0.
template <class T>
__global__ void pyramid0_kernel(const T* __restrict__ src, int64_t pitch, int crop_row, int crop_col, LevelImage dst,
                                uint32_t* __restrict__ pairs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y * blockDim.y + threadIdx.y;
  if (c >= dst.w || r >= dst.h) return;
  const T* row = src + (int64_t(crop_row) + r) * pitch + crop_col;
  const float v = float(row[c]);
  dst.v[size_t(r) * dst.w + c] = v;
  if (pairs) {
    const __half a = __float2half_rn(v), b = __float2half_rn(float(row[c + 1 < dst.w ? c + 1 : c]));
    pairs[size_t(r) * dst.w + c] = uint32_t(__half_as_ushort(a)) | (uint32_t(__half_as_ushort(b)) << 16);
  }
}

// level k+1 from level k: 2x2 sums with the reference's clamped neighbours
// (src/ncc_matching/matcher.cpp:436-453)
__global__ void pyramid_kernel(LevelImage src, LevelImage dst, int32_t* error_flag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y * blockDim.y + threadIdx.y;
  if (c >= dst.w || r >= dst.h) return;
  const int r0 = 2 * r, r1 = min(r0 + 1, src.h - 1), c0 = 2 * c, c1 = min(c0 + 1, src.w - 1);
  const float a = src.v[size_t(r0) * src.w + c0], b = src.v[size_t(r0) * src.w + c1];
  const float d = src.v[size_t(r1) * src.w + c0], e = src.v[size_t(r1) * src.w + c1];
  const float s = ((a + b) + d) + e;
  if (s >= 16777216.f) atomicExch(error_flag, int32_t(kUnsupported));
  dst.v[size_t(r) * dst.w + c] = s;
}

// row prefix sums {sum S, sum S^2}, one warp per row
__global__ void prefix_kernel(LevelImage lev) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= lev.h) return;
  const float* row = lev.v + size_t(warp) * lev.w;
  longlong2* out = lev.prefix + size_t(warp) * (lev.w + 1);
  uint2* out32 = lev.prefix32 ? lev.prefix32 + size_t(warp) * (lev.w + 1) : nullptr;
  if (lane == 0) {
    if (out32)
      out32[0] = make_uint2(0, 0);
    else
      out[0] = make_longlong2(0, 0);
  }
  if (out32) {
    // modulo 2^32: the same stored values from 32-bit sums and shuffles
    uint32_t c1 = 0, c2 = 0;
    for (int base = 0; base < lev.w; base += 32) {
      const int c = base + lane;
      const uint32_t s = c < lev.w ? uint32_t(row[c]) : 0u;
      uint32_t a = s, b = s * s;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ua = __shfl_up_sync(0xffffffffu, a, o);
        const uint32_t ub = __shfl_up_sync(0xffffffffu, b, o);
        if (lane >= o) {
          a += ua;
          b += ub;
        }
      }
      if (c < lev.w) out32[c + 1] = make_uint2(c1 + a, c2 + b);
      c1 += __shfl_sync(0xffffffffu, a, 31);
      c2 += __shfl_sync(0xffffffffu, b, 31);
    }
    return;
  }
  long long c1 = 0, c2 = 0;
  for (int base = 0; base < lev.w; base += 32) {
    const int c = base + lane;
    const long long s = c < lev.w ? (long long)row[c] : 0;
    long long a = s, b = s * s;
    for (int o = 1; o < 32; o <<= 1) {
      const long long ua = __shfl_up_sync(0xffffffffu, a, o);
      const long long ub = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += ua;
        b += ub;
      }
    }
    if (c < lev.w) out[c + 1] = make_longlong2(c1 + a, c2 + b);
    c1 += __shfl_sync(0xffffffffu, a, 31);
    c2 += __shfl_sync(0xffffffffu, b, 31);
  }
}

// ---------------------------------------------------------------- coarse scan
// Dense score planes of the top level for the kept coarse patches
// (src/ncc_matching/matcher.cpp:542-579).  Block = 32x8 positions of one
// patch; the image tile with the patch's reach is staged in shared memory.
constexpr int kTileW = 32, kTileH = 8;

__global__ void __launch_bounds__(256) coarse_kernel(CoarseArgs a) {
  extern __shared__ float tile[];
  const int p = blockIdx.z;
  if (a.skip && a.skip[p]) return;  // plane written by the tensor-core scan
  const PatchDesc pd = a.view.patches[a.plist[p]];
  const PosRange rg = a.ranges[p];
  const int R0 = blockIdx.y * kTileH, C0 = blockIdx.x * kTileW;
  const int TW = kTileW + pd.cmax - pd.cmin, TH = kTileH + pd.rmax - pd.rmin;
  const int tid = threadIdx.y * kTileW + threadIdx.x;
  const int w = a.lev.w, h = a.lev.h;
  // tiles with no valid position only write -inf
  const bool any = R0 < rg.r1 && R0 + kTileH > rg.r0 && C0 < rg.c1 && C0 + kTileW > rg.c0;
  if (any) {
    for (int i = tid; i < TW * TH; i += 256) {
      const int gr = R0 + pd.rmin + i / TW, gc = C0 + pd.cmin + i % TW;
      tile[i] = (gr >= 0 && gc >= 0 && gr < h && gc < w) ? a.lev.v[size_t(gr) * w + gc] : 0.f;
    }
  }
  __syncthreads();
  const int r = R0 + threadIdx.y, c = C0 + threadIdx.x;
  if (r >= h || c >= w) return;
  float score = -INFINITY;
  if (any && r >= rg.r0 && r < rg.r1 && c >= rg.c0 && c < rg.c1 &&
      may_contain(a.dom, lattice_pose(a.crop_row, a.scale, r, pd.orow, a.phase),
                  lattice_pose(a.crop_col, a.scale, c, pd.ocol, a.phase), a.scale)) {
    const int2* sw = a.view.sw + pd.sample_off;
    const float* base = tile + (threadIdx.y - pd.rmin) * TW + (threadIdx.x - pd.cmin);
    const int2 f0 = __ldg(sw);
    const float s0 = base[off_row(f0.x) * TW + off_col(f0.x)];
    float acc0 = 0.f, acc1 = 0.f;
    int i = 0;
    for (; i + 1 < pd.n; i += 2) {
      const int2 x = __ldg(sw + i), y = __ldg(sw + i + 1);
      acc0 = fmaf(__int_as_float(x.y), base[off_row(x.x) * TW + off_col(x.x)] - s0, acc0);
      acc1 = fmaf(__int_as_float(y.y), base[off_row(y.x) * TW + off_col(y.x)] - s0, acc1);
    }
    if (i < pd.n) {
      const int2 x = __ldg(sw + i);
      acc0 = fmaf(__int_as_float(x.y), base[off_row(x.x) * TW + off_col(x.x)] - s0, acc0);
    }
    long long s1, s2;
    window_moments(a.lev, w + 1, r, c, a.view.run2 + pd.run_off, pd.nruns, s1, s2);
    score = window_score(acc0 + acc1, s1, s2, pd.n, a.absolute);
  }
  a.planes[(size_t(p) * h + r) * w + c] = score;
}

// Pseudo-candidates of the tensor-core coarse scan: per virtual source, one
// per 5x5 block of top-level positions, centred in the block; they are
// already grouped by source, so the order is the identity and a source's
// tiles are runs of 16 consecutive candidates.
__global__ void coarse_lattice_kernel(Cand* cand, int2* rc, int nsrc, int nbr, int nbc, const int32_t* group_of_src,
                                      int32_t* order, TcTiles* tiles, QueryState* state, int slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = nbr * nbc, tps = (nb + kTcCands - 1) / kTcCands;  // tiles per source
  if (i == 0) {
    state->count[slot] = nsrc * nb;
    tiles->count = nsrc * tps;
    tiles->next = 0;
  }
  if (i < nsrc * tps) {
    const int src = i / tps, u = i % tps;
    tiles->group[i] = group_of_src[src];
    tiles->first[i] = src * nb + u * kTcCands;
    tiles->last[i] = src * nb + min(nb, (u + 1) * kTcCands);
  }
  if (i >= nsrc * nb) return;
  const int b = i % nb;
  Cand c{};
  c.patch = i / nb;
  cand[i] = c;
  order[i] = i;
  rc[i] = make_int2(5 * (b / nbc) + 2, 5 * (b % nbc) + 2);
}

// Score planes of the patches the tensor cores correlated: one thread per
// plane position (consecutive threads, consecutive columns: coalesced moment
// loads); exact moments and the score as coarse_kernel computes them.
__global__ void coarse_tc_score_kernel(CoarseTcArgs a) {
  const int w = a.lev.w, h = a.lev.h;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)a.nplist * h * w) return;
  const int j = int(idx / ((long long)h * w)), rem = int(idx % ((long long)h * w));
  const int src = a.src_of[j];
  if (src < 0) return;  // coarse_kernel's plane
  const int r = rem / w, c = rem % w;
  const PosRange rg = a.ranges[j];
  float score = -INFINITY;
  const PatchDesc pd = a.view.patches[a.plist[j]];
  if (r >= rg.r0 && r < rg.r1 && c >= rg.c0 && c < rg.c1 &&
      may_contain(a.dom, lattice_pose(a.crop_row, a.scale, r, pd.orow, a.phase),
                  lattice_pose(a.crop_col, a.scale, c, pd.ocol, a.phase), a.scale)) {
    const int ci = (src * a.lat_r + r / 5) * a.lat_c + c / 5;
    const int pos = (r % 5) * 5 + c % 5, k = a.k_of[j];
    long long s1, s2;
    window_moments(a.lev, w + 1, r, c, a.view.run2 + pd.run_off, pd.nruns, s1, s2);
    // sum w (S - S0) = sum w S - S0 sum w (first sample S0)
    const int2 f0 = __ldg(a.view.sw + pd.sample_off);
    const float s0 = a.lev.v[size_t(r + off_row(f0.x)) * w + c + off_col(f0.x)];
    const float dot = fmaf(-s0, a.groups[a.group_of_src[src]].weff_k[k], a.dots[size_t(ci) * kTcScoreStride + k * 25 + pos]);
    score = window_score(dot, s1, s2, pd.n, a.absolute);
  }
  a.planes[idx] = score;
}

// 3x3 local maxima >= 0.4*MinScore with the reference's tie rule, compacted
// into the candidate list (src/ncc_matching/matcher.cpp:581-593).
__global__ void nms_kernel(NmsArgs a) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t plane = int64_t(a.w) * a.h;
  if (idx >= plane * a.nplist) return;
  const int p = int(idx / plane);
  const int rem = int(idx % plane);
  const int r = rem / a.w, c = rem % a.w;
  const float* s = a.planes + size_t(p) * plane;
  const float v = s[rem];
  if (!(v >= a.threshold) || !isfinite(v)) return;
  for (int dr = -1; dr <= 1; ++dr)
    for (int dc = -1; dc <= 1; ++dc) {
      const int rr = r + dr, cc = c + dc;
      if (rr < 0 || cc < 0 || rr >= a.h || cc >= a.w || (!dr && !dc)) continue;
      const float o = s[rr * a.w + cc];
      if (o > v || (o == v && (dr < 0 || (!dr && dc < 0)))) return;
    }
  const int k = atomicAdd(&a.state->count[0], 1);
  if (k >= a.max_candidates) {
    atomicExch(&a.state->overflow, 1);
    return;
  }
  const int32_t pi = a.plist[p];
  const PatchDesc pd = a.view.patches[pi];
  Cand out;
  out.row = lattice_pose(a.crop_row, a.scale, r, pd.orow, a.phase);
  out.col = lattice_pose(a.crop_col, a.scale, c, pd.ocol, a.phase);
  out.angle = pd.angle;
  out.score = double(v);
  out.patch = pi;
  out.pad = 0;
  a.out[k] = out;
}

// ------------------------------------------------------------------ tracking
// One block per candidate: the target level's query patches inside the
// candidate's angle window (a precomputed list per source patch), 5x5
// positions each; the first strict maximum in (patch order, dr, dc) wins
// (src/ncc_matching/matcher.cpp:670-757).
//
// The union image window of all those placements is staged in shared memory,
// centred on one of its pixels (exact small integers in float) with the
// level's fixed row pitch, so each sample costs one shared load and one FMA
// against precomputed linear offsets.  Each thread scores one (patch,
// position) item, or a slice of its samples when items are few.  Windows
// larger than the level's staged geometry read the level directly.
constexpr int kTrackThreads = 256;
constexpr int kTrackMaxSel = 64;

__global__ void __launch_bounds__(kTrackThreads, 5) track_kernel(TrackArgs a) {
  extern __shared__ float win[];
  const int i = blockIdx.x;
  if (i >= live_count(a.state, a.in_slot)) return;
  __shared__ int s_sel[kTrackMaxSel];
  __shared__ int s_row[kTrackMaxSel], s_col[kTrackMaxSel];
  __shared__ unsigned char s_istc[kTrackMaxSel];
  __shared__ int s_n, s_split, s_wr0, s_wc0, s_wh, s_wcols, s_staged;
  __shared__ float s_centre;
  __shared__ float s_part[kTrackThreads];
  // moment partials of the slices (launches with tensor-core items only)
  long long* s_m1 = a.split_off >= 0 ? reinterpret_cast<long long*>(win + a.split_off) : nullptr;
  long long* s_m2 = s_m1 ? s_m1 + kTrackThreads : nullptr;
  __shared__ float s_wbest[kTrackThreads / 32];
  __shared__ int s_word[kTrackThreads / 32];
  const Cand cd = a.in[i];
  const int WW = a.view.lin_pitch;
  __shared__ int s_b, s_tc, s_bound[2][4];
  __shared__ float s_xr32, s_xc32;
  __shared__ double s_xr, s_xc;
  if (threadIdx.x == 0) {
    const int src = cd.patch;
    const int b = src >= 0 ? a.sel_off[src] : 0, e = src >= 0 ? a.sel_off[src + 1] : 0;
    s_b = b;
    s_n = min(e - b, kTrackMaxSel);
    // rotated patches of a tensor-core group were scored by tc_track_kernel
    s_tc = a.tc_dots && src >= 0 && a.tc_group_of_src[src] >= 0;
    // window centres: round((pose - crop - offset) / step - origin)
    if (a.exact32) {
      s_xr32 = __fmul_rn(__fsub_rn(__fsub_rn(float(cd.row), float(a.crop_row)), float(a.offset)), float(1.0 / a.step));
      s_xc32 = __fmul_rn(__fsub_rn(__fsub_rn(float(cd.col), float(a.crop_col)), float(a.offset)), float(1.0 / a.step));
    } else {
      s_xr = dsub(dsub(cd.row, a.crop_row), a.offset) / a.step;
      s_xc = dsub(dsub(cd.col, a.crop_col), a.offset) / a.step;
    }
  }
  __syncthreads();
  {
    // one thread per selected patch (at most 64: warps 0 and 1)
    int wr0 = INT32_MAX, wc0 = INT32_MAX, wr1 = INT32_MIN, wc1 = INT32_MIN;
    const int k = threadIdx.x;
    if (k < s_n) {
      const int j = a.sel_idx[s_b + k];
      s_sel[k] = j;
      const PatchDesc pd = a.view.patches[a.plist[j]];
      int row, col;
      if (a.exact32) {
        row = int(roundf(__fsub_rn(s_xr32, float(pd.orow))));
        col = int(roundf(__fsub_rn(s_xc32, float(pd.ocol))));
      } else {
        row = int(round(dsub(s_xr, pd.orow)));
        col = int(round(dsub(s_xc, pd.ocol)));
      }
      s_row[k] = row;
      s_col[k] = col;
      const bool istc = s_tc && pd.orow == 0 && pd.ocol == 0 && k < 16;
      s_istc[k] = istc;
      const PosRange rg = a.ranges[j];
      // only placements scored here need image data
      const int r_lo = max(row - 2, rg.r0), r_hi = min(row + 2, rg.r1 - 1);
      const int c_lo = max(col - 2, rg.c0), c_hi = min(col + 2, rg.c1 - 1);
      if (!istc && r_lo <= r_hi && c_lo <= c_hi) {
        wr0 = r_lo + pd.rmin;
        wr1 = r_hi + pd.rmax;
        wc0 = c_lo + pd.cmin;
        wc1 = c_hi + pd.cmax;
      }
    }
    if (threadIdx.x < 64) {
      for (int o = 16; o > 0; o >>= 1) {
        wr0 = min(wr0, __shfl_xor_sync(0xffffffffu, wr0, o));
        wc0 = min(wc0, __shfl_xor_sync(0xffffffffu, wc0, o));
        wr1 = max(wr1, __shfl_xor_sync(0xffffffffu, wr1, o));
        wc1 = max(wc1, __shfl_xor_sync(0xffffffffu, wc1, o));
      }
      if ((threadIdx.x & 31) == 0) {
        s_bound[threadIdx.x >> 5][0] = wr0;
        s_bound[threadIdx.x >> 5][1] = wr1;
        s_bound[threadIdx.x >> 5][2] = wc0;
        s_bound[threadIdx.x >> 5][3] = wc1;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int n = s_n;
    const int wr0 = min(s_bound[0][0], s_bound[1][0]), wr1 = max(s_bound[0][1], s_bound[1][1]);
    const int wc0 = min(s_bound[0][2], s_bound[1][2]), wc1 = max(s_bound[0][3], s_bound[1][3]);
    const int items = n * 25;
    s_split = items > 0 ? max(1, min(8, kTrackThreads / items)) : 1;
    const bool any = wr0 <= wr1;
    s_wr0 = any ? wr0 : 0;
    s_wc0 = any ? wc0 : 0;
    s_wh = any ? wr1 - wr0 + 1 : 0;
    s_wcols = any ? wc1 - wc0 + 1 : 0;
    s_staged = any && s_wh <= a.view.lin_rows && s_wcols <= WW && a.staged_ok;
    s_centre = any ? a.lev.v[size_t(wr0 + (wr1 - wr0) / 2) * a.lev.w + wc0 + (wc1 - wc0) / 2] : 0.f;
  }
  __syncthreads();
  const int n = s_n, split = s_split;
  const int pitch = a.lev.w;
  const bool staged = s_staged != 0;
  const int wr0 = s_wr0, wc0 = s_wc0;
  const float centre = s_centre;
  if (staged) {
    const int cols = s_wcols, cells = s_wh * cols;
    for (int t = threadIdx.x; t < cells; t += kTrackThreads) {
      const int rr = t / cols, cc = t % cols;
      win[rr * WW + cc] = a.lev.v[size_t(wr0 + rr) * pitch + wc0 + cc] - centre;
    }
  }
  __syncthreads();
  float best = -INFINITY;
  int border = INT32_MAX;
  const int items = n * 25;
  const int passes = (items * split + kTrackThreads - 1) / kTrackThreads;
  for (int pass = 0; pass < passes; ++pass) {
    // slices are part-major: the lanes of a warp work on neighbouring
    // placements of one sample (broadcast sample loads)
    const int t = pass * kTrackThreads + threadIdx.x;
    const int item = split > 1 ? t % items : t, part = split > 1 ? t / items : 0;
    bool valid = false, is_tc = false;
    int r = 0, c = 0;
    PatchDesc pd{};
    float acc = 0.f, x0 = 0.f;
    if (item < items && part < split) {
      const int k = item / 25, pos = item % 25;
      const int j = s_sel[k];
      pd = a.view.patches[a.plist[j]];
      const PosRange rg = a.ranges[j];
      r = s_row[k] + pos / 5 - 2;
      c = s_col[k] + pos % 5 - 2;
      valid = r >= rg.r0 && r < rg.r1 && c >= rg.c0 && c < rg.c1 &&
              may_contain(a.dom, lattice_pose(a.crop_row, a.step, r, pd.orow, a.offset),
                          lattice_pose(a.crop_col, a.step, c, pd.ocol, a.offset), a.step);
      is_tc = s_istc[k] != 0;
    }
    if (is_tc) {
      // precomputed on the tensor cores
    } else if (valid && staged) {
      // sum w (S - centre); the first-sample shift is applied once below
      const int2* lw = a.view.lw + pd.sample_off;
      const float* base = win + (r - wr0) * WW + (c - wc0);
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
      int s = part;
      for (; s + 3 * split < pd.n; s += 4 * split) {
        const int2 p0 = __ldg(lw + s), p1 = __ldg(lw + s + split), p2 = __ldg(lw + s + 2 * split),
                   p3 = __ldg(lw + s + 3 * split);
        a0 = fmaf(__int_as_float(p0.y), base[p0.x], a0);
        a1 = fmaf(__int_as_float(p1.y), base[p1.x], a1);
        a2 = fmaf(__int_as_float(p2.y), base[p2.x], a2);
        a3 = fmaf(__int_as_float(p3.y), base[p3.x], a3);
      }
      for (; s < pd.n; s += split) {
        const int2 p0 = __ldg(lw + s);
        a0 = fmaf(__int_as_float(p0.y), base[p0.x], a0);
      }
      acc = (a0 + a1) + (a2 + a3);
      if (part == 0) x0 = base[__ldg(lw).x];
    } else if (valid) {
      const int2* sw = a.view.sw + pd.sample_off;
      const float* base = a.lev.v + size_t(r) * pitch + c;
      const int2 f0 = __ldg(sw);
      const float s0 = base[off_row(f0.x) * pitch + off_col(f0.x)];
      float acc1 = 0.f;
      int s = part;
      for (; s + split < pd.n; s += 2 * split) {
        const int2 x = __ldg(sw + s), y = __ldg(sw + s + split);
        acc = fmaf(__int_as_float(x.y), base[off_row(x.x) * pitch + off_col(x.x)] - s0, acc);
        acc1 = fmaf(__int_as_float(y.y), base[off_row(y.x) * pitch + off_col(y.x)] - s0, acc1);
      }
      if (s < pd.n) {
        const int2 x = __ldg(sw + s);
        acc = fmaf(__int_as_float(x.y), base[off_row(x.x) * pitch + off_col(x.x)] - s0, acc);
      }
      acc += acc1;
    }
    // window moments: with scratch, the runs split over the item's slices
    // like the samples; otherwise in slice 0
    long long s1 = 0, s2 = 0;
    if (valid && (s_m1 || part == 0))
      window_moments(a.lev, pitch + 1, r, c, a.view.run2 + pd.run_off, pd.nruns, s1,
                     s2, s_m1 ? part : 0, s_m1 ? split : 1);
    // combine the slices of one item (threads item + q * items)
    if (split > 1) {
      s_part[threadIdx.x] = acc;
      if (s_m1) {
        s_m1[threadIdx.x] = s1;
        s_m2[threadIdx.x] = s2;
      }
      __syncthreads();
    }
    if (part == 0 && valid) {
      float dot;
      if (is_tc) {
        // sum w (S - S0) = sum w S - S0 sum w (first sample S0)
        const int k = item / 25;
        const int2 f0 = __ldg(a.view.sw + pd.sample_off);
        const float s0 = a.lev.v[size_t(r + off_row(f0.x)) * pitch + c + off_col(f0.x)];
        dot = fmaf(-s0, a.tc_groups[a.tc_group_of_src[cd.patch]].weff_k[k],
                   a.tc_dots[size_t(i) * kTcScoreStride + item]);
      } else {
        dot = acc;
        for (int q = 1; q < split; ++q) dot += s_part[threadIdx.x + q * items];
        // sum w (S - S0) = sum w (S - centre) - (S0 - centre) sum w
        if (staged) dot = fmaf(-x0, pd.wsum, dot);
      }
      if (s_m1)
        for (int q = 1; q < split; ++q) {
          s1 += s_m1[threadIdx.x + q * items];
          s2 += s_m2[threadIdx.x + q * items];
        }
      const float sc = window_score(dot, s1, s2, pd.n, a.absolute);
      if (better(sc, item, best, border)) {
        best = sc;
        border = item;
      }
    }
    if (split > 1) __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ob = __shfl_down_sync(0xffffffffu, best, o);
    const int oo = __shfl_down_sync(0xffffffffu, border, o);
    if (better(ob, oo, best, border)) {
      best = ob;
      border = oo;
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_wbest[warp] = best;
    s_word[warp] = border;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float bs = -INFINITY;
    int bo = INT32_MAX;
    unsigned long long macs = 0;
    for (int w = 0; w < kTrackThreads / 32; ++w)
      if (better(s_wbest[w], s_word[w], bs, bo)) {
        bs = s_wbest[w];
        bo = s_word[w];
      }
    for (int k = 0; k < n; ++k)
      if (!s_istc[k]) macs += 25ull * (unsigned long long)a.view.patches[a.plist[s_sel[k]]].n;
    atomicAdd(&a.state->track_macs, macs);
    Cand out = cd;
    out.score = -INFINITY;
    if (bo != INT32_MAX && bs > -INFINITY) {
      const int k = bo / 25, l = bo % 25;
      const int32_t pi = a.plist[s_sel[k]];
      const PatchDesc pd = a.view.patches[pi];
      const int r = s_row[k] + l / 5 - 2, c = s_col[k] + l % 5 - 2;
      if (a.exact32) {
        out.row = double(lattice_pose32(float(a.crop_row), float(a.step), r, float(pd.orow), float(a.offset)));
        out.col = double(lattice_pose32(float(a.crop_col), float(a.step), c, float(pd.ocol), float(a.offset)));
      } else {
        out.row = lattice_pose(a.crop_row, a.step, r, pd.orow, a.offset);
        out.col = lattice_pose(a.crop_col, a.step, c, pd.ocol, a.offset);
      }
      out.angle = pd.angle;
      out.score = double(bs);
      out.patch = pi;
    }
    a.out[i] = out;
  }
}

// ------------------------------------------------------------ merge_identical
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// Snap poses outside the image to the nearest in-image pixel within 4 rows
// and columns (full-image domain; src/ncc_matching/matcher.cpp:633-643).
__device__ void snap_pose(Cand& p, double height, double width) {
  const double rr = floor(p.row + .5), cc = floor(p.col + .5);
  if (rr >= 0 && cc >= 0 && rr < height && cc < width) return;
  double best = INFINITY, nr = p.row, nc = p.col;
  const double first = fmax(0., ceil(p.row - 4));
  for (double r = first; r <= p.row + 4 && r < height; r += 1) {
    const double c = fmin(fmax(round(p.col), 0.), width - 1);
    if (fabs(c - p.col) > 4) continue;
    const double dist = hypot(r - p.row, c - p.col);
    if (dist < best) {
      best = dist;
      nr = r;
      nc = c;
    }
  }
  if (isfinite(best)) {
    p.row = nr;
    p.col = nc;
    p.patch = -1;
  } else {
    p.score = -INFINITY;
  }
}

// The same for a reduced domain: the nearest pixel of the domain's runs
// within 4 rows and columns; runs are visited in (row, begin) order and only
// a strictly nearer one replaces the best (src/ncc_matching/matcher.cpp:633-643).
__device__ void snap_pose_domain(Cand& p, const DomainView& d) {
  if (domain_contains(d, p.row, p.col)) return;
  double best = INFINITY, nr = p.row, nc = p.col;
  const int first = max(0, int(ceil(p.row - 4)));
  const double rc = round(p.col);
  for (int y = first; y < d.h && y <= p.row + 4; ++y)
    for (int k = d.row_run[y]; k < d.row_run[y + 1]; ++k) {
      const int4 run = d.runs[k];
      const double c = fmin(fmax(rc, double(run.y)), double(run.z));
      if (fabs(c - p.col) > 4) continue;
      const double dist = hypot(double(run.x) - p.row, c - p.col);
      if (dist < best) {
        best = dist;
        nr = double(run.x);
        nc = c;
      }
    }
  if (isfinite(best)) {
    p.row = nr;
    p.col = nc;
    p.patch = -1;
  } else {
    p.score = -INFINITY;
  }
}

__global__ void snap_kernel(Cand* c, const QueryState* state, int slot, double height, double width, DomainView dom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= live_count(state, slot)) return;
  Cand p = c[i];
  if (dom.mask)
    snap_pose_domain(p, dom);
  else
    snap_pose(p, height, width);
  c[i] = p;
}

// merge_identical + threshold (src/ncc_matching/matcher.cpp:241-248,758-760):
// keep one candidate per exact (row, column, angle), drop non-finite scores
// and scores below the threshold; order is irrelevant downstream.
__global__ void dedup_kernel(DedupArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= live_count(a.state, a.in_slot)) return;
  const Cand p = a.in[i];
  if (!isfinite(p.score) || p.score < a.threshold) return;
  const unsigned long long kr = __double_as_longlong(p.row), kc = __double_as_longlong(p.col),
                           ka = __double_as_longlong(p.angle);
  const unsigned mask = unsigned(a.hash_slots - 1);
  unsigned slot = unsigned(mix64(kr ^ mix64(kc ^ mix64(ka)))) & mask;
  for (int probe = 0; probe < a.hash_slots; ++probe) {
    const int prev = atomicCAS(a.table + slot, -1, i);
    if (prev == -1) {
      const int k = atomicAdd(&a.state->count[a.out_slot], 1);
      a.out[k] = p;
      return;
    }
    const Cand q = a.in[prev];
    if ((unsigned long long)__double_as_longlong(q.row) == kr && (unsigned long long)__double_as_longlong(q.col) == kc &&
        (unsigned long long)__double_as_longlong(q.angle) == ka)
      return;
    slot = (slot + 1) & mask;
  }
}

// -------------------------------------------------- full-resolution scoring
// Totals of K per-thread values as FP32 pairs; valid on thread 0 only.
// scratch: K*64 floats.
template <int K>
__device__ void block_total(const float (&v)[K], F2 (&out)[K], float* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    F2 x = f2(v[k]);
    for (int o = 16; o > 0; o >>= 1) {
      const F2 y{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
      x = f2_add(x, y);
    }
    if (lane == 0) {
      scratch[(k * 32 + warp) * 2] = x.hi;
      scratch[(k * 32 + warp) * 2 + 1] = x.lo;
    }
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      F2 y = lane < nw ? F2{scratch[(k * 32 + lane) * 2], scratch[(k * 32 + lane) * 2 + 1]} : F2{0.f, 0.f};
      for (int o = 16; o > 0; o >>= 1) {
        const F2 z{__shfl_down_sync(0xffffffffu, y.hi, o), __shfl_down_sync(0xffffffffu, y.lo, o)};
        y = f2_add(y, z);
      }
      out[k] = y;
    }
  }
  __syncthreads();
}

// Pose in the frame of an integer anchor.
struct LocalPose {
  int R0, C0;        // integer anchor
  float fr, fc;      // fractional part of the pose relative to the anchor
  float ca, sa;
};

__device__ __forceinline__ LocalPose make_local(double row, double col, double angle) {
  LocalPose l;
  const double fr = floor(row), fc = floor(col);
  l.R0 = int(fr);
  l.C0 = int(fc);
  l.fr = float(row - fr);
  l.fc = float(col - fc);
  sincosf(float(angle), &l.sa, &l.ca);
  return l;
}

// True when every sample of the rotated original lies inside the image by a
// margin: the sample positions are affine in (dr, dc), so the corners of the
// offset box bound them (the margin covers FP32 rounding of the per-sample
// expressions).  Inside, the passes drop their per-sample bounds tests.
__device__ __forceinline__ bool samples_inside(const LocalPose& L, const OriginalView& o, float hmin, float hmax,
                                               float wmin, float wmax) {
  float y0 = INFINITY, y1 = -INFINITY, x0 = INFINITY, x1 = -INFINITY;
  const float drs[2] = {o.dr_min, o.dr_max}, dcs[2] = {o.dc_min, o.dc_max};
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float y = L.fr + (L.ca * drs[i] - L.sa * dcs[j]), x = L.fc + (L.sa * drs[i] + L.ca * dcs[j]);
      y0 = fminf(y0, y);
      y1 = fmaxf(y1, y);
      x0 = fminf(x0, x);
      x1 = fmaxf(x1, x);
    }
  const float m = 1e-2f;
  return y0 >= hmin + m && x0 >= wmin + m && y1 <= hmax - 1.f - m && x1 <= wmax - 1.f - m;
}

// Shared state of a block working on one pose at a time.
struct PoseShared {
  LocalPose lp;
  double score;       // result of the last continuous pass
  int ok;             // result flag of the last Gauss-Newton pass
  double gscore;      // score seen by the last Gauss-Newton pass (-inf if none)
  double delta[3];
  float scratch[19 * 64];
};

__device__ __forceinline__ float bilinear_at(const ImageView& img, int r, int c, float fy, float fx, int r1, int c1) {
  const float* v = img.v;
  return (1 - fy) * ((1 - fx) * __ldg(v + size_t(r) * img.w + c) + fx * __ldg(v + size_t(r) * img.w + c1)) +
         fy * ((1 - fx) * __ldg(v + size_t(r1) * img.w + c) + fx * __ldg(v + size_t(r1) * img.w + c1));
}

// FP32 score from pair totals of sum q, sum q^2, sum w q.
__device__ __forceinline__ float pair_score(F2 sum, F2 sq, F2 dot, int n, int absolute, bool* ok) {
  const F2 var = f2_sub(sq, f2_div(f2_mul(sum, sum), f2(float(n))));
  const float v = f2_val(var);
  *ok = v > 0;
  if (!*ok) return -INFINITY;
  float s = fminf(1.f, fmaxf(-1.f, f2_val(dot) / sqrtf(v)));
  return absolute ? fabsf(s) : s;
}

// continuous() of src/ncc_matching/matcher.cpp:144-156 at a level-local pose;
// every thread of the block calls it; sh.score holds the result afterwards.
__device__ void continuous_pass(const ImageView& img, const OriginalView& orig, double row, double col, double angle,
                                int absolute, PoseShared& sh) {
  if (threadIdx.x == 0) sh.lp = make_local(row, col, angle);
  __syncthreads();
  const LocalPose L = sh.lp;
  const float hmax = float(img.h - 1 - L.R0), wmax = float(img.w - 1 - L.C0);
  const float hmin = float(-L.R0), wmin = float(-L.C0);
  float offset = 0.f;
  {
    const float dr = orig.dr[0], dc = orig.dc[0];
    const float y = L.fr + (L.ca * dr - L.sa * dc), x = L.fc + (L.sa * dr + L.ca * dc);
    if (y >= hmin && x >= wmin && y <= hmax && x <= wmax) {
      const float fy0 = floorf(y), fx0 = floorf(x);
      const int r = L.R0 + int(fy0), c = L.C0 + int(fx0);
      offset = bilinear_at(img, r, c, y - fy0, x - fx0, min(r + 1, img.h - 1), min(c + 1, img.w - 1));
    }
  }
  float acc[4] = {0.f, 0.f, 0.f, 0.f};  // sum q, sum q^2, sum w q, out-of-image flag
  if (samples_inside(L, orig, hmin, hmax, wmin, wmax)) {
    // every sample and its 2x2 neighbourhood is inside: no tests, 32-bit offsets
    const float* base = img.v + (size_t(L.R0) * img.w + L.C0);
    const uint32_t* pbase = img.pairs ? img.pairs + (size_t(L.R0) * img.w + L.C0) : nullptr;
    const int w = img.w;
    // four samples per step, all loads issued before the arithmetic; each
    // thread still adds its samples in order s, s + blockDim.x, ...
    constexpr int U = 4;
    const int stride = blockDim.x;
    for (int s0 = threadIdx.x; s0 < orig.n; s0 += U * stride) {
      float4 p[U];
      float fy[U], fx[U], va[U], vb[U], vd[U], ve[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u * stride;
        p[u] = s < orig.n ? __ldg(orig.dcw + s) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float y = L.fr + (L.ca * p[u].x - L.sa * p[u].y), x = L.fc + (L.sa * p[u].x + L.ca * p[u].y);
        const int iy = __float2int_rd(y), ix = __float2int_rd(x);
        fy[u] = y - float(iy);
        fx[u] = x - float(ix);
        if (pbase) {
          const uint32_t* pp = pbase + (iy * w + ix);
          const uint32_t aq = __ldg(pp), bq = __ldg(pp + w);
          va[u] = __half2float(__ushort_as_half(aq & 0xffff));
          vb[u] = __half2float(__ushort_as_half(aq >> 16));
          vd[u] = __half2float(__ushort_as_half(bq & 0xffff));
          ve[u] = __half2float(__ushort_as_half(bq >> 16));
        } else {
          const float* v = base + (iy * w + ix);
          va[u] = __ldg(v);
          vb[u] = __ldg(v + 1);
          vd[u] = __ldg(v + w);
          ve[u] = __ldg(v + w + 1);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (s0 + u * stride >= orig.n) break;
        const float q = (1 - fy[u]) * ((1 - fx[u]) * va[u] + fx[u] * vb[u]) +
                        fy[u] * ((1 - fx[u]) * vd[u] + fx[u] * ve[u]) - offset;
        acc[0] += q;
        acc[1] = fmaf(q, q, acc[1]);
        acc[2] = fmaf(p[u].z, q, acc[2]);
      }
    }
  } else
  for (int s = threadIdx.x; s < orig.n; s += blockDim.x) {
    const float dr = __ldg(orig.dr + s), dc = __ldg(orig.dc + s), w = __ldg(orig.w + s);
    const float y = L.fr + (L.ca * dr - L.sa * dc), x = L.fc + (L.sa * dr + L.ca * dc);
    if (!(y >= hmin && x >= wmin && y <= hmax && x <= wmax)) {
      acc[3] = 1.f;
      continue;
    }
    const float fy0 = floorf(y), fx0 = floorf(x);
    const int r = L.R0 + int(fy0), c = L.C0 + int(fx0);
    const float q = bilinear_at(img, r, c, y - fy0, x - fx0, min(r + 1, img.h - 1), min(c + 1, img.w - 1)) - offset;
    acc[0] += q;
    acc[1] = fmaf(q, q, acc[1]);
    acc[2] = fmaf(w, q, acc[2]);
  }
  F2 t[4];
  block_total<4>(acc, t, sh.scratch);
  if (threadIdx.x == 0) {
    bool ok = false;
    const float sc = t[3].hi > 0 ? -INFINITY : pair_score(t[0], t[1], t[2], orig.n, absolute, &ok);
    sh.score = (t[3].hi > 0 || !ok) ? -INFINITY : double(sc);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(128, 12) score_kernel(ScoreArgs a) {
  __shared__ PoseShared sh;
  const int i = blockIdx.x;
  if (i >= live_count(a.state, a.slot)) return;
  const Cand c = a.cand[i];
  if (!isfinite(c.score)) return;
  const double row = (c.row - a.crop_row - a.phase) / a.scale;
  const double col = (c.col - a.crop_col - a.phase) / a.scale;
  continuous_pass(a.img, a.orig, row, col, c.angle, a.absolute, sh);
  if (threadIdx.x == 0) a.cand[i].score = sh.score;
}

// ------------------------------------------------------------- NCC adjoint
// Scale degree of freedom (no counterpart in the rigid reference).  Sample i
// of the original (offsets dr, dc from the model origin, weight w) lands at
//   y = row + s (ca dr - sa dc),  x = col + s (sa dr + ca dc),
// q_i is the bilinear image value there, and
//   NCC = D / sqrt(E),  D = sum w q - (sum q / n) sum w,  E = sum q^2 - (sum q)^2 / n
// (continuous(), src/ncc_matching/matcher.cpp:121-157, with the scale).  With
// the bilinear cell gradient (gy, gx), dq/dp = gy dy/dp + gx dx/dp for p in
// (row, col, angle, scale), and
//   dNCC = dD / sqrt(E) - D dE / (2 E^1.5),
//   dD = sum w dq - (sum dq / n) sum w,  dE = 2 sum q dq - 2 (sum q)(sum dq) / n.
// Per-thread sums in FP32 (q centred by the first sample, which changes
// neither NCC nor its gradient), block totals as FP32 pairs, the final
// algebra in FP64.
constexpr int kAdjointThreads = 256;

__global__ void __launch_bounds__(kAdjointThreads) adjoint_kernel(AdjointArgs a) {
  __shared__ float scratch[17 * 64];
  __shared__ float s_off;
  const int k = blockIdx.x;
  if (k >= a.n) return;
  const double row = a.poses[4 * k], col = a.poses[4 * k + 1], angle = a.poses[4 * k + 2],
               scale = a.poses[4 * k + 3];
  const ImageView img = a.img;
  const OriginalView orig = a.orig;
  const double R = floor(row), Cc = floor(col);
  const int R0 = int(R), C0 = int(Cc);
  const float fr = float(row - R), fc = float(col - Cc);
  double sd, cd;
  sincos(angle, &sd, &cd);
  const float ca = float(cd), sa = float(sd), sc = float(scale);
  const float hmin = float(-R0), wmin = float(-C0), hmax = float(img.h - 1 - R0), wmax = float(img.w - 1 - C0);
  if (threadIdx.x == 0) {
    float off = 0.f;
    const float u = ca * orig.dr[0] - sa * orig.dc[0], v = sa * orig.dr[0] + ca * orig.dc[0];
    const float y = fr + sc * u, x = fc + sc * v;
    if (y >= hmin && x >= wmin && y <= hmax && x <= wmax) {
      const float fy0 = floorf(y), fx0 = floorf(x);
      const int r = R0 + int(fy0), c = C0 + int(fx0);
      off = bilinear_at(img, r, c, y - fy0, x - fx0, min(r + 1, img.h - 1), min(c + 1, img.w - 1));
    }
    s_off = off;
  }
  __syncthreads();
  const float off = s_off;
  // 0 sum q, 1 sum q^2, 2 sum w q, 3..6 sum dq, 7..10 sum q dq, 11..14 sum w dq, 15 sum w, 16 outside
  float acc[17];
#pragma unroll
  for (int j = 0; j < 17; ++j) acc[j] = 0.f;
  for (int s = threadIdx.x; s < orig.n; s += blockDim.x) {
    const float4 p = __ldg(orig.dcw + s);
    const float u = ca * p.x - sa * p.y, v = sa * p.x + ca * p.y;
    const float y = fr + sc * u, x = fc + sc * v;
    acc[15] += p.z;
    if (!(y >= hmin && x >= wmin && y <= hmax && x <= wmax)) {
      acc[16] = 1.f;
      continue;
    }
    const float fy0 = floorf(y), fx0 = floorf(x);
    const float fy = y - fy0, fx = x - fx0;
    const int r = R0 + int(fy0), c = C0 + int(fx0);
    const int r1 = min(r + 1, img.h - 1), c1 = min(c + 1, img.w - 1);
    const float va = __ldg(img.v + size_t(r) * img.w + c), vb = __ldg(img.v + size_t(r) * img.w + c1);
    const float vd = __ldg(img.v + size_t(r1) * img.w + c), ve = __ldg(img.v + size_t(r1) * img.w + c1);
    const float q = (1 - fy) * ((1 - fx) * va + fx * vb) + fy * ((1 - fx) * vd + fx * ve) - off;
    const float gy = (1 - fx) * (vd - va) + fx * (ve - vb), gx = (1 - fy) * (vb - va) + fy * (ve - vd);
    // dy/dp, dx/dp: row (1, 0), col (0, 1), angle (-s v, s u), scale (u, v)
    const float dq[4] = {gy, gx, sc * (gx * u - gy * v), gy * u + gx * v};
    acc[0] += q;
    acc[1] = fmaf(q, q, acc[1]);
    acc[2] = fmaf(p.z, q, acc[2]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      acc[3 + j] += dq[j];
      acc[7 + j] = fmaf(q, dq[j], acc[7 + j]);
      acc[11 + j] = fmaf(p.z, dq[j], acc[11 + j]);
    }
  }
  F2 t[17];
  block_total<17>(acc, t, scratch);
  if (threadIdx.x == 0) {
    auto dv = [](const F2& x) { return double(x.hi) + double(x.lo); };
    const double n = double(orig.n);
    const double sq = dv(t[0]), sqq = dv(t[1]), swq = dv(t[2]), sw = dv(t[15]);
    const double D = swq - sq / n * sw, E = sqq - sq * sq / n;
    double* g = a.grad + 4 * k;
    if (t[16].hi > 0 || !(E > 0)) {
      a.score[k] = -INFINITY;
      g[0] = g[1] = g[2] = g[3] = 0;
      return;
    }
    const double rs = 1 / sqrt(E);
    double ncc = D * rs;
    const double sign = a.absolute && ncc < 0 ? -1. : 1.;
    a.score[k] = sign * ncc;
    for (int j = 0; j < 4; ++j) {
      const double sdq = dv(t[3 + j]), sqdq = dv(t[7 + j]), swdq = dv(t[11 + j]);
      const double dD = swdq - sdq / n * sw, dE = 2 * (sqdq - sq * sdq / n);
      g[j] = sign * (dD * rs - D * dE * .5 * rs * rs * rs);
    }
  }
}

// Similarity pass for the 4-parameter refinement: per-thread sums of
// 0 q, 1 q^2, 2 w q, 3..6 g, 7..10 q g, 11..14 w g, 15..24 g_i g_j (i <= j),
// 25 w, 26 outside, with g = dq / d(row, col, angle, scale).
constexpr int kSimSums = 27;

__device__ void sim_pass(const ImageView& img, const OriginalView& orig, const double* pose, bool derivs,
                         float (&acc)[kSimSums], float* s_off) {
  const double R = floor(pose[0]), Cc = floor(pose[1]);
  const int R0 = int(R), C0 = int(Cc);
  const float fr = float(pose[0] - R), fc = float(pose[1] - Cc);
  double sd, cd;
  sincos(pose[2], &sd, &cd);
  const float ca = float(cd), sa = float(sd), sc = float(pose[3]);
  const float hmin = float(-R0), wmin = float(-C0), hmax = float(img.h - 1 - R0), wmax = float(img.w - 1 - C0);
  __syncthreads();
  if (threadIdx.x == 0) {
    float off = 0.f;
    const float u = ca * orig.dr[0] - sa * orig.dc[0], v = sa * orig.dr[0] + ca * orig.dc[0];
    const float y = fr + sc * u, x = fc + sc * v;
    if (y >= hmin && x >= wmin && y <= hmax && x <= wmax) {
      const float fy0 = floorf(y), fx0 = floorf(x);
      const int r = R0 + int(fy0), c = C0 + int(fx0);
      off = bilinear_at(img, r, c, y - fy0, x - fx0, min(r + 1, img.h - 1), min(c + 1, img.w - 1));
    }
    *s_off = off;
  }
  __syncthreads();
  const float off = *s_off;
#pragma unroll
  for (int j = 0; j < kSimSums; ++j) acc[j] = 0.f;
  for (int s = threadIdx.x; s < orig.n; s += blockDim.x) {
    const float4 p = __ldg(orig.dcw + s);
    const float u = ca * p.x - sa * p.y, v = sa * p.x + ca * p.y;
    const float y = fr + sc * u, x = fc + sc * v;
    acc[25] += p.z;
    if (!(y >= hmin && x >= wmin && y <= hmax && x <= wmax)) {
      acc[26] = 1.f;
      continue;
    }
    const float fy0 = floorf(y), fx0 = floorf(x);
    const float fy = y - fy0, fx = x - fx0;
    const int r = R0 + int(fy0), c = C0 + int(fx0);
    const int r1 = min(r + 1, img.h - 1), c1 = min(c + 1, img.w - 1);
    const float va = __ldg(img.v + size_t(r) * img.w + c), vb = __ldg(img.v + size_t(r) * img.w + c1);
    const float vd = __ldg(img.v + size_t(r1) * img.w + c), ve = __ldg(img.v + size_t(r1) * img.w + c1);
    const float q = (1 - fy) * ((1 - fx) * va + fx * vb) + fy * ((1 - fx) * vd + fx * ve) - off;
    acc[0] += q;
    acc[1] = fmaf(q, q, acc[1]);
    acc[2] = fmaf(p.z, q, acc[2]);
    if (!derivs) continue;
    const float gy = (1 - fx) * (vd - va) + fx * (ve - vb), gx = (1 - fy) * (vb - va) + fy * (ve - vd);
    const float g[4] = {gy, gx, sc * (gx * u - gy * v), gy * u + gx * v};
    int at = 15;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc[3 + i] += g[i];
      acc[7 + i] = fmaf(q, g[i], acc[7 + i]);
      acc[11 + i] = fmaf(p.z, g[i], acc[11 + i]);
#pragma unroll
      for (int j = i; j < 4; ++j) {
        acc[at] = fmaf(g[i], g[j], acc[at]);
        ++at;
      }
    }
  }
}

// One block per pose.  Each iteration: the normal equations of the NCC in
// the four parameters (Gauss-Newton on the centred, normalised samples, as
// the reference's refinement_step), an FP64 Gauss-Jordan solve with partial
// pivoting, the step clipped to the limits, and up to four halvings; a step
// is taken only when the score strictly increases.
constexpr int kRefine4Threads = 256;

__global__ void __launch_bounds__(kRefine4Threads) refine4_kernel(Refine4Args a) {
  __shared__ float scratch[kSimSums * 64];
  __shared__ float s_off;
  __shared__ double s_pose[4], s_try[4], s_delta[4], s_score, s_factor;
  __shared__ int s_go;
  const int k = blockIdx.x;
  if (k >= a.n) return;
  if (threadIdx.x < 4) s_pose[threadIdx.x] = a.poses[4 * k + threadIdx.x];
  if (threadIdx.x == 0) s_score = -INFINITY;
  __syncthreads();
  float acc[kSimSums];
  F2 t[kSimSums];
  auto dv = [](const F2& x) { return double(x.hi) + double(x.lo); };
  const double n = double(a.orig.n);
  for (int it = 0; it <= a.iterations; ++it) {
    sim_pass(a.img, a.orig, s_pose, true, acc, &s_off);
    block_total<kSimSums>(acc, t, scratch);
    if (threadIdx.x == 0) {
      s_go = 0;
      const double sq = dv(t[0]), sqq = dv(t[1]), swq = dv(t[2]), sw = dv(t[25]);
      const double E = sqq - sq * sq / n, D = swq - sq / n * sw;
      if (t[26].hi == 0 && E > 0) {
        const double rs = 1 / sqrt(E);
        const double ncc = D * rs, sign = a.absolute && ncc < 0 ? -1. : 1.;
        s_score = sign * ncc;
        if (it < a.iterations) {
          double m[4][5];
          double gi[4], qi[4];
          for (int i = 0; i < 4; ++i) {
            gi[i] = dv(t[3 + i]);
            qi[i] = dv(t[7 + i]) - sq / n * gi[i];
          }
          int at = 15;
          for (int i = 0; i < 4; ++i)
            for (int j = i; j < 4; ++j, ++at) {
              const double e = ((dv(t[at]) - gi[i] * gi[j] / n) - qi[i] * qi[j] / E) / E;
              m[i][j] = m[j][i] = e;
            }
          for (int i = 0; i < 4; ++i)
            m[i][4] = sign * (dv(t[11 + i]) - gi[i] / n * sw) * rs - s_score * qi[i] / E;
          bool good = true;
          for (int i = 0; i < 4 && good; ++i) {
            int pv = i;
            for (int j = i + 1; j < 4; ++j)
              if (fabs(m[j][i]) > fabs(m[pv][i])) pv = j;
            if (fabs(m[pv][i]) < 1e-14) {
              good = false;
              break;
            }
            for (int c = i; c < 5; ++c) {
              const double tmp = m[i][c];
              m[i][c] = m[pv][c];
              m[pv][c] = tmp;
            }
            const double inv = 1 / m[i][i];
            for (int c = i; c < 5; ++c) m[i][c] *= inv;
            for (int j = 0; j < 4; ++j)
              if (j != i) {
                const double f = m[j][i];
                for (int c = i; c < 5; ++c) m[j][c] -= f * m[i][c];
              }
          }
          if (good) {
            for (int i = 0; i < 4; ++i) s_delta[i] = m[i][4];
            double f = 1;
            f = fmin(f, a.max_shift / fmax(1e-20, fabs(s_delta[0])));
            f = fmin(f, a.max_shift / fmax(1e-20, fabs(s_delta[1])));
            f = fmin(f, a.max_angle / fmax(1e-20, fabs(s_delta[2])));
            f = fmin(f, a.max_scale / fmax(1e-20, fabs(s_delta[3])));
            s_factor = f;
            s_go = isfinite(f) && isfinite(s_delta[0]) && isfinite(s_delta[1]) && isfinite(s_delta[2]) &&
                   isfinite(s_delta[3]);
          }
        }
      }
    }
    __syncthreads();
    if (!s_go) break;
    bool accepted = false;
    for (int bt = 0; bt < 4 && !accepted; ++bt) {
      if (threadIdx.x < 4) s_try[threadIdx.x] = s_pose[threadIdx.x] + ldexp(s_factor, -bt) * s_delta[threadIdx.x];
      __syncthreads();
      sim_pass(a.img, a.orig, s_try, false, acc, &s_off);
      block_total<kSimSums>(acc, t, scratch);
      if (threadIdx.x == 0) {
        const double sq = dv(t[0]), sqq = dv(t[1]), swq = dv(t[2]), sw = dv(t[25]);
        const double E = sqq - sq * sq / n, D = swq - sq / n * sw;
        s_go = 0;
        if (t[26].hi == 0 && E > 0) {
          const double ncc = D / sqrt(E), sc = a.absolute ? fabs(ncc) : ncc;
          if (sc > s_score) {
            for (int i = 0; i < 4; ++i) s_pose[i] = s_try[i];
            s_go = 1;
          }
        }
      }
      __syncthreads();
      accepted = s_go != 0;
    }
    if (!accepted) break;
    if (threadIdx.x == 0) {
      const double st = s_factor;
      s_go = hypot(st * s_delta[0], st * s_delta[1]) >= 1e-4 || fabs(st * s_delta[2]) >= 1e-5 ||
             fabs(st * s_delta[3]) >= 1e-6;
    }
    __syncthreads();
    if (!s_go) {
      // converged: the score at the final pose
      sim_pass(a.img, a.orig, s_pose, false, acc, &s_off);
      block_total<kSimSums>(acc, t, scratch);
      if (threadIdx.x == 0) {
        const double sq = dv(t[0]), sqq = dv(t[1]), swq = dv(t[2]), sw = dv(t[25]);
        const double E = sqq - sq * sq / n, D = swq - sq / n * sw;
        s_score = t[26].hi == 0 && E > 0 ? (a.absolute ? fabs(D / sqrt(E)) : D / sqrt(E)) : -INFINITY;
      }
      __syncthreads();
      break;
    }
  }
  if (threadIdx.x < 4) a.poses[4 * k + threadIdx.x] = s_pose[threadIdx.x];
  if (threadIdx.x == 0) a.score[k] = s_score;
}

// --------------------------------------------------------------------- sort
// fp16 pairs (v[x], v[x+1]) of an fp16-exact level (last column repeats).
__global__ void pairs_kernel(const float* __restrict__ v, int w, int h, uint32_t* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)w * h) return;
  const int x = int(i % w);
  const __half a = __float2half_rn(v[i]), b = __float2half_rn(v[x + 1 < w ? i + 1 : i]);
  out[i] = uint32_t(__half_as_ushort(a)) | (uint32_t(__half_as_ushort(b)) << 16);
}

// 64-bit keys ordering scores descending (order-preserving bit transform).
__device__ __forceinline__ unsigned long long desc_key(double s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(s);
  const unsigned long long asc = (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
  return ~asc;
}

// Rank sort: the output position of a candidate is the number of candidates
// before it in the reference's order (score descending, then row, column,
// angle; matcher.cpp:824-827).  Poses are unique after the merge, so the
// ranks are a permutation.  A block ranks 64 candidates, four threads each
// counting over a quarter of every 2048-key tile of the list in shared
// memory; pose ties (equal keys) read the poses from global memory.
constexpr int kSortPer = 64;
__global__ void __launch_bounds__(256) sort_kernel(SortArgs a) {
  __shared__ unsigned long long s_key[2048];
  __shared__ int s_finite;
  const int n = live_count(a.state, a.slot);
  if (int(blockIdx.x) * kSortPer >= n) return;
  if (a.keys && n > kRankSortMax) return;  // the bitonic sort takes it
  const int lane4 = threadIdx.x & 3;
  const int i = blockIdx.x * kSortPer + (threadIdx.x >> 2);
  Cand me{};
  unsigned long long key = ~0ULL;
  if (i < n) {
    me = a.in[i];
    key = desc_key(me.score);
  }
  if (threadIdx.x == 0) s_finite = 0;
  int rank = 0;
  for (int base = 0; base < n; base += 2048) {
    const int m = min(2048, n - base);
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += 256) s_key[k] = desc_key(a.in[base + k].score);
    __syncthreads();
    if (i < n) {
      int r0 = 0, r1 = 0;
      int k = lane4;
      for (; k + 4 < m; k += 8) {
        const unsigned long long k0 = s_key[k], k1 = s_key[k + 4];
        r0 += k0 < key;
        r1 += k1 < key;
        if (k0 == key || k1 == key) {
          for (int q = 0; q < 2; ++q) {
            const int kk = k + 4 * q;
            if (s_key[kk] != key) continue;
            const Cand c = a.in[base + kk];
            if (c.row < me.row || (c.row == me.row && (c.col < me.col || (c.col == me.col && c.angle < me.angle))))
              ++r0;
          }
        }
      }
      for (; k < m; k += 4) {
        const unsigned long long k0 = s_key[k];
        r0 += k0 < key;
        if (k0 == key) {
          const Cand c = a.in[base + k];
          if (c.row < me.row || (c.row == me.row && (c.col < me.col || (c.col == me.col && c.angle < me.angle))))
            ++r0;
        }
      }
      rank += r0 + r1;
    }
  }
  rank += __shfl_xor_sync(0xffffffffu, rank, 1);
  rank += __shfl_xor_sync(0xffffffffu, rank, 2);
  if (i < n && lane4 == 0) {
    a.out[rank] = me;
    if (isfinite(me.score)) atomicAdd(&s_finite, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_finite) atomicAdd(&a.state->sorted_count, s_finite);
}

// Bitonic sort of long candidate lists (more than kRankSortMax): (key,
// index) pairs, padded to the power of two at or above the live count with
// entries that order after every candidate; the comparator is the rank
// sort's order (descending score key, then row, column, angle; the index for
// exact duplicates).  Stages with k up to 2048 and the j < 2048 steps of
// longer stages run in shared memory, one 2048-entry segment per block.
__device__ __forceinline__ bool sort_before(unsigned long long ka, int ia, unsigned long long kb, int ib,
                                            const Cand* __restrict__ in) {
  if (ia == INT32_MAX) return false;
  if (ib == INT32_MAX) return true;
  if (ka != kb) return ka < kb;
  const Cand x = in[ia], y = in[ib];
  if (x.row != y.row) return x.row < y.row;
  if (x.col != y.col) return x.col < y.col;
  if (x.angle != y.angle) return x.angle < y.angle;
  return ia < ib;
}

__device__ __forceinline__ int bitonic_live(const SortArgs& a) {
  const int n = live_count(a.state, a.slot);
  if (n <= kRankSortMax) return 0;
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

__global__ void __launch_bounds__(256) bitonic_init_kernel(SortArgs a) {
  const int np = bitonic_live(a);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= np) return;
  const int n = live_count(a.state, a.slot);
  a.keys[r] = r < n ? desc_key(a.in[r].score) : ~0ULL;
  a.idx[r] = r < n ? r : INT32_MAX;
}

// all steps j <= min(k, 2048) / 2 of the stages k0 .. k1 (k0 <= k1 <= 2048:
// the whole network up to 2048; k0 == k1 > 2048: the shared-memory tail of
// one stage) on this block's 2048-entry segment
__global__ void __launch_bounds__(1024) bitonic_block_kernel(SortArgs a, int k0, int k1) {
  __shared__ unsigned long long s_key[2048];
  __shared__ int s_idx[2048];
  const int np = bitonic_live(a);
  const int base = blockIdx.x * 2048;
  if (base >= np || k0 > np) return;
  const int t = threadIdx.x;
  s_key[t] = a.keys[base + t];
  s_idx[t] = a.idx[base + t];
  s_key[t + 1024] = a.keys[base + t + 1024];
  s_idx[t + 1024] = a.idx[base + t + 1024];
  __syncthreads();
  for (int k = k0; k <= k1; k <<= 1) {
    for (int j = min(k, 2048) >> 1; j > 0; j >>= 1) {
      const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i + j;
      const bool up = ((base + i) & k) == 0;
      const unsigned long long ki = s_key[i], kl = s_key[l];
      const int ii = s_idx[i], il = s_idx[l];
      if (sort_before(kl, il, ki, ii, a.in) == up) {
        s_key[i] = kl;
        s_key[l] = ki;
        s_idx[i] = il;
        s_idx[l] = ii;
      }
      __syncthreads();
    }
  }
  a.keys[base + t] = s_key[t];
  a.idx[base + t] = s_idx[t];
  a.keys[base + t + 1024] = s_key[t + 1024];
  a.idx[base + t + 1024] = s_idx[t + 1024];
}

// one step j >= 2048 of stage k, in global memory
__global__ void __launch_bounds__(256) bitonic_step_kernel(SortArgs a, int k, int j) {
  const int np = bitonic_live(a);
  if (k > np) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (np >> 1)) return;
  const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i + j;
  const bool up = (i & k) == 0;
  const unsigned long long ki = a.keys[i], kl = a.keys[l];
  const int ii = a.idx[i], il = a.idx[l];
  if (sort_before(kl, il, ki, ii, a.in) == up) {
    a.keys[i] = kl;
    a.keys[l] = ki;
    a.idx[i] = il;
    a.idx[l] = ii;
  }
}

__global__ void __launch_bounds__(256) bitonic_gather_kernel(SortArgs a) {
  __shared__ int s_finite;
  const int np = bitonic_live(a);
  if (!np) return;
  const int n = live_count(a.state, a.slot);
  if (threadIdx.x == 0) s_finite = 0;
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) {
    const Cand c = a.in[a.idx[r]];
    a.out[r] = c;
    if (isfinite(c.score)) atomicAdd(&s_finite, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_finite) atomicAdd(&a.state->sorted_count, s_finite);
}

// ----------------------------------------------------------------- overlap
// Rotated rectangle of a pose: FP64 cos/sin once per pose, a conservative
// FP32 box for the cheap disjointness test.
__device__ RectAux make_rect(const Cand& m, const RectGeom& g) {
  RectAux r;
  sincos(m.angle, &r.sa, &r.ca);
  float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
  const double xs[2] = {g.left, g.right}, ys[2] = {g.top, g.bottom};
  for (double x : xs)
    for (double y : ys) {
      const float px = float(m.col) + float(r.ca) * float(x) + float(r.sa) * float(y);
      const float py = float(m.row) - float(r.sa) * float(x) + float(r.ca) * float(y);
      x0 = fminf(x0, px);
      x1 = fmaxf(x1, px);
      y0 = fminf(y0, py);
      y1 = fmaxf(y1, py);
    }
  const float pad = 1e-3f * (1.f + fabsf(float(m.row)) + fabsf(float(m.col)));
  r.x0 = x0 - pad;
  r.y0 = y0 - pad;
  r.x1 = x1 + pad;
  r.y1 = y1 + pad;
  return r;
}

__device__ __forceinline__ bool boxes_disjoint(const RectAux& a, const RectAux& b) {
  return a.x1 < b.x0 || b.x1 < a.x0 || a.y1 < b.y0 || b.y1 < a.y0;
}

struct Pt {
  double x, y;
};

// Intersection area of two rotated template rectangles over the template
// area (src/ncc_matching/matcher.cpp:252-277); a is the candidate, b the
// accepted match.  Corners are relative to a's centre.
__device__ double overlap_ratio(const Cand& a, const RectAux& ra, const Cand& b, const RectAux& rb, const RectGeom& g) {
  if (boxes_disjoint(ra, rb)) return 0.;
  const Pt in[4] = {{g.left, g.top}, {g.right, g.top}, {g.right, g.bottom}, {g.left, g.bottom}};
  Pt clip[4], poly[16], next[16];
  for (int i = 0; i < 4; ++i) {
    clip[i].x = dadd(dadd(dsub(b.col, a.col), dmul(rb.ca, in[i].x)), dmul(rb.sa, in[i].y));
    clip[i].y = dadd(dsub(dsub(b.row, a.row), dmul(rb.sa, in[i].x)), dmul(rb.ca, in[i].y));
    poly[i].x = dadd(dmul(ra.ca, in[i].x), dmul(ra.sa, in[i].y));
    poly[i].y = dadd(-dmul(ra.sa, in[i].x), dmul(ra.ca, in[i].y));
  }
  int count = 4;
  for (int edge = 0; edge < 4 && count; ++edge) {
    const Pt p = clip[edge], q = clip[(edge + 1) & 3];
    int out = 0;
    for (int i = 0; i < count; ++i) {
      const Pt u = poly[i], v = poly[(i + 1) % count];
      const double du = dsub(dmul(dsub(q.x, p.x), dsub(u.y, p.y)), dmul(dsub(q.y, p.y), dsub(u.x, p.x)));
      const double dv = dsub(dmul(dsub(q.x, p.x), dsub(v.y, p.y)), dmul(dsub(q.y, p.y), dsub(v.x, p.x)));
      if (du >= 0 && out < 16) next[out++] = u;
      if ((du >= 0) != (dv >= 0) && out < 16) {
        const double t = du / dsub(du, dv);
        next[out++] = Pt{dadd(u.x, dmul(t, dsub(v.x, u.x))), dadd(u.y, dmul(t, dsub(v.y, u.y)))};
      }
    }
    for (int i = 0; i < out; ++i) poly[i] = next[i];
    count = out;
  }
  double area = 0;
  for (int i = 0; i < count; ++i)
    area = dadd(area, dsub(dmul(poly[i].x, poly[(i + 1) % count].y), dmul(poly[(i + 1) % count].x, poly[i].y)));
  return fabs(area) * .5 / g.area;
}

// The same clip in FP32 (corners relative to a's centre are small numbers):
// within 1e-3 of the true ratio, used to decide clear cases without FP64.
__device__ float overlap_ratio32(const Cand& a, const RectAux& ra, const Cand& b, const RectAux& rb, const RectGeom& g) {
  if (boxes_disjoint(ra, rb)) return 0.f;
  const float L = float(g.left), R = float(g.right), T = float(g.top), B = float(g.bottom);
  const float inx[4] = {L, R, R, L}, iny[4] = {T, T, B, B};
  const float dx = float(b.col - a.col), dy = float(b.row - a.row);
  const float bca = float(rb.ca), bsa = float(rb.sa), aca = float(ra.ca), asa = float(ra.sa);
  float cx[4], cy[4], px[16], py[16], nx[16], ny[16];
  for (int i = 0; i < 4; ++i) {
    cx[i] = dx + bca * inx[i] + bsa * iny[i];
    cy[i] = dy - bsa * inx[i] + bca * iny[i];
    px[i] = aca * inx[i] + asa * iny[i];
    py[i] = -asa * inx[i] + aca * iny[i];
  }
  int count = 4;
  for (int edge = 0; edge < 4 && count; ++edge) {
    const float p0x = cx[edge], p0y = cy[edge], qx = cx[(edge + 1) & 3], qy = cy[(edge + 1) & 3];
    int out = 0;
    for (int i = 0; i < count; ++i) {
      const int j = (i + 1) % count;
      const float du = (qx - p0x) * (py[i] - p0y) - (qy - p0y) * (px[i] - p0x);
      const float dv = (qx - p0x) * (py[j] - p0y) - (qy - p0y) * (px[j] - p0x);
      if (du >= 0 && out < 16) {
        nx[out] = px[i];
        ny[out++] = py[i];
      }
      if ((du >= 0) != (dv >= 0) && out < 16) {
        const float t = du / (du - dv);
        nx[out] = px[i] + t * (px[j] - px[i]);
        ny[out++] = py[i] + t * (py[j] - py[i]);
      }
    }
    for (int i = 0; i < out; ++i) {
      px[i] = nx[i];
      py[i] = ny[i];
    }
    count = out;
  }
  float area = 0;
  for (int i = 0; i < count; ++i) area += px[i] * py[(i + 1) % count] - px[(i + 1) % count] * py[i];
  return fabsf(area) * .5f / float(g.area);
}

// overlap(a, b) > thr, deciding in FP32 when the FP32 ratio is clearly on
// one side and in FP64 otherwise.
__device__ __forceinline__ bool overlaps(const Cand& a, const RectAux& ra, const Cand& b, const RectAux& rb,
                                         const RectGeom& g, double thr) {
  if (boxes_disjoint(ra, rb)) return 0. > thr;
  const float r32 = overlap_ratio32(a, ra, b, rb, g);
  if (double(r32) > thr + 1e-3) return true;
  if (double(r32) < thr - 1e-3) return false;
  return overlap_ratio(a, ra, b, rb, g) > thr;
}

__global__ void rects_kernel(const Cand* sorted, RectAux* aux, const QueryState* state, RectGeom g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= state->sorted_count) return;
  aux[i] = make_rect(sorted[i], g);
}

// Greedy MaxOverlap selection over the sorted candidates
// (src/ncc_matching/matcher.cpp:1063-1076).  A window of candidates is tested
// against the accepted matches in parallel; the first unsuppressed one is
// then accepted or rejected from its refinement result.  When it has none,
// the kernel queues it and the next unsuppressed, unrefined candidates that
// do not overlap a higher-ranked queued one, and returns with need = 1.
constexpr int kSelectThreads = 1024;

__global__ void __launch_bounds__(kSelectThreads) select_kernel(SelectArgs a) {
  __shared__ int s_next, s_acc, s_first, s_hit;
  __shared__ unsigned char s_sup[kSelectThreads];
  __shared__ int s_batch[64];
  QueryState* st = a.state;
  if (st->done) return;
  const int total = st->sorted_count;
  const double thr = a.max_overlap + 1e-12;
  if (threadIdx.x == 0) {
    s_next = st->next;
    s_acc = st->accepted;
    st->need = 0;
  }
  __syncthreads();
  while (true) {
    const int base = s_next, acc = s_acc;
    if (base >= total || (a.num_matches && acc >= a.num_matches)) break;
    // suppression of the window by the accepted matches; each candidate is
    // tested only against matches accepted since its last test
    const int wcount = min(kSelectThreads, total - base);
    const int t = threadIdx.x;
    bool sup = true;
    if (t < wcount) {
      const int idx = base + t;
      sup = a.sup[idx] != 0;
      const int from = a.tested[idx];
      if (!sup && from < acc) {
        const Cand c = a.sorted[idx];
        const RectAux rc = a.aux[idx];
        for (int j = from; j < acc && !sup; ++j)
          if (overlaps(c, rc, a.accepted[j], a.accepted_aux[j], a.geom, thr)) sup = true;
        a.tested[idx] = acc;
        if (sup) a.sup[idx] = 1;
      }
    }
    s_sup[t] = sup ? 1 : 0;
    if (t == 0) s_first = INT32_MAX;
    __syncthreads();
    if (!sup) atomicMin(&s_first, t);
    __syncthreads();
    const int first = s_first;
    if (first == INT32_MAX) {
      __syncthreads();
      if (threadIdx.x == 0) s_next = base + wcount;
      __syncthreads();
      continue;
    }
    const int i = base + first;
    if (a.refined_flag[i] != 2) {
      // queue i and the next unsuppressed, unrefined candidates of the window
      // that no higher-ranked queued candidate overlaps (speculation only)
      if (threadIdx.x == 0) {
        int nb = 0;
        s_batch[nb++] = i;
        for (int k = first + 1; k < wcount && nb < a.batch_limit && nb < 64; ++k) {
          const int idx = base + k;
          if (s_sup[k] || a.refined_flag[idx] == 2) continue;
          const RectAux rk = a.aux[idx];
          bool dup = false;
          for (int q = 0; q < nb && !dup; ++q) {
            const RectAux rq = a.aux[s_batch[q]];
            // boxes overlapping by more than half of the smaller box
            const float ix = fminf(rk.x1, rq.x1) - fmaxf(rk.x0, rq.x0), iy = fminf(rk.y1, rq.y1) - fmaxf(rk.y0, rq.y0);
            if (ix > 0 && iy > 0) {
              const float ak = (rk.x1 - rk.x0) * (rk.y1 - rk.y0), aq = (rq.x1 - rq.x0) * (rq.y1 - rq.y0);
              if (ix * iy > 0.5f * fminf(ak, aq)) dup = true;
            }
          }
          if (!dup) s_batch[nb++] = idx;
        }
        for (int q = 0; q < nb; ++q) {
          a.batch[q] = s_batch[q];
          a.refined_flag[s_batch[q]] = 1;
        }
        st->batch_count = nb;
        st->need = 1;
        st->next = i;
        st->accepted = acc;
      }
      return;
    }
    const Refined r = a.refined[i];
    const bool keep = r.ok != 0;
    Cand rc;
    rc.row = r.row;
    rc.col = r.col;
    rc.angle = r.angle;
    rc.score = r.score;
    rc.patch = -1;
    rc.pad = 0;
    // re-check against the accepted matches with the refined pose
    if (threadIdx.x == 0) s_hit = 0;
    __syncthreads();
    if (keep)
      for (int j = threadIdx.x; j < acc; j += kSelectThreads)
        if (overlaps(rc, r.rect, a.accepted[j], a.accepted_aux[j], a.geom, thr)) s_hit = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
      if (keep && !s_hit) {
        a.accepted[acc] = rc;
        a.accepted_aux[acc] = r.rect;
        s_acc = acc + 1;
      }
      s_next = i + 1;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    st->next = s_next;
    st->accepted = s_acc;
    // final order: score desc, row, column, angle (src/ncc_matching/matcher.cpp:1072-1075)
    const int n = s_acc;
    for (int x = 1; x < n; ++x) {
      const Cand v = a.accepted[x];
      int y = x - 1;
      while (y >= 0) {
        const Cand u = a.accepted[y];
        const bool after = u.score != v.score ? u.score < v.score
                           : u.row != v.row   ? u.row > v.row
                           : u.col != v.col   ? u.col > v.col
                                              : u.angle > v.angle;
        if (!after) break;
        a.accepted[y + 1] = u;
        --y;
      }
      a.accepted[y + 1] = v;
    }
    st->done = 1;
  }
}

// --------------------------------------------------------------- refinement
// refinement_step of src/ncc_matching/matcher.cpp:170-240 at a level-local
// pose: bilinear samples with the analytic gradient, FP32 per thread, pair
// totals, normal equations in pair arithmetic and the Gauss-Jordan solve in
// FP64 on thread 0.  Afterwards sh.ok / sh.gscore / sh.delta hold the result.
__device__ void gn_pass(const ImageView& img, const OriginalView& orig, double row, double col, double angle,
                        int absolute, int rotate, bool use_minimum, double minimum, PoseShared& sh) {
  if (threadIdx.x == 0) sh.lp = make_local(row, col, angle);
  __syncthreads();
  const LocalPose L = sh.lp;
  const float hmax = float(img.h - 1 - L.R0), wmax = float(img.w - 1 - L.C0);
  const float hmin = float(-L.R0), wmin = float(-L.C0);
  float offset = 0.f;
  {
    const float dr = orig.dr[0], dc = orig.dc[0];
    const float y = L.fr + (L.ca * dr - L.sa * dc), x = L.fc + (L.sa * dr + L.ca * dc);
    if (y >= hmin && x >= wmin && y < hmax && x < wmax) {
      const float fy0 = floorf(y), fx0 = floorf(x);
      const int r = L.R0 + int(fy0), c = L.C0 + int(fx0);
      offset = bilinear_at(img, r, c, y - fy0, x - fx0, r + 1, c + 1);
    }
  }
  // 0 sum q, 1 sum q^2, 2 sum wq, 3..5 gs, 6..8 qg, 9..11 wg, 12..17 gg (00,10,11,20,21,22), 18 out
  float acc[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) acc[k] = 0.f;
  const bool inside = samples_inside(L, orig, hmin, hmax, wmin, wmax);
  const float* base = img.v + (size_t(L.R0) * img.w + L.C0);
  for (int s = threadIdx.x; s < orig.n; s += blockDim.x) {
    const float4 p = __ldg(orig.dcw + s);
    const float dr = p.x, dc = p.y, w = p.z;
    const float y = L.fr + (L.ca * dr - L.sa * dc), x = L.fc + (L.sa * dr + L.ca * dc);
    if (!inside && !(y >= hmin && x >= wmin && y < hmax && x < wmax)) {
      acc[18] = 1.f;
      continue;
    }
    const int iy = __float2int_rd(y), ix = __float2int_rd(x);
    const float fy = y - float(iy), fx = x - float(ix);
    float va, vb, vd, ve;
    if (inside && img.pairs) {
      const uint32_t* pp = img.pairs + (size_t(L.R0) * img.w + L.C0) + (iy * img.w + ix);
      const uint32_t aq = __ldg(pp), bq = __ldg(pp + img.w);
      va = __half2float(__ushort_as_half(aq & 0xffff));
      vb = __half2float(__ushort_as_half(aq >> 16));
      vd = __half2float(__ushort_as_half(bq & 0xffff));
      ve = __half2float(__ushort_as_half(bq >> 16));
    } else {
      const float* v = base + (iy * img.w + ix);
      va = __ldg(v);
      vb = __ldg(v + 1);
      vd = __ldg(v + img.w);
      ve = __ldg(v + img.w + 1);
    }
    const float q = (1 - fy) * ((1 - fx) * va + fx * vb) + fy * ((1 - fx) * vd + fx * ve) - offset;
    const float gy = (1 - fx) * (vd - va) + fx * (ve - vb), gx = (1 - fy) * (vb - va) + fy * (ve - vd);
    const float g2 = gy * (-L.sa * dr - L.ca * dc) + gx * (L.ca * dr - L.sa * dc);
    acc[0] += q;
    acc[1] = fmaf(q, q, acc[1]);
    acc[2] = fmaf(w, q, acc[2]);
    acc[3] += gy;
    acc[4] += gx;
    acc[5] += g2;
    acc[6] = fmaf(q, gy, acc[6]);
    acc[7] = fmaf(q, gx, acc[7]);
    acc[8] = fmaf(q, g2, acc[8]);
    acc[9] = fmaf(w, gy, acc[9]);
    acc[10] = fmaf(w, gx, acc[10]);
    acc[11] = fmaf(w, g2, acc[11]);
    acc[12] = fmaf(gy, gy, acc[12]);
    acc[13] = fmaf(gx, gy, acc[13]);
    acc[14] = fmaf(gx, gx, acc[14]);
    acc[15] = fmaf(g2, gy, acc[15]);
    acc[16] = fmaf(g2, gx, acc[16]);
    acc[17] = fmaf(g2, g2, acc[17]);
  }
  F2 t[19];
  block_total<19>(acc, t, sh.scratch);
  if (threadIdx.x < 32) {
    // totals from lane 0 to the warp; every lane evaluates the scalar terms,
    // lane l < axes*(axes+1) one matrix/rhs entry, lane 0 the elimination
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < 19; ++k) {
      t[k].hi = __shfl_sync(0xffffffffu, t[k].hi, 0);
      t[k].lo = __shfl_sync(0xffffffffu, t[k].lo, 0);
    }
    const F2 n = f2(float(orig.n));
    const F2 sum = t[0], dot = t[2];
    const F2 energy = f2_sub(t[1], f2_div(f2_mul(sum, sum), n));
    const float ef = f2_val(energy);
    const bool scored = !(t[18].hi > 0) && ef > 0;
    const float sign = absolute && f2_val(dot) < 0 ? -1.f : 1.f;
    const float sq = scored ? sqrtf(ef) : 1.f;
    const float score = sign * f2_val(dot) / sq;
    const double gscore = scored ? double(fminf(1.f, fmaxf(-1.f, score))) : -INFINITY;
    const bool solve = scored && !(use_minimum && gscore <= minimum);
    const int axes = rotate ? 3 : 2;
    double entry = 0;
    if (solve && lane < axes * (axes + 1)) {
      const int i = lane / (axes + 1), j = lane % (axes + 1);
      const F2 gs[3] = {t[3], t[4], t[5]}, wg[3] = {t[9], t[10], t[11]};
      const F2 gg[3][3] = {{t[12], t[13], t[15]}, {t[13], t[14], t[16]}, {t[15], t[16], t[17]}};
      const F2 sn = f2_div(sum, n);
      const F2 inv_e = f2_div(f2(1.f), energy);
      const F2 qi = f2_sub(t[6 + i], f2_mul(sn, gs[i]));
      if (j < axes) {
        const F2 qj = f2_sub(t[6 + j], f2_mul(sn, gs[j]));
        const F2 e = f2_sub(f2_sub(gg[i][j], f2_div(f2_mul(gs[i], gs[j]), n)), f2_mul(f2_mul(qi, qj), inv_e));
        entry = f2_dbl(f2_mul(e, inv_e));
      } else {
        entry = f2_dbl(f2_sub(f2_mul(f2(sign / sq), wg[i]), f2_mul(f2_mul(f2(score), qi), inv_e)));
      }
    }
    double m[3][4];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) m[i][j] = 0;
    for (int l = 0; l < axes * (axes + 1); ++l) {
      const double v = __shfl_sync(0xffffffffu, entry, l);
      m[l / (axes + 1)][l % (axes + 1)] = v;
    }
    if (lane == 0) {
      sh.ok = 0;
      sh.gscore = gscore;
      sh.delta[0] = sh.delta[1] = sh.delta[2] = 0;
      if (solve) {
        bool good = true;
        for (int i = 0; i < axes && good; ++i) {
          int pivot = i;
          for (int j = i + 1; j < axes; ++j)
            if (fabs(m[j][i]) > fabs(m[pivot][i])) pivot = j;
          if (fabs(m[pivot][i]) < 1e-14) {
            good = false;
            break;
          }
          for (int k = i; k <= axes; ++k) {
            const double tmp = m[i][k];
            m[i][k] = m[pivot][k];
            m[pivot][k] = tmp;
          }
          const double inv = 1.0 / m[i][i];
          for (int k = i; k <= axes; ++k) m[i][k] *= inv;
          for (int j = 0; j < axes; ++j)
            if (j != i) {
              const double f = m[j][i];
              for (int k = i; k <= axes; ++k) m[j][k] -= f * m[i][k];
            }
        }
        if (good) {
          for (int i = 0; i < axes; ++i) sh.delta[i] = m[i][axes];
          if (!rotate) sh.delta[2] = 0;
          sh.ok = isfinite(sh.delta[0]) && isfinite(sh.delta[1]) && isfinite(sh.delta[2]);
        }
      }
    }
  }
  __syncthreads();
}


// Per-block fit state; scalar decisions are made by thread 0 and read by all
// threads after a barrier.
struct FitShared {
  PoseShared ps;
  Cand c, imp, best, seed;
  double next_delta[3], delta[3], factor;
  int cached, accepted, next_valid, flag;
  float wbest[32];
  int word[32];
};

__device__ __forceinline__ double local_row(const RefineArgs& a, double row) { return (row - a.crop_row - a.phase) / a.scale; }
__device__ __forceinline__ double local_col(const RefineArgs& a, double col) { return (col - a.crop_col - a.phase) / a.scale; }

__device__ void score_pose(const RefineArgs& a, FitShared& f, const Cand& p) {
  continuous_pass(a.img, a.orig, local_row(a, p.row), local_col(a, p.col), p.angle, a.absolute, f.ps);
}

__device__ __forceinline__ double step_factor(const double d[3], int rotate, double angle_step) {
  double fct = fmin(1., fmin(.75 / fmax(1e-20, fabs(d[0])), .75 / fmax(1e-20, fabs(d[1]))));
  if (rotate) fct = fmin(fct, angle_step / fmax(1e-20, fabs(d[2])));
  return fct;
}

// fit() of src/ncc_matching/matcher.cpp:903-982 for the candidate in f.c
// (single-model query: no memo, no background guard).
__device__ void fit_full(const RefineArgs& a, FitShared& f) {
  if (!a.subpixel) return;
  if (threadIdx.x == 0) f.cached = 0;
  __syncthreads();
  for (int it = 0; it < 6; ++it) {
    if (!f.cached) {
      gn_pass(a.img, a.orig, local_row(a, f.c.row), local_col(a, f.c.col), f.c.angle, a.absolute, a.rotate, false, 0.,
              f.ps);
      if (!f.ps.ok) break;
      if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) f.delta[k] = f.ps.delta[k];
    } else if (threadIdx.x == 0) {
      for (int k = 0; k < 3; ++k) f.delta[k] = f.next_delta[k];
    }
    if (threadIdx.x == 0) {
      f.cached = 0;
      f.factor = step_factor(f.delta, a.rotate, a.angle_step);
      f.accepted = 0;
    }
    __syncthreads();
    for (int bt = 0; bt < 4; ++bt) {
      if (threadIdx.x == 0) {
        const double st = ldexp(f.factor, -bt);
        Cand imp = f.c;
        imp.row = dadd(imp.row, dmul(st, f.delta[0]));
        imp.col = dadd(imp.col, dmul(st, f.delta[1]));
        imp.angle = fmin(fmax(dadd(imp.angle, dmul(st, f.delta[2])), a.angle_start), a.angle_end);
        f.imp = imp;
        f.flag = domain_contains(a.dom, imp.row, imp.col);
        f.next_valid = 0;
      }
      __syncthreads();
      if (!f.flag) continue;
      if (bt == 0 && it + 1 < 6) {
        gn_pass(a.img, a.orig, local_row(a, f.imp.row), local_col(a, f.imp.col), f.imp.angle, a.absolute, a.rotate,
                true, f.c.score, f.ps);
        if (threadIdx.x == 0) {
          f.imp.score = f.ps.gscore;
          f.next_valid = f.ps.ok;
          for (int k = 0; k < 3; ++k) f.next_delta[k] = f.ps.delta[k];
        }
        __syncthreads();
        if (!isfinite(f.imp.score)) {
          score_pose(a, f, f.imp);
          if (threadIdx.x == 0) f.imp.score = f.ps.score;
        }
      } else {
        score_pose(a, f, f.imp);
        if (threadIdx.x == 0) f.imp.score = f.ps.score;
      }
      __syncthreads();
      if (threadIdx.x == 0 && f.imp.score > f.c.score) {
        f.c = f.imp;
        f.accepted = 1;
        f.cached = f.next_valid;
      }
      __syncthreads();
      if (f.accepted) break;
    }
    if (threadIdx.x == 0)
      f.flag = !f.accepted || (hypot(f.delta[0], f.delta[1]) < 1e-4 && fabs(f.delta[2]) < 1e-5);
    __syncthreads();
    if (f.flag) break;
  }
  __syncthreads();
}

// refine_coarse_candidate of src/ncc_matching/matcher.cpp:853-877
__device__ void fit_coarse(const RefineArgs& a, FitShared& f) {
  if (!a.subpixel) return;
  for (int it = 0; it < 6; ++it) {
    gn_pass(a.img, a.orig, local_row(a, f.c.row), local_col(a, f.c.col), f.c.angle, a.absolute, a.rotate, false, 0.,
            f.ps);
    if (!f.ps.ok) break;
    if (threadIdx.x == 0) {
      for (int k = 0; k < 3; ++k) f.delta[k] = f.ps.delta[k];
      f.factor = step_factor(f.delta, a.rotate, a.angle_step);
      f.accepted = 0;
    }
    __syncthreads();
    for (int bt = 0; bt < 4; ++bt) {
      if (threadIdx.x == 0) {
        const double st = ldexp(f.factor, -bt);
        Cand nx = f.c;
        nx.row = dadd(nx.row, dmul(dmul(a.scale, st), f.delta[0]));
        nx.col = dadd(nx.col, dmul(dmul(a.scale, st), f.delta[1]));
        nx.angle = fmin(fmax(dadd(nx.angle, dmul(st, f.delta[2])), a.angle_start), a.angle_end);
        f.imp = nx;
        f.flag = domain_contains(a.dom, nx.row, nx.col);
      }
      __syncthreads();
      if (!f.flag) continue;
      score_pose(a, f, f.imp);
      if (threadIdx.x == 0) {
        f.imp.score = f.ps.score;
        if (f.imp.score > f.c.score) {
          f.c = f.imp;
          f.accepted = 1;
        }
      }
      __syncthreads();
      if (f.accepted) break;
    }
    if (!f.accepted) break;
  }
  __syncthreads();
}

// Discrete level-0 search around the seed (matcher.cpp:986-1059): one warp per
// (patch, position), exact integer moments in the loop.  Leaves the first
// strict maximum over (patch order, dr, dc) in f.best (score -inf if none).
__device__ void recovery_search(const RefineArgs& a, FitShared& f) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const Cand seed = f.seed;
  float best = -INFINITY;
  int border = INT32_MAX;
  int k = 0;
  for (int j = 0; j < a.nplist0; ++j) {
    const PatchDesc pd = a.view0.patches[a.plist0[j]];
    if (fabs(pd.angle - seed.angle) > a.angle_step * 1.01) continue;
    const PosRange rg = a.ranges0[j];
    const int r0 = int(round(seed.row - a.crop_row - pd.orow)), c0 = int(round(seed.col - a.crop_col - pd.ocol));
    for (int pos = warp; pos < 25; pos += nw) {
      const int r = r0 + pos / 5 - 2, c = c0 + pos % 5 - 2;
      if (r < rg.r0 || r >= rg.r1 || c < rg.c0 || c >= rg.c1) continue;
      if (a.dom.mask && !domain_contains(a.dom, double((long long)a.crop_row + r) + pd.orow,
                                         double((long long)a.crop_col + c) + pd.ocol))
        continue;
      const int2* sw = a.view0.sw + pd.sample_off;
      const float* base = a.lev0.v + size_t(r) * a.lev0.w + c;
      const int2 f0 = __ldg(sw);
      const float s0 = base[off_row(f0.x) * a.lev0.w + off_col(f0.x)];
      float dot = 0.f;
      long long s1 = 0, s2 = 0;
      for (int s = lane; s < pd.n; s += 32) {
        const int2 o = __ldg(sw + s);
        const float x = base[off_row(o.x) * a.lev0.w + off_col(o.x)] - s0;
        dot = fmaf(__int_as_float(o.y), x, dot);
        const long long xi = (long long)x;
        s1 += xi;
        s2 += xi * xi;
      }
      for (int o = 16; o > 0; o >>= 1) {
        dot += __shfl_down_sync(0xffffffffu, dot, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
      }
      if (lane == 0) {
        const float sc = window_score(dot, s1, s2, pd.n, a.absolute);
        const int order = k * 25 + pos;
        if (better(sc, order, best, border)) {
          best = sc;
          border = order;
        }
      }
    }
    ++k;
  }
  if (lane == 0) {
    f.wbest[warp] = best;
    f.word[warp] = border;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float bs = -INFINITY;
    int bo = INT32_MAX;
    for (int w = 0; w < nw; ++w)
      if (better(f.wbest[w], f.word[w], bs, bo)) {
        bs = f.wbest[w];
        bo = f.word[w];
      }
    Cand out = seed;
    out.score = -INFINITY;
    if (bo != INT32_MAX && bs > -INFINITY) {
      int kk = 0;
      for (int j = 0; j < a.nplist0; ++j) {
        const PatchDesc pd = a.view0.patches[a.plist0[j]];
        if (fabs(pd.angle - seed.angle) > a.angle_step * 1.01) continue;
        if (kk == bo / 25) {
          const int r0 = int(round(seed.row - a.crop_row - pd.orow)), c0 = int(round(seed.col - a.crop_col - pd.ocol));
          out.row = double((long long)a.crop_row + r0 + (bo % 25) / 5 - 2) + pd.orow;
          out.col = double((long long)a.crop_col + c0 + (bo % 25) % 5 - 2) + pd.ocol;
          out.angle = pd.angle;
          out.score = double(bs);
          break;
        }
        ++kk;
      }
    }
    f.best = out;
  }
  __syncthreads();
}

constexpr int kRefineThreads = 512;

// refine_candidate (src/ncc_matching/matcher.cpp:878-1061) for one queued
// candidate per block.
__global__ void __launch_bounds__(kRefineThreads) refine_kernel(RefineArgs a) {
  __shared__ FitShared f;
  const int b = blockIdx.x;
  // a queued round after the end of the selection has nothing to refine
  if (a.batch_count < 0 && a.state->done) return;
  if (b >= (a.batch_count >= 0 ? a.batch_count : a.state->batch_count)) return;
  const int i = a.batch[b];
  if (threadIdx.x == 0) {
    f.c = a.sorted[i];
    f.seed = f.c;
  }
  __syncthreads();
  if (a.finest) {
    fit_coarse(a, f);
  } else {
    fit_full(a, f);
    if (a.subpixel && a.top > 0 && f.c.score < a.min_score) {
      recovery_search(a, f);
      // the search starts from the fitted candidate: only a strictly higher
      // discrete score moves it
      if (threadIdx.x == 0) {
        if (!(f.best.score > f.c.score)) f.best = f.c;
        f.flag = f.best.row != f.c.row || f.best.col != f.c.col || f.best.angle != f.c.angle;
      }
      __syncthreads();
      if (f.flag) {
        score_pose(a, f, f.best);
        if (threadIdx.x == 0) {
          f.best.score = f.ps.score;
          f.seed = f.c;  // keep the fitted candidate
          f.c = f.best;
        }
        __syncthreads();
        fit_full(a, f);
        if (threadIdx.x == 0 && !(f.c.score > f.seed.score)) f.c = f.seed;
        __syncthreads();
      }
    }
  }
  if (threadIdx.x == 0) {
    Refined r;
    r.row = f.c.row;
    r.col = f.c.col;
    r.angle = f.c.angle;
    r.score = f.c.score;
    r.ok = (f.c.score >= a.min_score) && domain_contains(a.dom, f.c.row, f.c.col);
    r.pad = 0;
    r.rect = make_rect(f.c, a.geom);
    a.refined[i] = r;
    __threadfence();
    a.refined_flag[i] = 2;
  }
}

}  // namespace

// 2-D prefix counts of a domain mask, (h + 1) x (w + 1): row prefixes (one
// thread per row), then column sums (one thread per column, coalesced).
__global__ void domain_rows_kernel(const uint8_t* mask, int w, int h, int32_t* count) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t pitch = size_t(w) + 1;
  if (y == 0)
    for (int x = 0; x <= w; ++x) count[x] = 0;
  if (y >= h) return;
  int32_t sum = 0;
  int32_t* out = count + size_t(y + 1) * pitch;
  out[0] = 0;
  const uint8_t* row = mask + size_t(y) * w;
  for (int x = 0; x < w; ++x) {
    sum += row[x] != 0;
    out[x + 1] = sum;
  }
}

__global__ void domain_cols_kernel(int w, int h, int32_t* count) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x > w) return;
  const size_t pitch = size_t(w) + 1;
  int32_t sum = 0;
  for (int y = 1; y <= h; ++y) {
    sum += count[size_t(y) * pitch + x];
    count[size_t(y) * pitch + x] = sum;
  }
}

// --------------------------------------------------------------- launchers
cudaError_t launch_domain_count(const uint8_t* mask, int w, int h, int32_t* count, cudaStream_t s) {
  domain_rows_kernel<<<(h + 127) / 128, 128, 0, s>>>(mask, w, h, count);
  domain_cols_kernel<<<(w + 1 + 255) / 256, 256, 0, s>>>(w, h, count);
  return cudaGetLastError();
}

cudaError_t reserve_dynamic_smem(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> granted;
  int dev = 0;
  if (const cudaError_t e = cudaGetDevice(&dev)) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = granted[{kernel, dev}];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess) cur = bytes;
  return e;
}

cudaError_t launch_pyramid0(const void* src, int type, int64_t pitch_elems, int crop_row, int crop_col, LevelImage dst,
                            int32_t* error_flag, cudaStream_t s, uint32_t* pairs) {
  (void)error_flag;
  const dim3 block(32, 8), grid((dst.w + 31) / 32, (dst.h + 7) / 8);
  if (type == 1)
    pyramid0_kernel<uint16_t><<<grid, block, 0, s>>>(static_cast<const uint16_t*>(src), pitch_elems, crop_row, crop_col,
                                                     dst, pairs);
  else
    pyramid0_kernel<uint8_t><<<grid, block, 0, s>>>(static_cast<const uint8_t*>(src), pitch_elems, crop_row, crop_col,
                                                    dst, pairs);
  return cudaGetLastError();
}

cudaError_t launch_pyramid(const LevelImage& src, LevelImage dst, int32_t* error_flag, cudaStream_t s) {
  const dim3 block(32, 8), grid((dst.w + 31) / 32, (dst.h + 7) / 8);
  pyramid_kernel<<<grid, block, 0, s>>>(src, dst, error_flag);
  return cudaGetLastError();
}

cudaError_t launch_prefix(const LevelImage& lev, cudaStream_t s) {
  const int warps = lev.h, threads = 256;
  const int blocks = (warps * 32 + threads - 1) / threads;
  prefix_kernel<<<blocks, threads, 0, s>>>(lev);
  return cudaGetLastError();
}

cudaError_t launch_coarse(const CoarseArgs& a, int max_bh, int max_bw, cudaStream_t s, size_t smem_limit) {
  const size_t smem = size_t(kTileH + max_bh) * size_t(kTileW + max_bw) * sizeof(float);
  if (smem > smem_limit) return cudaErrorInvalidConfiguration;
  if (const cudaError_t e = reserve_dynamic_smem(reinterpret_cast<const void*>(coarse_kernel), smem)) return e;
  const dim3 block(kTileW, kTileH), grid((a.lev.w + kTileW - 1) / kTileW, (a.lev.h + kTileH - 1) / kTileH, a.nplist);
  coarse_kernel<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_nms(const NmsArgs& a, cudaStream_t s) {
  const int64_t n = int64_t(a.w) * a.h * a.nplist;
  nms_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_track(const TrackArgs& a, int max_candidates, cudaStream_t s, size_t smem_limit) {
  TrackArgs b = a;
  size_t smem = size_t(a.view.lin_pitch) * size_t(a.view.lin_rows) * sizeof(float);
  const size_t fixed = 8 * 1024;  // static shared memory of the kernel
  const size_t scratch = a.tc_dots ? 2 * kTrackThreads * sizeof(long long) : 0;
  if (smem + scratch + fixed > smem_limit || smem > 160 * 1024) {
    b.staged_ok = 0;
    smem = 0;
  } else {
    b.staged_ok = 1;
  }
  // tensor-core items leave the sample slices idle: they split the runs
  // instead, through a scratch after the window
  if (scratch) {
    smem = (smem + 15) & ~size_t(15);  // 8-byte entries: start on a 16-byte boundary
    b.split_off = int(smem / sizeof(float));
    smem += scratch;
  } else {
    b.split_off = -1;
  }
  if (const cudaError_t e = reserve_dynamic_smem(reinterpret_cast<const void*>(track_kernel), smem)) return e;
  track_kernel<<<max_candidates, kTrackThreads, smem, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_dedup(const DedupArgs& a, int max_candidates, cudaStream_t s) {
  const unsigned blocks = unsigned((max_candidates + 255) / 256);
  if (a.snap)
    snap_kernel<<<blocks, 256, 0, s>>>(const_cast<Cand*>(a.in), a.state, a.in_slot, a.height, a.width, a.dom);
  dedup_kernel<<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const AdjointArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  adjoint_kernel<<<a.n, kAdjointThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_refine4(const Refine4Args& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  refine4_kernel<<<a.n, kRefine4Threads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_score(const ScoreArgs& a, int max_candidates, cudaStream_t s) {
  score_kernel<<<max_candidates, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_coarse_lattice(Cand* cand, int2* rc, int nsrc, int nbr, int nbc, const int32_t* group_of_src,
                                  int32_t* order, TcTiles* tiles, QueryState* state, int slot, cudaStream_t s) {
  const int n = std::max(1, nsrc * nbr * nbc);
  coarse_lattice_kernel<<<(n + 255) / 256, 256, 0, s>>>(cand, rc, nsrc, nbr, nbc, group_of_src, order, tiles, state,
                                                        slot);
  return cudaGetLastError();
}

cudaError_t launch_coarse_tc_score(const CoarseTcArgs& a, cudaStream_t s) {
  const long long n = (long long)a.nplist * a.lev.h * a.lev.w;
  coarse_tc_score_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pairs(const float* v, int w, int h, uint32_t* pairs, cudaStream_t s) {
  const long long n = (long long)w * h;
  pairs_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(v, w, h, pairs);
  return cudaGetLastError();
}

cudaError_t launch_sort(const SortArgs& a, int max_candidates, cudaStream_t s) {
  sort_kernel<<<(max_candidates + kSortPer - 1) / kSortPer, 256, 0, s>>>(a);
  if (a.keys) {
    // every launch reads the live count and returns when it has no work
    if (a.npow < max_candidates || a.npow < 4096 || (a.npow & (a.npow - 1))) return cudaErrorInvalidValue;
    const unsigned segs = unsigned(a.npow / 2048), pairs = unsigned(a.npow / 2 / 256);
    bitonic_init_kernel<<<unsigned(a.npow / 256), 256, 0, s>>>(a);
    bitonic_block_kernel<<<segs, 1024, 0, s>>>(a, 2, 2048);
    for (int k = 4096; k <= a.npow; k <<= 1) {
      for (int j = k >> 1; j >= 2048; j >>= 1) bitonic_step_kernel<<<pairs, 256, 0, s>>>(a, k, j);
      bitonic_block_kernel<<<segs, 1024, 0, s>>>(a, k, k);
    }
    bitonic_gather_kernel<<<unsigned((max_candidates + 255) / 256), 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_rects(const Cand* sorted, RectAux* aux, const QueryState* state, RectGeom g, int max_candidates,
                         cudaStream_t s) {
  rects_kernel<<<unsigned((max_candidates + 255) / 256), 256, 0, s>>>(sorted, aux, state, g);
  return cudaGetLastError();
}

cudaError_t launch_select(const SelectArgs& a, cudaStream_t s) {
  select_kernel<<<1, kSelectThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_refine(const RefineArgs& a, int batch_limit, cudaStream_t s) {
  refine_kernel<<<batch_limit, kRefineThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mvg
