// Tensor-core (tcgen05) correlation for the coarse-to-fine tracking step.
//
// The candidates of one tracking step are grouped by the patch they were
// found with: all candidates of a group search the same target patches (the
// reference's angle window, src/ncc_matching/matcher.cpp:680-697), so the
// group shares one weight matrix per grid row.  A tile is up to 16
// candidates of a group and one MMA computes, for a chunk of rg grid rows
// y .. y + rg - 1 of the patches' union grid (k < rg),
//
//   D[(candidate g, row m)][(patch p, column placement dc, k, half)]
//     += sum_x window_g(y + m, x) * w_{p,half}(y + k, x - dc)
//
// Window row y + m is placement m at grid row y and placement m - k at grid
// row y + k, so the dot product of placement dr is the sum over k of
// D_k[(g, dr + k)] (dr + k <= 7 for dr < 5, rg <= 4).  One window tile thus
// serves rg grid rows: the MMAs are bound by fetching that tile, so rg
// divides their count.  M = 16 x 8 rows, N = 10 P rg, K = the window columns
// plus one 16-column step that subtracts the candidate's centre value times
// the row sum of each weight column (centred accumulation, as the CUDA-core
// path's window centring).  Chunks accumulate round-robin into up to four
// accumulator sets in tensor memory, summed in FP32 by the epilogue.
// Windows come straight from fp16 copies of the level ("planes", exact
// integers: the level minus an offset, as one to four base-64 digit planes
// when a level's values exceed fp16's integer range), one bulk copy (TMA
// engine) per candidate and 8-column segment, into the canonical
// no-swizzle K-major layout whose row pitch is 16 bytes, so grid row y is
// the same tiles started y rows later.  The planes are column-blocked (the
// rows of an 8-column block contiguous), eight column-shifted copies keep
// every segment on a 16-byte boundary, and planes start 8 columns left of
// the level.  Weights (fp16 high and low
// halves of the scaled weights) stream through a ring of shared-memory
// buffers with bulk copies (TMA engine).  The block is warp-specialised:
// four window-producer warps (two slab buffers), a weight-producer
// thread, an MMA-issue thread and four epilogue warps that also set up the
// tiles, with two tiles in flight; accumulation is FP32 in tensor memory.  The epilogue
// writes sum w (S - S0) per placement; track_kernel adds the exact integer
// window moments and applies the reference's selection rule.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ncc_kernels.h"

namespace mvg {
namespace {

constexpr int kTcThreads = 320;  // warp 0 MMA, warp 1 weights, warps 2-5 windows, warps 6-9 epilogue and set-up
constexpr int kTcWindowThreads = 128;
constexpr int kTcEpilogueThreads = 128;
constexpr int kTcRows = 128;                  // MMA M
constexpr uint32_t kTmemCols = 512 / kTcBlocksPerSm;  // two accumulator regions
constexpr uint32_t kTcRegionCols = kTmemCols / 2;      // accumulator sets x columns per set, per region
constexpr unsigned long long kWaitNs = 1000000000ull;  // an mbarrier wait gives up after one second

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// shared-memory matrix descriptor: canonical layout without swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = uint64_t((addr & 0x3FFFF) >> 4);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count = 1) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// raises the current phase's expected transaction bytes without arriving
__device__ __forceinline__ void expect_tx_only(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bounded wait for the completion of the phase with parity `parity`
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase with the given parity; false once kWaitNs passed
// without it, or (given `fail`) once another role of the block has failed
// (the caller records the failure and leaves).
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, const int* fail = nullptr) {
  unsigned long long start = 0;
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (fail && *reinterpret_cast<const volatile int*>(fail)) return false;
    const unsigned long long now = global_ns();
    if (!start)
      start = now;
    else if (now - start > kWaitNs)
      return false;
  }
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// One tile in flight: its set-up, written by the epilogue warps and shared
// with the other roles (info_full hands it over; info_empty, arrived by the
// MMA thread, the weight producer and the window warps, hands the slot back).
struct __align__(16) TcSlot {
  TcArgs job;    // the tile's job (job tables only)
  TcGroup grp;
  int gtile;     // launch tile; -1: the block has no more tiles
  int cnt;       // candidates of the tile
  int ci[kTcCands], R[kTcCands], x0a[kTcCands], delta[kTcCands];
  float centre[kTcCands];  // window centre value minus the plane offset (exact integer)
  uint4 cwords[kTcCands];  // its centring words: (-c_q, -c_q) half2 per digit q, then zeros
};

struct __align__(16) TcShared {
  uint64_t a_full[2], slab_done[2], drain;
  uint64_t b_full[kTcMaxStages], b_empty[kTcMaxStages];
  uint64_t info_full[2], info_empty[2];  // tile slots
  uint64_t acc_full[2], acc_empty[2];    // accumulator regions in tensor memory (tile s: region s mod 2)
  TcSlot slot[2];
  int job_base[kTcMaxJobs + 1];  // first launch tile of each job
  uint32_t tmem;
  int fail;
  int claim;         // the epilogue warps' next tile (broadcast)
  long long cm, cb;  // weight chunks consumed (MMA thread) / loaded (weight producer), at exit
};

// Shape of one tile's operands.
struct TcShape {
  int segs, nplane, nseg, K, ksteps, Y, nslabs, chunks;
  uint32_t lbo, sbo, bchunk;
  __device__ explicit TcShape(const TcGroup& G) {
    segs = G.kw / 8;
    nplane = G.parts * segs;  // plane segments; two centring segments follow
    nseg = nplane + 2;
    K = 8 * nseg;
    ksteps = K / 16;
    Y = (G.rows_slab - 7) / G.rg * G.rg;  // grid rows per window slab (whole chunks)
    nslabs = (G.kr + Y - 1) / Y;
    chunks = (G.kr + G.rg - 1) / G.rg;
    lbo = uint32_t(G.rows_slab) * 16;
    sbo = uint32_t(nseg) * lbo;
    bchunk = uint32_t(G.n) * uint32_t(K) * 2;
  }
};

// A role gave up (a wait ran out, or another role failed): the others leave
// at their next wait; the launch's jobs get the error flag at the end.
__device__ __forceinline__ void tc_fail(TcShared& sh) { atomicExch(&sh.fail, 1); }

// Named barriers of one role's warps (warp-divergent forms).  The AND form
// gives every thread the same verdict, so a group leaves its loop together.
__device__ __forceinline__ void named_sync(int id, int threads) {
  asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
__device__ __forceinline__ bool named_and(int id, int threads, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n barrier.red.and.pred po, %2, %3, pi;\n"
      " selp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"(uint32_t(v)), "r"(id), "r"(threads)
      : "memory");
  return r != 0;
}

// Position in the weight ring: buffer index and phase parity of chunk count,
// advanced incrementally (no division on the issue path).
struct RingPos {
  long long count = 0;
  int stage = 0;
  uint32_t phase = 0;
  __device__ void advance(int stages) {
    ++count;
    if (++stage == stages) {
      stage = 0;
      phase ^= 1u;
    }
  }
};

// MMA issue (one thread), one tile: per slab, wait for the windows, then per
// grid row wait for its weights, issue K/16 MMAs into accumulator set
// y mod sets and release the weight buffer; release the window buffer after
// the slab, and the accumulators to the epilogue after the tile.
__device__ bool tc_mma_tile(const TcArgs& a, const TcSlot& ts, TcShared& sh, uint8_t* wbase, uint8_t* abase,
                            uint32_t tmem, uint64_t* acc_full, RingPos& cm, int& sm) {
  const TcGroup& G = ts.grp;
  const TcShape sp(G);
  const int S = a.stages;
  const uint32_t idesc = (1u << 4) | (uint32_t(G.n >> 3) << 17) | (uint32_t(kTcRows >> 4) << 24);
  for (int sl = 0; sl < sp.nslabs; ++sl) {
    const int buf = sm & 1;
    if (!bar_wait(&sh.a_full[buf], uint32_t((sm >> 1) & 1), &sh.fail)) return false;
    // descriptors advance by plain adds of the 16-byte address units: one row
    // per grid row, two segments (2 lbo) per K step; weights 256 bytes per K step
    const uint64_t a_desc0 = smem_desc(smem_u32(abase + size_t(buf) * a.abuf_bytes), sp.lbo, sp.sbo);
    const uint64_t a_kstep = uint64_t(2 * sp.lbo) >> 4;
    const uint64_t b_desc0 = smem_desc(smem_u32(wbase), 128, uint32_t(sp.K / 8) * 128);
    const uint64_t b_stage = uint64_t(a.stage_bytes) >> 4;
    const int y0 = sl * sp.Y, y1 = min(G.kr, y0 + sp.Y);
    int chunk = y0 / G.rg;
    uint32_t d = tmem + uint32_t((chunk % a.sets) * a.npad);
    const uint32_t d_end = tmem + uint32_t(a.sets * a.npad);
    for (int y = y0; y < y1; y += G.rg, ++chunk) {
      if (!bar_wait(&sh.b_full[cm.stage], cm.phase, &sh.fail)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint64_t ad = a_desc0 + uint64_t(y - y0), bd = b_desc0 + uint64_t(cm.stage) * b_stage;
      mma_f16(d, ad, bd, idesc, chunk >= a.sets ? 1u : 0u);
#pragma unroll 4
      for (int j = 1; j < sp.ksteps; ++j) {
        ad += a_kstep;
        bd += 16;
        mma_f16(d, ad, bd, idesc, 1u);
      }
      mma_commit(&sh.b_empty[cm.stage]);
      cm.advance(S);
      d += uint32_t(a.npad);
      if (d == d_end) d = tmem;
    }
    mma_commit(&sh.slab_done[buf]);
    ++sm;
  }
  mma_commit(acc_full);
  return true;
}

// Window producers (four warps), one tile: per slab, once the MMAs of the
// slab that last used the buffer are done, one bulk copy (TMA engine) per
// (candidate, plane segment) of the slab's rows that lie inside the level:
// the planes are column-blocked, so a segment's rows are contiguous in
// global memory and land as one run of 16-byte rows, the canonical
// no-swizzle layout.  Rows outside the level and segments outside the plane
// are zeroed by plain stores, as are the centring columns of the tile's
// candidates.  Each thread announces its copies' bytes on the buffer's
// barrier, orders its own stores for the tensor cores (proxy fence) and
// arrives (128 arrivals); the phase completes when every byte has landed.
// Rows of candidates beyond the tile's count are left as they are: their
// accumulator rows are never read.
__device__ bool tc_window_tile(const TcArgs& a, const TcSlot& ts, TcShared& sh, uint8_t* abase, int& sa, int pt) {
  const TcGroup& G = ts.grp;
  const TcShape sp(G);
  const int cnt = ts.cnt, rows = G.rows_slab, H = a.lev.h, groups = a.plane_pitch / 8;
  const size_t plane = size_t(H) * size_t(a.plane_pitch);     // elements of one shifted plane
  const size_t part_stride = size_t(kTcPlaneShifts) * plane;  // one part's planes -> the next part's
  const int ncopies = cnt * sp.nplane;
  const int g_first = pt / rows, r_first = pt - g_first * rows;  // first centring row of this thread
  const uint4 zero = make_uint4(0, 0, 0, 0);
  for (int sl = 0; sl < sp.nslabs; ++sl) {
    const int buf = sa & 1;
    if (sa >= 2 && !bar_wait(&sh.slab_done[buf], uint32_t(((sa >> 1) - 1) & 1), &sh.fail)) return false;
    uint8_t* dst0 = abase + size_t(buf) * a.abuf_bytes;
    const int y0 = sl * sp.Y;
    // copy i = (candidate g, segment sg): rows [lo, hi) of the slab lie in the level
    auto piece = [&](int i, int& g, int& sg, int& xb, int& lo, int& hi) {
      g = i / sp.nplane;
      sg = i - g * sp.nplane;
      const int q = sg / sp.segs;  // part of the level value
      xb = (ts.x0a[g] + kTcPlaneMargin) / 8 + (sg - q * sp.segs);
      const int row0 = ts.R[g] - 2 + G.rmin + y0;
      lo = min(rows, max(0, -row0));
      hi = max(lo, min(rows, H - row0));
      if (xb < 0 || xb >= groups) hi = lo;  // outside the plane: all zero
      return q;
    };
    uint32_t bytes = 0;
    for (int i = pt; i < ncopies; i += kTcWindowThreads) {
      int g, sg, xb, lo, hi;
      piece(i, g, sg, xb, lo, hi);
      bytes += uint32_t(hi - lo) * 16u;
    }
    if (bytes) expect_tx_only(&sh.a_full[buf], bytes);
    for (int i = pt; i < ncopies; i += kTcWindowThreads) {
      int g, sg, xb, lo, hi;
      const int q = piece(i, g, sg, xb, lo, hi);
      uint8_t* dst = dst0 + size_t(g) * sp.sbo + size_t(sg) * sp.lbo;
      if (hi > lo) {
        const int row0 = ts.R[g] - 2 + G.rmin + y0;
        const uint16_t* src = a.planes + size_t(q) * part_stride + size_t(ts.delta[g]) * plane +
                              (size_t(xb) * size_t(H) + size_t(row0 + lo)) * 8;
        bulk_load(dst + size_t(lo) * 16, src, uint32_t(hi - lo) * 16u, &sh.a_full[buf]);
      }
      for (int r = 0; r < lo; ++r) *reinterpret_cast<uint4*>(dst + size_t(r) * 16) = zero;
      for (int r = max(hi, lo); r < rows; ++r) *reinterpret_cast<uint4*>(dst + size_t(r) * 16) = zero;
    }
    // centring columns: (candidate g, row r) for g < cnt, 128 rows apart
    for (int g = g_first, r = r_first; g < cnt;) {
      uint8_t* row = dst0 + size_t(g) * sp.sbo + size_t(sp.nplane) * sp.lbo + size_t(r) * 16;
      *reinterpret_cast<uint4*>(row) = ts.cwords[g];
      *reinterpret_cast<uint4*>(row + sp.lbo) = zero;
      r += kTcWindowThreads;
      while (r >= rows) {
        r -= rows;
        ++g;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bar_arrive(&sh.a_full[buf]);
    ++sa;
  }
  return true;
}

// Weight producer (one thread), one tile: its grid-row chunks through the
// ring, as far ahead as the ring allows (into the next tile while the MMAs
// of this one run).
__device__ bool tc_weight_tile(const TcArgs& a, const TcSlot& ts, TcShared& sh, uint8_t* wbase, RingPos& cb) {
  if (a.withhold_weights) return true;  // test hook: the MMA thread's weight wait runs out
  const TcShape sp(ts.grp);
  const int S = a.stages;
  const uint8_t* src = ts.grp.b;
  for (int i = 0; i < sp.chunks; ++i) {
    // the buffer's previous chunk (count - S) has been consumed
    if (cb.count >= S && !bar_wait(&sh.b_empty[cb.stage], cb.phase ^ 1u, &sh.fail)) return false;
    expect_tx(&sh.b_full[cb.stage], sp.bchunk);
    bulk_load(wbase + size_t(cb.stage) * a.stage_bytes, src, sp.bchunk, &sh.b_full[cb.stage]);
    src += sp.bchunk;
    cb.advance(S);
  }
  return true;
}

// Tile set-up (the epilogue warps, 128 threads): the tile's job (job
// tables), group and candidates into the slot, one candidate per thread.
template <bool Multi>
__device__ void tc_setup(const TcArgs* jobs, const TcShared& sh, TcSlot& ts, int gtile, int ntiles, int pt) {
  if (gtile >= ntiles) {
    if (pt == 0) ts.gtile = -1;
    return;
  }
  int jb = 0;
  if (Multi)
    while (gtile >= sh.job_base[jb + 1]) ++jb;
  const TcArgs& a = jobs[jb];
  const int tile = gtile - sh.job_base[jb];
  if (Multi) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&a);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&ts.job);
    for (int w = pt; w < int(sizeof(TcArgs) / 4); w += kTcEpilogueThreads) dst[w] = src[w];
  }
  const int gi = a.tiles->group[tile];
  const TcGroup& gsrc = a.groups[gi];
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&gsrc);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&ts.grp);
    for (int w = pt; w < int(sizeof(TcGroup) / 4); w += kTcEpilogueThreads) dst[w] = src[w];
  }
  const int first = a.tiles->first[tile];
  const int cnt = min(kTcCands, a.tiles->last[tile] - first);
  if (pt == 0) {
    ts.gtile = gtile;
    ts.cnt = cnt;
  }
  if (pt < cnt) {
    const int ci = a.order[first + pt];
    const Cand cd = a.in[ci];
    int R, C;
    if (a.rc) {
      R = a.rc[ci].x;
      C = a.rc[ci].y;
    } else if (a.exact32) {
      const float s = float(1.0 / a.step);
      R = int(roundf(__fmul_rn(__fsub_rn(__fsub_rn(float(cd.row), float(a.crop_row)), float(a.offset)), s)));
      C = int(roundf(__fmul_rn(__fsub_rn(__fsub_rn(float(cd.col), float(a.crop_col)), float(a.offset)), s)));
    } else {
      R = int(round(dsub(dsub(cd.row, a.crop_row), a.offset) / a.step));
      C = int(round(dsub(dsub(cd.col, a.crop_col), a.offset) / a.step));
    }
    ts.ci[pt] = ci;
    ts.R[pt] = R;
    const int cr = min(max(R, 0), a.lev.h - 1), cc = min(max(C, 0), a.lev.w - 1);
    const float centre = a.lev.v[size_t(cr) * a.lev.w + cc] -
                         tc_plane_offset(a.plane_offset, a.dyn_offset ? a.state : nullptr, a.level_mult);
    ts.centre[pt] = centre;
    // the centre split like the planes, c = sum_q c_q 64^(parts - 1 - q),
    // as the pairs (-c_q, -c_q), q = 0 .. parts - 1, then zeros
    const int parts = gsrc.parts;
    uint32_t wd[kTcMaxParts];
    float rem = centre;
#pragma unroll
    for (int q = 0; q < kTcMaxParts; ++q) {
      const int sh6 = 6 * (parts - 1 - q);
      const float unit = sh6 >= 0 ? float(1 << max(sh6, 0)) : 0.f;
      const float dq = q >= parts ? 0.f : q + 1 < parts ? floorf(rem * (1.f / unit)) : rem;
      const __half2 h = __floats2half2_rn(-dq, -dq);
      wd[q] = q < parts ? *reinterpret_cast<const uint32_t*>(&h) : 0u;
      rem -= dq * unit;
    }
    ts.cwords[pt] = make_uint4(wd[0], wd[1], wd[2], wd[3]);
    const int x0 = C - 2 + gsrc.cmin;
    ts.x0a[pt] = x0 & ~7;  // floor to a multiple of 8 (16-byte copy start)
    ts.delta[pt] = x0 - (x0 & ~7);
  }
}

// Epilogue (four warps), one tile: warp w reads tensor-memory lanes
// 32 (w mod 4) .. + 31, accumulator row m = 8 g + r of candidate g.  The
// columns of output u = (patch q, column placement dc) are the rg grid-row
// slots k and two weight halves side by side, (u rg + k) 2 + half, so 32
// columns hold 16 / rg whole outputs.  Per 32 columns the accumulator sets
// are summed (set order), slot k comes from row m + k (a shuffle within the
// candidate's 8 rows), and the dot of placement (dr = r, dc) is
// sum_k (D[m + k][.., half 0] + D[m + k][.., half 1]) in k order.
template <int RG>
__device__ void tc_epilogue(const TcArgs& a, const TcSlot& ts, uint32_t trow, int quarter, int lane) {
  const TcGroup& G = ts.grp;
  constexpr int kPer = 16 / RG;  // outputs per 32 accumulator columns
  const int nout = G.p * 5;
  const int nsets = min(a.sets, (G.kr + RG - 1) / RG);
  const int g = quarter * 4 + (lane >> 3), dr = lane & 7;
  const bool live = g < ts.cnt && dr < 5;
  const float poff = tc_plane_offset(a.plane_offset, a.dyn_offset ? a.state : nullptr, a.level_mult);
  const float cen = live ? ts.centre[g] : 0.f;
  float* out = a.dots + (live ? size_t(ts.ci[g]) * kTcScoreStride + size_t(dr) * 5 : 0);
  for (int u0 = 0; u0 < nout; u0 += kPer) {
    const uint32_t c0 = uint32_t(u0 * RG * 2);  // a multiple of 32
    float x[32];
    tmem_ld32(trow + c0, x);
    for (int set = 1; set < nsets; ++set) {
      float v[32];
      tmem_ld32(trow + uint32_t(set * a.npad) + c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) x[j] += v[j];
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      float sum = 0.f;
#pragma unroll
      for (int k = 0; k < RG; ++k) {
        const float v0 = __shfl_down_sync(0xffffffffu, x[(j * RG + k) * 2], k);
        const float v1 = __shfl_down_sync(0xffffffffu, x[(j * RG + k) * 2 + 1], k);
        sum += v0 + v1;
      }
      const int u = u0 + j;
      if (live && u < nout) {
        const int q = u / 5, dc = u - q * 5;
        // sum w S = sum w (S' - c) + c ecorr + offset weff (S' = S - offset);
        // the consumers subtract S0 weff (first sample S0) themselves
        out[G.k_of[q] * 25 + dc] = sum * G.inv_scale + (cen * G.ecorr[q] + poff * G.weff[q]);
      }
    }
  }
}

// Persistent and warp-specialised, tiles pipelined: the launch's tiles are
// those of its jobs in job order; block b takes tile b first, then the next
// unclaimed tile from a global counter (tiles differ in cost, so a static
// stride leaves blocks idle at the end).  Warp 0 issues the MMAs, warp 1
// streams weights, warps 2-5 stage windows, warps 6-9 run the epilogue and
// set up the tiles (tile s + 2 after the epilogue of tile s, in the slot it
// frees).  Two tile slots let the set-up, windows and weights of the
// next tile go ahead while the MMAs of this one run, and two accumulator
// regions in tensor memory (tile s in region s mod 2) let the next tile's
// MMAs run while the epilogue reads this one.  Shared memory:
// weight ring (stages x stage_bytes) | two window buffers, the same for
// every job of the launch.  Every wait is bounded; a role that gives up
// makes the others leave, the block drains its copies and MMAs and flags
// every job of the launch.
// Multi: a table of jobs in device memory, a tile's job copied into its
// slot; otherwise the one job of the launch parameters (read through the
// constant bank).
template <bool Multi>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_track_kernel(const __grid_constant__ TcLaunch L) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ TcShared sh;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const TcArgs* jobs = Multi ? L.jobs : &L.single;
  const int njobs = Multi ? L.njobs : 1;
  // first launch tile of each job (the jobs' tile lists were planned on the device)
  if (t == 0) {
    int n = 0;
    for (int j = 0; j < njobs; ++j) {
      sh.job_base[j] = n;
      n += jobs[j].tiles->count;
    }
    sh.job_base[njobs] = n;
  }
  __syncthreads();
  const int ntiles = sh.job_base[njobs];
  if (int(blockIdx.x) >= ntiles) return;
  // launch shape: equal for every job
  const int stages = jobs[0].stages, stage_bytes = jobs[0].stage_bytes;
  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  uint8_t* wbase = smem;
  uint8_t* abase = smem + size_t(stages) * stage_bytes;
  if (t == 0) {
    bar_init(&sh.a_full[0], kTcWindowThreads);
    bar_init(&sh.a_full[1], kTcWindowThreads);
    bar_init(&sh.slab_done[0]);
    bar_init(&sh.slab_done[1]);
    bar_init(&sh.drain);
    for (int s = 0; s < kTcMaxStages; ++s) {
      bar_init(&sh.b_full[s]);
      bar_init(&sh.b_empty[s]);
    }
    for (int b = 0; b < 2; ++b) {
      bar_init(&sh.info_full[b]);
      bar_init(&sh.info_empty[b], 2 + kTcWindowThreads);  // MMA thread, weight producer, window warps
    }
    for (int b = 0; b < 2; ++b) {
      bar_init(&sh.acc_full[b]);
      bar_init(&sh.acc_empty[b]);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sh.fail = 0;
    sh.cm = sh.cb = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh.tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sh.tmem;
  if (warp == 0) {
    if (lane == 0) {
      RingPos cm;
      int sm = 0;
      for (int s = 0;; ++s) {
        const int b = s & 1;
        if (!bar_wait(&sh.info_full[b], uint32_t((s >> 1) & 1), &sh.fail)) {
          tc_fail(sh);
          break;
        }
        const TcSlot& ts = sh.slot[b];
        if (ts.gtile < 0) break;
        // the region's previous tile (s - 2) has been read by the epilogue
        if (s >= 2 && !bar_wait(&sh.acc_empty[b], uint32_t(((s >> 1) - 1) & 1), &sh.fail)) {
          tc_fail(sh);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!tc_mma_tile(Multi ? ts.job : L.single, ts, sh, wbase, abase, tmem + uint32_t(b) * kTcRegionCols,
                         &sh.acc_full[b], cm, sm)) {
          tc_fail(sh);
          break;
        }
        bar_arrive(&sh.info_empty[b]);
      }
      sh.cm = cm.count;
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      RingPos cb;
      for (int s = 0;; ++s) {
        const int b = s & 1;
        if (!bar_wait(&sh.info_full[b], uint32_t((s >> 1) & 1), &sh.fail)) {
          tc_fail(sh);
          break;
        }
        const TcSlot& ts = sh.slot[b];
        if (ts.gtile < 0) break;
        if (!tc_weight_tile(Multi ? ts.job : L.single, ts, sh, wbase, cb)) {
          tc_fail(sh);
          break;
        }
        bar_arrive(&sh.info_empty[b]);
      }
      sh.cb = cb.count;
    }
    __syncwarp();
  } else if (warp < 6) {
    // window warps: stage the tiles the epilogue warps set up
    const int pt = t - 64;
    int sa = 0;
    for (int s = 0;; ++s) {
      const int b = s & 1;
      if (!bar_wait(&sh.info_full[b], uint32_t((s >> 1) & 1), &sh.fail)) {
        tc_fail(sh);
        break;
      }
      const TcSlot& ts = sh.slot[b];
      if (ts.gtile < 0) break;
      if (!tc_window_tile(Multi ? ts.job : L.single, ts, sh, abase, sa, pt)) {
        tc_fail(sh);
        break;
      }
      bar_arrive(&sh.info_empty[b]);
    }
  } else {
    // epilogue warps (named barrier 2): the epilogue of tile s, then the
    // set-up of tile s + 2 in the slot it frees (tiles 0 and 1 first)
    const int quarter = warp & 3, et = t - 192;
    auto setup = [&](int sq) {
      if (et == 0) sh.claim = sq == 0 ? int(blockIdx.x) : int(gridDim.x) + atomicAdd(L.next, 1);
      named_sync(2, kTcEpilogueThreads);
      const int gtile = sh.claim;
      tc_setup<Multi>(jobs, sh, sh.slot[sq & 1], gtile, ntiles, et);
      named_sync(2, kTcEpilogueThreads);
      if (et == 0) bar_arrive(&sh.info_full[sq & 1]);
      return gtile < ntiles;
    };
    bool more = setup(0);
    if (more) more = setup(1);
    for (int s = 0;; ++s) {
      const int b = s & 1;
      const TcSlot& ts = sh.slot[b];
      if (ts.gtile < 0) break;
      bool ok = bar_wait(&sh.acc_full[b], uint32_t((s >> 1) & 1), &sh.fail);
      if (!named_and(2, kTcEpilogueThreads, ok)) {
        tc_fail(sh);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const TcArgs& a = Multi ? ts.job : L.single;
      const uint32_t trow = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b) * kTcRegionCols;
      if (ts.grp.rg == 4)
        tc_epilogue<4>(a, ts, trow, quarter, lane);
      else if (ts.grp.rg == 2)
        tc_epilogue<2>(a, ts, trow, quarter, lane);
      else
        tc_epilogue<1>(a, ts, trow, quarter, lane);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      named_sync(2, kTcEpilogueThreads);
      if (et == 0) {
        bar_arrive(&sh.acc_empty[b]);
        const TcGroup& G = ts.grp;
        atomicAdd(&a.state_rw->tc_macs, (unsigned long long)G.macs * (unsigned long long)ts.cnt);
        atomicAdd(&a.state_rw->tc_issued,
                  (unsigned long long)kTcRows * G.n * (G.parts * G.kw + 16) * ((G.kr + G.rg - 1) / G.rg));
      }
      if (more) {
        // the MMA thread, the weight producer and the window warps are done with tile s
        ok = bar_wait(&sh.info_empty[b], uint32_t((s >> 1) & 1), &sh.fail);
        if (!named_and(2, kTcEpilogueThreads, ok)) {
          tc_fail(sh);
          break;
        }
        more = setup(s + 2);
      }
    }
  }
  __syncthreads();
  if (sh.fail) {
    // drain in-flight weight copies and MMAs (bounded) before leaving, and
    // flag every job: tiles of any of them may be incomplete
    if (t == 0) {
      for (long long c = sh.cm; c < sh.cb; ++c)
        bar_wait(&sh.b_full[int(c % stages)], uint32_t((c / stages) & 1));
      mma_commit(&sh.drain);
      bar_wait(&sh.drain, 0);
      for (int j = 0; j < njobs; ++j) atomicExch(jobs[j].error, int32_t(kInternal));
    }
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// fp16 planes: thread = one row and one 8-column block, all 8 shifted
// planes (plane d holds level column x - kTcPlaneMargin + d at column x, so
// the block's planes need level columns 8 gx - 8 .. 8 gx + 6, read once),
// column-blocked: element (row y, column x) at ((x / 8) h + y) 8 + x mod 8,
// so the rows of an 8-column block are one contiguous run of 16-byte rows;
// consecutive threads take consecutive rows (coalesced stores)
template <int Parts>
__global__ void tc_planes_kernel(LevelImage lev, __half* planes, int pitch, float fixed_offset,
                                 const QueryState* state, float level_mult) {
  const float offset = tc_plane_offset(fixed_offset, state, level_mult);
  const int groups = pitch / 8;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)lev.h * groups) return;
  const int y = int(idx % lev.h);
  const int gx = int(idx / lev.h);
  const int x0 = gx * 8 - kTcPlaneMargin;
  const float* row = lev.v + size_t(y) * lev.w;
  float v[15];
#pragma unroll
  for (int j = 0; j < 15; ++j) {
    const int x = x0 + j;
    v[j] = x >= 0 && x < lev.w ? row[x] - offset : 0.f;
  }
  const size_t plane = size_t(lev.h) * pitch;
  const size_t at = (size_t(gx) * lev.h + y) * 8;
#pragma unroll
  for (int d = 0; d < kTcPlaneShifts; ++d) {
    __align__(16) __half pv[Parts][8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      // v = sum_q digit_q 64^(Parts - 1 - q): the first digit signed, the
      // others in [0, 64); every step is exact in float (|v| < 2^24)
      float r = v[e + d];
#pragma unroll
      for (int q = 0; q < Parts; ++q) {
        const float unit = float(1 << (6 * (Parts - 1 - q)));
        const float dq = q + 1 < Parts ? floorf(r * (1.f / unit)) : r;
        pv[q][e] = __float2half_rn(dq);
        r -= dq * unit;
      }
    }
#pragma unroll
    for (int q = 0; q < Parts; ++q)
      *reinterpret_cast<uint4*>(planes + (size_t(q) * kTcPlaneShifts + d) * plane + at) =
          *reinterpret_cast<const uint4*>(pv[q]);
  }
}

// Grouping of the step's candidates: counts per group, tile list, order.
__global__ void tc_count_kernel(const Cand* in, const QueryState* state, int slot, const int32_t* group_of_src,
                                int32_t* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= live_count(state, slot)) return;
  const int src = in[i].patch;
  const int gi = src >= 0 ? group_of_src[src] : -1;
  if (gi >= 0) atomicAdd(counts + gi, 1);
}

// Tile list: per group, tiles of up to 16 candidates in order (block-wide
// scan of the per-group candidate and tile counts, 1024 threads).
__global__ void __launch_bounds__(1024) tc_plan_kernel(const int32_t* counts, int ngroups, int32_t* offsets,
                                                       int32_t* cursor, TcTiles* tiles, int max_tiles) {
  __shared__ int s_cand[1024], s_tile[1024];
  const int t = threadIdx.x, per = (ngroups + 1023) / 1024;
  const int g0 = min(ngroups, t * per), g1 = min(ngroups, g0 + per);
  int c = 0, n = 0;
  for (int g = g0; g < g1; ++g) {
    c += counts[g];
    n += (counts[g] + kTcCands - 1) / kTcCands;
  }
  s_cand[t] = c;
  s_tile[t] = n;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int a = t >= off ? s_cand[t - off] : 0, b = t >= off ? s_tile[t - off] : 0;
    __syncthreads();
    s_cand[t] += a;
    s_tile[t] += b;
    __syncthreads();
  }
  int at = s_cand[t] - c, nt = s_tile[t] - n;
  for (int g = g0; g < g1; ++g) {
    offsets[g] = at;
    cursor[g] = 0;
    const int cg = counts[g];
    for (int f = 0; f < cg; f += kTcCands, ++nt) {
      if (nt >= max_tiles) continue;
      tiles->group[nt] = g;
      tiles->first[nt] = at + f;
      tiles->last[nt] = at + min(cg, f + kTcCands);
    }
    at += cg;
  }
  if (t == 1023) {
    tiles->count = min(s_tile[1023], max_tiles);
    tiles->next = 0;
  }
}

__global__ void tc_scatter_kernel(const Cand* in, const QueryState* state, int slot, const int32_t* group_of_src,
                                  const int32_t* offsets, int32_t* cursor, int32_t* order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= live_count(state, slot)) return;
  const int src = in[i].patch;
  const int gi = src >= 0 ? group_of_src[src] : -1;
  if (gi < 0) return;
  order[offsets[gi] + atomicAdd(cursor + gi, 1)] = i;
}

}  // namespace

size_t tc_kernel_static_smem() { return sizeof(TcShared); }

cudaError_t launch_tc_planes(const LevelImage& lev, uint16_t* planes, int pitch, int parts, float offset,
                             cudaStream_t s, const QueryState* state, float level_mult) {
  const long long total = (long long)lev.h * (pitch / 8);
  const unsigned blocks = unsigned((total + 255) / 256);
  __half* p = reinterpret_cast<__half*>(planes);
  switch (parts) {
    case 1: tc_planes_kernel<1><<<blocks, 256, 0, s>>>(lev, p, pitch, offset, state, level_mult); break;
    case 2: tc_planes_kernel<2><<<blocks, 256, 0, s>>>(lev, p, pitch, offset, state, level_mult); break;
    case 3: tc_planes_kernel<3><<<blocks, 256, 0, s>>>(lev, p, pitch, offset, state, level_mult); break;
    case 4: tc_planes_kernel<4><<<blocks, 256, 0, s>>>(lev, p, pitch, offset, state, level_mult); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

namespace {
// min / max of a level (exact integers held as float), grid-stride
__global__ void level_range_kernel(LevelImage lev, QueryState* state) {
  const size_t n = size_t(lev.w) * size_t(lev.h);
  float mn = INFINITY, mx = -INFINITY;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float v = lev.v[i];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  for (int o = 16; o; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0 && mn <= mx) {
    atomicMin(&state->pix_min, int(mn));
    atomicMax(&state->pix_max, int(mx));
  }
}
}  // namespace

cudaError_t launch_level_range(const LevelImage& lev0, QueryState* state, cudaStream_t s) {
  level_range_kernel<<<608, 256, 0, s>>>(lev0, state);
  return cudaGetLastError();
}

cudaError_t launch_tc_group(const TcArgs& a, int ngroups, int32_t* counts, int32_t* offsets, int32_t* cursor,
                            int max_candidates, cudaStream_t s) {
  if (cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * size_t(ngroups), s)) return e;
  const unsigned blocks = unsigned((max_candidates + 255) / 256);
  tc_count_kernel<<<blocks, 256, 0, s>>>(a.in, a.state, a.in_slot, a.group_of_src, counts);
  tc_plan_kernel<<<1, 1024, 0, s>>>(counts, ngroups, offsets, cursor, a.tiles, kTcMaxTiles);
  tc_scatter_kernel<<<blocks, 256, 0, s>>>(a.in, a.state, a.in_slot, a.group_of_src, offsets, cursor, a.order);
  return cudaGetLastError();
}

cudaError_t launch_tc_track(const TcLaunch& l, size_t smem, int grid, cudaStream_t s) {
  if (l.njobs < 1 || l.njobs > kTcMaxJobs) return cudaErrorInvalidValue;
  const void* fn = l.jobs ? reinterpret_cast<const void*>(tc_track_kernel<true>)
                           : reinterpret_cast<const void*>(tc_track_kernel<false>);
  if (cudaError_t e = reserve_dynamic_smem(fn, smem)) return e;
  // a single job's counter (its tile list's) is reset by the tile planner
  if (l.jobs)
    if (cudaError_t e = cudaMemsetAsync(l.next, 0, sizeof(int), s)) return e;
  if (l.jobs)
    tc_track_kernel<true><<<grid, kTcThreads, smem, s>>>(l);
  else
    tc_track_kernel<false><<<grid, kTcThreads, smem, s>>>(l);
  return cudaGetLastError();
}

}  // namespace mvg
