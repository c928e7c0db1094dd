// tcgen05 (5th-gen tensor core) triple-product contraction, bf16x3 / bf16.
//
//   C[(i,j), l] += sum_x P_ij(x) * F3_l(x),   P_ij = F1_i * F2_j  (FP32, formed on chip)
//
// One persistent CTA per SM walks work items (tile of 128 pair rows x nc <= 64
// columns, K slice of `slice` points), slice-major so that the CTAs running at
// the same time share field data in L2.  Per 128-point pipeline stage:
//   * warp 0 (one lane) TMA-loads into an SMEM ring (3 stages with one source
//     tile, 2 with two) the bf16 hi and lo tiles of the column fields in one copy
//     from their chunk-major split ([block][plane][nc rows][64 points] per stage:
//     per 64-point K block an operand of nc hi rows followed by nc lo rows;
//     SWIZZLE_128B, K-major), and the FP32 tile(s) of the pair-factor shells
//     (one tile when one range covers both factors of every row, as for auto
//     spectra), each with only as many shell rows (a multiple of 8) as the tile uses.
//     A stage's source tiles are refilled as soon as the A-operand warps have read
//     them and its B tiles once the stage's MMAs completed, each part with its own
//     "landed" barrier, so the sources get about one more stage of lead time;
//   * warps 10..25 (AGW = 4 per TMEM lane quadrant, one 32-point quarter each) read the
//     row's F1_i, F2_j from SMEM (one 8-point group ahead of the math), form
//     P = F1_i*F2_j with packed f32x2 arithmetic, split P = hi + lo (bf16
//     round-to-nearest) and store them with tcgen05.st into the 2-stage TMEM
//     A-operand ring (lane = GEMM row);
//   * warp 1 runs the stage loop and one elected lane issues, per 16-point K step,
//     tcgen05.mma kind::f16 with A from TMEM and B from SMEM: hi x [Bhi; Blo]
//     (N = 2 nc: one MMA yields both hi*Bhi and hi*Blo) and, for bf16x3, lo x [Bhi; Blo]
//     into the same columns (lo*Bhi onto hi*Bhi, lo*Blo onto hi*Blo): all four cross
//     products of the two-term splits.  The tensor pipe is not this kernel's limit, so the
//     fourth product (lo x Blo, below 2^-18 of a term) costs ~3% of the contraction and
//     narrows the tail of the per-bin errors.  The tensor core's FP32 accumulate
//     truncates, so an accumulator is only ever fed one stage (16 MMAs) before it is
//     handed over;
//   * warps 2..9 (2 per lane quadrant, 32 columns each) drain each finished
//     accumulator with tcgen05.ld (hi*Bhi + lo*Bhi columns and hi*Blo + lo*Blo columns),
//     add it into per-thread FP32 registers (round-to-nearest), and at the end
//     of the slice add the entries that are triangle bins into the FP64 output
//     (atomics).
// The MMAs' completion is committed once per stage, to a ring of mbarriers that
// the TMA producer (the stage's B tiles free), the A-operand warps (TMEM A stage free)
// and the drain (accumulator ready) all wait on.  Stages are 128 points long so that the
// fixed cost of a stage's barrier round trips is spread over 16 MMAs.  Every wait is bounded
// (globaltimer); on expiry the kernel records an error flag, stops issuing work, drains
// its own MMAs and frees TMEM.
#include <cuda.h>

#include <atomic>

#include "bsk_internal.cuh"

namespace bsk {
namespace tc {

constexpr int KCH = 128;                      // points per pipeline stage
constexpr int ACC_CHUNKS = 1;                 // stages summed inside one TMEM accumulator
constexpr int ASTAGES = 2;                    // TMEM A-operand ring
constexpr int NACC = 2;                       // TMEM accumulators
constexpr int B_TILE = kMaxCols * 128;        // 8 KB: 64 rows x 64 bf16 (one 64-point SWIZZLE_128B
                                              // K block of the B operand, hi or lo)
constexpr int B_BLOCK = 2 * B_TILE;           // 16 KB: hi then lo of one K block
constexpr int A_QUARTER = kMaxSrcRows * 128;  // 8 KB: 64 rows x 32 fp32
constexpr int A_TILE = 4 * A_QUARTER;         // 32 KB: one source tile of a stage
// A-operand warps per TMEM lane quadrant, one 128 / AGW-point part of a stage each.  Their
// shared-memory loads are latency-bound: 4 per quadrant ran 3.5% faster than 2, with 72
// registers a thread instead of 96.
constexpr int AGW = 4;
constexpr int NUM_WARPS = 10 + 4 * AGW;       // producer, MMA, 8 drain, 4 AGW A-operand
constexpr int THREADS = NUM_WARPS * 32;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_COL = 0;               // accumulator b at 128 b: [0,nc) hi*Bhi+lo*Bhi, [nc,2nc) hi*Blo+lo*Blo
constexpr uint32_t A_COL = 256;               // A stage a at 256 + 128 a: hi +0..63, lo +64..127
// Points per work item: 32 768 when that still gives every SM at least kMinItemsPerSm
// items (one CTA per SM walks them), else 16 384.  Longer slices spread the per-item
// epilogue (the FP64 atomics of the tile's bins) over more stages: 24.2 -> 23.1 ms on the
// 512^3 headline; shorter ones keep small problems spread over all SMs.
constexpr int64_t kSliceLong = 32768, kSliceShort = 16384;
constexpr int64_t kMinItemsPerSm = 8;
constexpr unsigned long long kTimeoutNs = 2000000000ull;

// An SMEM stage holds two K blocks of B hi / lo (32 KB) + one or two FP32 source
// tiles (32 KB each).
template <bool kTwoSrc> struct Ring {
  static constexpr int kStageBytes = 2 * B_BLOCK + (kTwoSrc ? 2 : 1) * A_TILE;
  static constexpr int kStages = kTwoSrc ? 2 : 3;
};
constexpr int MAX_SSTAGES = 3;

// One commit per stage serves every consumer of "the stage's MMAs are complete": the TMA
// producer (the stage's B tiles free, SST stages later), the A-operand warps (TMEM A stage free,
// ASTAGES later) and the drain (accumulator ready, the same stage).  DONE_RING > all of
// those distances, so no barrier of the ring completes twice before each of its waiters
// has seen the phase (each waiter's progress gates the MMA thread's).
constexpr int DONE_RING = 4;
static_assert(ACC_CHUNKS == 1, "the drain waits on the per-stage completion");

struct Bars {
  uint64_t full[MAX_SSTAGES];      // the stage's source tiles landed (TMA bytes)
  uint64_t full_b[MAX_SSTAGES];    // the stage's B tiles landed (TMA bytes)
  uint64_t src_free[MAX_SSTAGES];  // the A-operand warps have read the stage's sources (4 AGW)
  uint64_t done[DONE_RING];        // the MMAs of stage c completed (tcgen05.commit), c % 4
  uint64_t afull[ASTAGES];         // A operand of the chunk is in TMEM (4 AGW warp arrivals)
  uint64_t accempty[NACC];
  uint64_t all_done;
  uint32_t tmem_base;
};

template <bool kTwoSrc>
constexpr int smem_bytes() {
  return Ring<kTwoSrc>::kStages * Ring<kTwoSrc>::kStageBytes + 1024 /*bars*/ + 1024 /*align*/;
}

// Tensor maps of one launch.  B: a 5D view of the chunk-major bf16 split {64 points,
// shell, hi/lo plane, 64-point block, 128-point chunk} with box {64, nc, 2, 2, 1}: one
// contiguous copy per stage, one map per nc = 8, 16, ..., 64.  Sources: FP32 [shell][K]
// with 16/32/64-row boxes (2D, one 32-point block per copy) and, when the grid is a
// multiple of 128 points, the one-copy view {32 points, shell, 32-point block} with box
// {32, rows, 4}, one map per rows = 8, 16, ..., 64.
constexpr int kRowSizes = kMaxCols / 8;
struct Maps {
  CUtensorMap f1_16, f1_32, f1_64, f2_16, f2_32, f2_64;
  CUtensorMap b[kRowSizes], a1[kRowSizes], a2[kRowSizes];
};
static_assert(kMaxSrcRows == kMaxCols, "one row-size list serves B and the sources");

__device__ int g_tc_error;  // 0 ok, 1 a bounded wait expired

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the wait expired or another role already gave up.
// mbarrier.try_wait suspends the thread in hardware for a while, so the loop
// is cheap; the clock is read every 16 polls and global memory (the shared
// error flag, the wall clock) only about every 2^20 cycles, so that no memory
// round trip sits between a barrier's completion and the waiter seeing it.
__device__ __noinline__ bool mbar_wait_slow(uint64_t* bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  long long c0 = clock64();
  unsigned long long t0 = 0;
  while (true) {
#pragma unroll 1
    for (int i = 0; i < 16; ++i)
      if (mbar_try(bar, parity)) return true;
    const long long c = clock64();
    if (c - c0 > (1ll << 20)) {
      c0 = c;
      if (*(volatile int*)&g_tc_error) return false;
      const unsigned long long t = globaltimer();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > kTimeoutNs) {
        atomicExch(&g_tc_error, 1);
        return false;
      }
    }
  }
}
// A phase that is already complete costs one try_wait inline; the polling loop is
// out of line.  (A call per wait was a measurable share of the MMA thread's time.)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  return mbar_wait_slow(bar, parity);
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z, int w, int v) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(v),
      "r"(smem_u32(bar))
      : "memory");
}
// The map of a list for a row count n (a multiple of 8, 8..64).
__device__ __forceinline__ const CUtensorMap* by_rows(const CUtensorMap (&maps)[kRowSizes],
                                                      int n) {
  return &maps[(n >> 3) - 1];
}
// One lane of a fully active warp (elect.sync picks the lowest active lane).
__device__ __forceinline__ bool elect_one() {
  uint32_t pred = 0;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "elect.sync _|p, 0xffffffff;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(pred));
  return pred != 0;
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// D[tmem] (+)= A[tmem] * B[smem]^T, kind::f16 (bf16 in, f32 accumulate)
__device__ __forceinline__ void mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc,
                                       uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(
          taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// UMMA shared-memory descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (16 B, unused for SW128)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                    // layout: SWIZZLE_128B
  return d;
}
// Instruction descriptor: D=F32, A=B=BF16, both K-major, M=128, N=n.
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// Rows a load of `n` shell rows covers: 16, 32, 48 (32 + 16) or 64.
__host__ __device__ __forceinline__ int box_rows(int n) {
  return n <= 16 ? 16 : n <= 32 ? 32 : n <= 48 ? 48 : 64;
}
// Load rows [y, y + box_rows(n)) of 128-B rows at x into dst (SWIZZLE_128B layout).
__device__ __forceinline__ void load_rows(uint32_t dst, const CUtensorMap* m16,
                                          const CUtensorMap* m32, const CUtensorMap* m64,
                                          uint64_t* bar, int x, int y, int n) {
  if (n > 48) {
    tma_load_2d(dst, m64, bar, x, y);
  } else if (n > 16) {
    tma_load_2d(dst, m32, bar, x, y);
    if (n > 32) tma_load_2d(dst + 32 * 128, m16, bar, x, y + 32);
  } else {
    tma_load_2d(dst, m16, bar, x, y);
  }
}

// Packed FP32x2 helpers (two lanes of a 64-bit register pair).
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint32_t bf16x2_of(unsigned long long p) {
  return pack_bf16(__uint_as_float((uint32_t)p), __uint_as_float((uint32_t)(p >> 32)));
}
// hi/lo split of two products held as f32x2: returns (hi bf16x2, lo bf16x2), lo = bf16(p - hi).
__device__ __forceinline__ void split2(unsigned long long p, uint32_t& hi, uint32_t& lo) {
  hi = bf16x2_of(p);
  const unsigned long long g =
      ((unsigned long long)(hi & 0xFFFF0000u) << 32) | (unsigned long long)(hi << 16);
  lo = bf16x2_of(f2_sub(p, g));
}

// 26 warps: 7 share one SM sub-partition, whose 16K registers allow 73 per thread.
template <bool kTwoSrc, bool kLongSlice>
__global__ void __launch_bounds__(THREADS, 1)
    contract_tc_kernel(const __grid_constant__ Maps maps, const TileDesc* __restrict__ tiles,
                       const int16_t* __restrict__ row_i, const int16_t* __restrict__ row_j,
                       const int32_t* __restrict__ map, int n_tiles, int same_src,
                       int64_t k_begin, int64_t k_end, int64_t n_items, int terms, int fused,
                       double* __restrict__ out, double scale) {
  constexpr int64_t slice = kLongSlice ? kSliceLong : kSliceShort;
  constexpr int STAGE_BYTES = Ring<kTwoSrc>::kStageBytes;
  constexpr int SST = Ring<kTwoSrc>::kStages;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  Bars* bars = reinterpret_cast<Bars*>(smem + SST * STAGE_BYTES);
  const uint32_t sbase = raw + pad;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < SST; ++s) {
      mbar_init(&bars->full[s], 1);
      mbar_init(&bars->full_b[s], 1);
      mbar_init(&bars->src_free[s], 4 * AGW);

    }
    for (int a = 0; a < ASTAGES; ++a) {
      mbar_init(&bars->afull[a], 4 * AGW);

    }
    for (int b = 0; b < NACC; ++b) {

      mbar_init(&bars->accempty[b], 8);
    }
    for (int d = 0; d < DONE_RING; ++d) mbar_init(&bars->done[d], 1);
    mbar_init(&bars->all_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&bars->tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = bars->tmem_base;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      uint32_t chunk = 0;
      bool ok = true;
      for (int64_t item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
        const int64_t sl = item / n_tiles;
        const TileDesc td = tiles[item % n_tiles];
        const bool one_src = !kTwoSrc || (same_src && td.i0 == td.j0);
        const int64_t x_begin = k_begin + sl * slice;
        const int64_t x_end = min(k_end, x_begin + slice);
        // bytes per stage: the four 32-point quarters of each source tile; the column rows
        // of hi and lo in both K blocks
        const uint32_t src_bytes =
            fused ? (uint32_t)(4 * 128 * (td.ni + (one_src ? 0 : td.nj)))
                  : (uint32_t)(4 * 128 * (box_rows(td.ni) + (one_src ? 0 : box_rows(td.nj))));
        const uint32_t b_bytes = (uint32_t)(4 * td.nc * 128);
        for (int64_t x = x_begin; x < x_end; x += KCH, ++chunk) {
          const int s = chunk % SST;
          const uint32_t st = sbase + s * STAGE_BYTES;
          const int xi = (int)x;
          // The source tiles of SMEM stage s were last read by the A-operand warps of stage
          // chunk - SST, its B tiles by that stage's MMAs, which complete ~one A-operand
          // stage later: the sources are refilled as soon as they are free.
          if (chunk >= SST &&
              !mbar_wait(&bars->src_free[s], (uint32_t)((chunk - SST) / SST) & 1)) {
            ok = false;
            break;
          }
          mbar_arrive_tx(&bars->full[s], src_bytes);
          if (fused) {
            // one copy per source tile ([32-point block][rows])
            tma_load_3d(st + 2 * B_BLOCK, by_rows(maps.a1, td.ni), &bars->full[s], 0, td.i0,
                        xi / 32);
            if (!one_src)
              tma_load_3d(st + 2 * B_BLOCK + 4 * 128 * td.ni, by_rows(maps.a2, td.nj),
                          &bars->full[s], 0, td.j0, xi / 32);
          } else {
            for (int q = 0; q < 4; ++q) {
              load_rows(st + 2 * B_BLOCK + q * A_QUARTER, &maps.f1_16, &maps.f1_32, &maps.f1_64,
                        &bars->full[s], xi + 32 * q, td.i0, td.ni);
              if (!one_src)
                load_rows(st + 2 * B_BLOCK + A_TILE + q * A_QUARTER, &maps.f2_16, &maps.f2_32,
                          &maps.f2_64, &bars->full[s], xi + 32 * q, td.j0, td.nj);
            }
          }
          if (chunk >= SST && !mbar_wait(&bars->done[(chunk - SST) % DONE_RING],
                                          ((chunk - SST) / DONE_RING) & 1)) {
            ok = false;
            break;
          }
          mbar_arrive_tx(&bars->full_b[s], b_bytes);
          // one contiguous copy for B: the stage's 128-point chunk of the split, nc shells,
          // both planes, both 64-point blocks -> [block][plane][nc rows][64]
          tma_load_5d(st, by_rows(maps.b, td.nc), &bars->full_b[s], 0, td.l0, 0, 0, xi / KCH);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    // The whole warp runs the loop (barrier waits, stage addresses and descriptors are
    // warp-uniform values) and one elected lane issues each stage's 16 MMAs and its commit
    // as one straight run; a loop run by a single lane issued 3-4x slower.
    uint32_t chunk = 0, grp = 0;
    bool ok = true;
    for (int64_t item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const int64_t sl = item / n_tiles;
      const TileDesc td = tiles[item % n_tiles];
      const int64_t x_begin = k_begin + sl * slice;
      const int64_t x_end = min(k_end, x_begin + slice);
      // hi x [Bhi; Blo] and lo x [Bhi; Blo] (the lo rows of a block sit right after its nc
      // hi rows; N = 2 nc, a multiple of 16).  bf16 (one term): hi x Bhi, N = nc rounded up
      // to 16 (with nc an odd multiple of 8 the last 8 columns take lo rows, never read).
      const int n16 = (td.nc + 15) & ~15;
      const uint32_t kb_bytes = 2u * td.nc * 128u;
      const uint32_t idesc_stack = idesc_bf16(terms >= 3 ? 2 * td.nc : n16);
      for (int64_t x = x_begin; x < x_end; x += KCH, ++chunk) {
        // a fresh accumulator per stage, once the drain has emptied it
        const uint32_t b = grp % NACC;
        const int s = chunk % SST;
        const uint32_t ph = (chunk / SST) & 1;
        const int a = chunk % ASTAGES;
        const uint32_t pa = (chunk / ASTAGES) & 1;
        if (!__all_sync(0xffffffffu, mbar_wait(&bars->accempty[b], ((grp / NACC) & 1) ^ 1) &&
                                         mbar_wait(&bars->full_b[s], ph) &&
                                         mbar_wait(&bars->afull[a], pa))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d_tmem = tmem + ACC_COL + b * 128;
        const uint32_t st = sbase + s * STAGE_BYTES;
        const uint32_t a_hi = tmem + A_COL + a * 128;
        const uint32_t a_lo = a_hi + 64;
        if (elect_one()) {
          uint32_t accum = 0;
#pragma unroll
          for (int k = 0; k < KCH / 16; ++k) {
            const uint64_t bdesc = desc_sw128(st + (k >> 2) * kb_bytes + 32 * (k & 3));
            mma_ts(d_tmem, a_hi + 8 * k, bdesc, idesc_stack, accum);
            if (terms >= 3) mma_ts(d_tmem, a_lo + 8 * k, bdesc, idesc_stack, 1);
            accum = 1;
          }
          tc_commit(&bars->done[chunk % DONE_RING]);
        }
        __syncwarp();
        ++grp;
      }
    }
    // all MMAs of this CTA complete before TMEM is released (the elected lane is the
    // same lane every time: elect.sync over a full warp picks its lowest lane)
    if (elect_one()) tc_commit(&bars->all_done);
    __syncwarp();
    mbar_wait(&bars->all_done, 0);
  } else if (warp < 10) {
    // ------------------------------------------------------------ accumulator drain
    const int qd = warp & 3;
    const int c0 = ((warp - 2) >> 2) * 32;  // this warp's 32 accumulator columns
    const int r = qd * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(qd * 32) << 16) + c0;
    uint32_t grp = 0;
    bool ok = true;
    for (int64_t item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const int64_t sl = item / n_tiles;
      const TileDesc td = tiles[item % n_tiles];
      const int64_t x_begin = k_begin + sl * slice;
      const int64_t x_end = min(k_end, x_begin + slice);
      const int64_t nch = (x_end - x_begin + KCH - 1) / KCH;
      const int64_t ngrp = (nch + ACC_CHUNKS - 1) / ACC_CHUNKS;
      float acc[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) acc[c] = 0.f;
      for (int64_t g = 0; g < ngrp; ++g, ++grp) {
        const uint32_t b = grp % NACC;
        if (!__all_sync(0xffffffffu,
                        mbar_wait(&bars->done[grp % DONE_RING], (grp / DONE_RING) & 1))) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
          if (c0 + cc * 16 < td.nc) {
            uint32_t v[16];
            tmem_ld16(taddr + ACC_COL + b * 128 + cc * 16, v);
#pragma unroll
            for (int e = 0; e < 16; ++e) acc[cc * 16 + e] += __uint_as_float(v[e]);
            if (terms >= 3) {
              tmem_ld16(taddr + ACC_COL + b * 128 + td.nc + cc * 16, v);
#pragma unroll
              for (int e = 0; e < 16; ++e) acc[cc * 16 + e] += __uint_as_float(v[e]);
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars->accempty[b]);
      }
      if (!ok) break;
      const int32_t* mp = map + td.map_off + c0 * kTileRows + r;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        if (c0 + c < td.nc) {
          const int t = __ldg(mp + c * kTileRows);
          if (t >= 0) atomicAdd(out + t, (double)acc[c] * scale);
        }
      }
    }
  } else {
    // ------------------------------------------------------------ A-operand producers
    const int qd = warp & 3;
    constexpr int PPW = KCH / AGW, NG = PPW / 8;  // points per warp, 8-point groups
    const int part = (warp - 10) >> 2;  // points [PPW part, PPW part + PPW) of a stage
    const int r = qd * 32 + lane;
    const uint32_t tlane = (uint32_t)(qd * 32) << 16;
    uint32_t chunk = 0;
    bool ok = true;
    for (int64_t item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const int64_t sl = item / n_tiles;
      const TileDesc td = tiles[item % n_tiles];
      const bool one_src = !kTwoSrc || (same_src && td.i0 == td.j0);
      const int64_t x_begin = k_begin + sl * slice;
      const int64_t x_end = min(k_end, x_begin + slice);
      const int ri = row_i[td.row_off + r];
      const int rj = row_j[td.row_off + r];
      const bool valid = ri >= 0;
      const int pi = valid ? ri - td.i0 : 0;
      const int pj = valid ? rj - td.j0 : 0;
      // source tiles: [32-point quarter][rows] with the quarter stride of the copy
      const int qstride = fused ? td.ni * 128 : A_QUARTER;
      const int src2 = one_src ? 0 : (fused ? 4 * qstride : A_TILE);
      const int qstride2 = one_src ? qstride : (fused ? td.nj * 128 : A_QUARTER);
      for (int64_t x = x_begin; x < x_end; x += KCH, ++chunk) {
        const int s = chunk % SST;
        const uint32_t ph = (chunk / SST) & 1;
        const int a = chunk % ASTAGES;
        if (!__all_sync(0xffffffffu, mbar_wait(&bars->full[s], ph))) { ok = false; break; }
        // TMEM A stage a was last read by the MMAs of stage chunk - ASTAGES
        if (chunk >= ASTAGES &&
            !__all_sync(0xffffffffu, mbar_wait(&bars->done[(chunk - ASTAGES) % DONE_RING],
                                               ((chunk - ASTAGES) / DONE_RING) & 1))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint8_t* st = smem + s * STAGE_BYTES;
        const uint32_t a_hi = tmem + tlane + A_COL + a * 128 + part * (PPW / 2);
        // The warp's PPW points in NG groups of 8; the shared-memory loads of group g + 1
        // are issued before the math of group g (software pipelining: the loads' latency,
        // not the load pipe's bandwidth, bounds these warps).  Group g (stage points p0 ..
        // p0 + 7) covers the 16-byte chunks (p0 % 32) / 4 + e (e < 2) of 32-point quarter
        // p0 / 32 of the source tile; two groups fill one 16-point K step of the A operand.
        auto load_group = [&](int g, ulonglong2 (&va)[2], ulonglong2 (&vb)[2]) {
          const int p0 = part * PPW + 8 * g;
          const int qq = p0 >> 5;
          const uint8_t* row1 = st + 2 * B_BLOCK + qq * qstride + pi * 128;
          const uint8_t* row2 = st + 2 * B_BLOCK + src2 + qq * qstride2 + pj * 128;
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int c = ((p0 & 31) >> 2) + e;
            va[e] = *reinterpret_cast<const ulonglong2*>(row1 + ((c ^ (pi & 7)) << 4));
            vb[e] = *reinterpret_cast<const ulonglong2*>(row2 + ((c ^ (pj & 7)) << 4));
          }
        };
        ulonglong2 ca[2], cb[2], na[2], nb[2];
        load_group(0, ca, cb);
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          if (g + 1 < NG) load_group(g + 1, na, nb);
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int c4 = (g & 1) * 2 + e;
            split2(f2_mul(ca[e].x, cb[e].x), hi[2 * c4], lo[2 * c4]);
            split2(f2_mul(ca[e].y, cb[e].y), hi[2 * c4 + 1], lo[2 * c4 + 1]);
          }
          if (g & 1) {
            if (!valid) {  // rows past the tile's pairs: zeros (their sums are never read)
#pragma unroll
              for (int e = 0; e < 8; ++e) hi[e] = lo[e] = 0u;
            }
            tmem_st8(a_hi + (g >> 1) * 8, hi);
            tmem_st8(a_hi + 64 + (g >> 1) * 8, lo);
          }
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            ca[e] = na[e];
            cb[e] = nb[e];
          }
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&bars->afull[a]);
          mbar_arrive(&bars->src_free[s]);  // this warp's loads of the stage's sources are done
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  // resolved once (thread-safe static initialisation; a throw leaves it for the next call)
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    BSK_CHECK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                    cudaEnableDefault, &q));
    BSK_REQUIRE(q == cudaDriverEntryPointSuccess && p, BSK_ERR_CUDA,
                "cuTensorMapEncodeTiled entry point unavailable");
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// 2D map over a [rows][K] array: box = {box_x elements, box_y rows}, SWIZZLE_128B.
void make_map(CUtensorMap* m, CUtensorMapDataType dt, int esize, const void* base, int64_t K,
              int rows, int box_x, int box_y) {
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * esize};
  cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(m, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  BSK_REQUIRE(r == CUDA_SUCCESS, BSK_ERR_CUDA,
              "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

// View of a [rows][K] array with K cut into blocks of `blk` points:
// dims {blk, rows, K / blk}; box {blk, box_rows, nblk}.  Returns false (map unusable)
// instead of failing when the CUDA driver rejects the layout.
bool make_block_map(CUtensorMap* m, CUtensorMapDataType dt, int esize, const void* base,
                    int64_t K, int rows, int blk, int box_rows, int nblk) {
  cuuint64_t dims[3] = {(cuuint64_t)blk, (cuuint64_t)rows, (cuuint64_t)(K / blk)};
  cuuint64_t strides[2] = {(cuuint64_t)K * esize, (cuuint64_t)blk * esize};
  cuuint32_t box[3] = {(cuuint32_t)blk, (cuuint32_t)box_rows, (cuuint32_t)nblk};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode_fn()(m, dt, 3, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The chunk-major bf16 split (split_index) as {64 points, shell, hi/lo plane, 64-point
// block, 128-point chunk}; box {64, box_rows, 2, 2, 1} lands as [block][plane][rows][64].
void make_split_map(CUtensorMap* m, const __nv_bfloat16* split, int S, int64_t K, int box_rows) {
  cuuint64_t dims[5] = {64, (cuuint64_t)S, 2, 2, (cuuint64_t)((K + KCH - 1) / KCH)};
  cuuint64_t strides[4] = {256, (cuuint64_t)S * 256, 128, (cuuint64_t)S * 512};
  cuuint32_t box[5] = {64, (cuuint32_t)box_rows, 2, 2, 1};
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5,
                           const_cast<__nv_bfloat16*>(split), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  BSK_REQUIRE(r == CUDA_SUCCESS, BSK_ERR_CUDA,
              "cuTensorMapEncodeTiled (split) failed: " + std::to_string((int)r));
}

}  // namespace tc

void launch_contract_tc(const DeviceSchedule& s, const float* f1, const float* f2,
                        const __nv_bfloat16* f3_split, int split_shells, int n_shells,
                        int64_t K, int64_t k_begin, int64_t k_end, int terms, double* out,
                        int num_sms, cudaStream_t st, double scale) {
  if (s.n_tiles == 0 || k_end <= k_begin) return;
  BSK_REQUIRE(k_begin % tc::KCH == 0, BSK_ERR_ARG, "k_begin must be a multiple of 128");
  BSK_REQUIRE(k_end % tc::KCH == 0 || k_end == K, BSK_ERR_ARG,
              "k_end must be a multiple of 128 or the whole grid");
  BSK_REQUIRE(K < (int64_t)1 << 31, BSK_ERR_UNSUPPORTED, "grid too large for 32-bit TMA x");
  BSK_REQUIRE(K % 8 == 0, BSK_ERR_UNSUPPORTED, "K must be a multiple of 8");
  tc::Maps m;
  const auto F32 = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  tc::make_map(&m.f1_16, F32, 4, f1, K, n_shells, 32, 16);
  tc::make_map(&m.f1_32, F32, 4, f1, K, n_shells, 32, 32);
  tc::make_map(&m.f1_64, F32, 4, f1, K, n_shells, 32, 64);
  tc::make_map(&m.f2_16, F32, 4, f2, K, n_shells, 32, 16);
  tc::make_map(&m.f2_32, F32, 4, f2, K, n_shells, 32, 32);
  tc::make_map(&m.f2_64, F32, 4, f2, K, n_shells, 32, 64);
  for (int i = 0; i < tc::kRowSizes; ++i)
    tc::make_split_map(&m.b[i], f3_split, split_shells, K, 8 * (i + 1));
  // one copy per stage per source tile when K is a multiple of the stage
  bool fused = K % tc::KCH == 0;
  for (int i = 0; i < tc::kRowSizes && fused; ++i) {
    fused = tc::make_block_map(&m.a1[i], F32, 4, f1, K, n_shells, 32, 8 * (i + 1), 4) &&
            tc::make_block_map(&m.a2[i], F32, 4, f2, K, n_shells, 32, 8 * (i + 1), 4);
  }
  bool two_src = f1 != f2;
  for (const TileDesc& d : s.h_tiles) two_src = two_src || d.i0 != d.j0;
  const bool long_slice = (k_end - k_begin + tc::kSliceLong - 1) / tc::kSliceLong * s.n_tiles >=
                         tc::kMinItemsPerSm * num_sms;
  const int64_t slice = long_slice ? tc::kSliceLong : tc::kSliceShort;
  const int64_t n_slices = (k_end - k_begin + slice - 1) / slice;
  const int64_t n_items = n_slices * s.n_tiles;
  constexpr int kMaxDev = 64;
  static std::atomic<bool> attr_set[kMaxDev][4];  // zero-initialised: false
  int dev = 0;
  BSK_CHECK_CUDA(cudaGetDevice(&dev));
  BSK_REQUIRE(dev < kMaxDev, BSK_ERR_UNSUPPORTED, "device ordinal above 63");
  auto kern = two_src ? (long_slice ? tc::contract_tc_kernel<true, true>
                                    : tc::contract_tc_kernel<true, false>)
                      : (long_slice ? tc::contract_tc_kernel<false, true>
                                    : tc::contract_tc_kernel<false, false>);
  const int smem = two_src ? tc::smem_bytes<true>() : tc::smem_bytes<false>();
  const int variant = (two_src ? 2 : 0) + (long_slice ? 1 : 0);
  if (!attr_set[dev][variant]) {
    BSK_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr_set[dev][variant] = true;
  }
  int64_t grid = num_sms;
  if (grid > n_items) grid = n_items;
  kern<<<(unsigned)grid, tc::THREADS, smem, st>>>(
      m, s.tiles, s.row_i, s.row_j, s.map, s.n_tiles, f1 == f2 ? 1 : 0, k_begin, k_end,
      n_items, terms, fused ? 1 : 0, out, scale);
  BSK_CHECK_CUDA(cudaGetLastError());
}

int tc_error_flag(bool reset) {
  int v = 0;
  BSK_CHECK_CUDA(cudaMemcpyFromSymbol(&v, tc::g_tc_error, sizeof(int)));
  if (reset && v) {
    int z = 0;
    BSK_CHECK_CUDA(cudaMemcpyToSymbol(tc::g_tc_error, &z, sizeof(int)));
  }
  return v;
}

}  // namespace bsk
