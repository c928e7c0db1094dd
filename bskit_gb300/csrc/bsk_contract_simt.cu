// SIMT triple-product contraction: the plain-FP32 path and the FP64 yardstick.
//
// The FP64 variants (FP32 or FP64 fields, FP64 products and sums):
// Work item = (sub-tile of 128 pair rows x 32 third-shell columns, K slice).
// Per 32-point chunk the block forms the 128 pair products P[r][x] =
// F1[i_r](x) * F2[j_r](x) and the 32 column values F3[l](x) in shared memory
// (double buffered, register prefetch of the next chunk), then a 4x4
// register-tiled outer-product loop accumulates C[r][c] += P[r][x] * F3[c][x].
// At the end of the slice the tile sums are added to the FP64 output with
// atomics (only entries that are triangle bins); warps whose 16 x 32 entries hold
// no bin skip the multiply-adds.  Items are ordered slice-major
// so that blocks running at the same time share field data in L2.
#include "bsk_internal.cuh"

namespace bsk {
namespace {

constexpr int KC = 32;     // points per chunk
constexpr int ROWS = 128;  // pair rows per sub-tile
constexpr int COLS = 32;   // columns per sub-tile
constexpr int APAD = 4;
constexpr int BPAD = 4;
constexpr int THREADS = 256;

template <typename Tin, typename Tacc>
__device__ __forceinline__ Tacc prod(Tin a, Tin b) {
  return (Tacc)a * (Tacc)b;
}

template <typename Tin, typename Tacc>
__global__ void __launch_bounds__(THREADS) contract_simt_kernel(
    const TileDesc* __restrict__ tiles, const int2* __restrict__ subs, int n_sub,
    const int16_t* __restrict__ row_i, const int16_t* __restrict__ row_j,
    const int32_t* __restrict__ map, const Tin* __restrict__ f1, const Tin* __restrict__ f2,
    const Tin* __restrict__ f3, int n_shells, int64_t K, int64_t k_begin, int64_t k_end,
    int64_t slice, int64_t n_slices, double* __restrict__ out, double scale) {
  extern __shared__ __align__(16) unsigned char simt_smem[];
  typedef Tacc ATile[KC][ROWS + APAD];
  typedef Tacc BTile[KC][COLS + BPAD];
  ATile* As = reinterpret_cast<ATile*>(simt_smem);
  BTile* Bs = reinterpret_cast<BTile*>(simt_smem + 2 * sizeof(ATile));
  const int tid = threadIdx.x;
  const int tx = tid & 7, ty = tid >> 3;          // micro-tile rows ty*4.., cols tx*4..
  const int ar = tid & (ROWS - 1), ah = tid >> 7;  // A-gen: row ar, points ah*16 .. +16
  const int bc = tid >> 3, bp = (tid & 7) * 4;     // B-gen: column bc, points bp .. +4
  const int64_t n_items = (int64_t)n_sub * n_slices;

  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int64_t sl = item / n_sub;
    const int2 sub = subs[item % n_sub];
    const TileDesc td = tiles[sub.x];
    const int c0 = sub.y;
    const int ri = row_i[td.row_off + ar];
    const int rj = row_j[td.row_off + ar];
    const int lcol = td.l0 + c0 + bc;
    const bool bvalid = (c0 + bc < td.nc) && (lcol < n_shells);
    const Tin* pa = f1 + (int64_t)(ri >= 0 ? ri : 0) * K;
    const Tin* pb = f2 + (int64_t)(ri >= 0 ? rj : 0) * K;
    const Tin* pc = f3 + (int64_t)(bvalid ? lcol : 0) * K;
    const int64_t x_begin = k_begin + sl * slice;
    const int64_t x_end = min(k_end, x_begin + slice);

    Tacc acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = (Tacc)0;
    // A warp (16 rows x 32 columns) whose entries hold no triangle bin skips the
    // multiply-adds; it still loads its share of the tiles the whole block uses.
    bool mine = false;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = c0 + tx * 4 + q;
        if (c < td.nc && map[td.map_off + c * ROWS + ty * 4 + p] >= 0) mine = true;
      }
    const bool warp_busy = __any_sync(0xffffffffu, mine);

    Tacc ra[16], rc[4];
    auto load = [&](int64_t x0) {
      const int64_t xa = x0 + ah * 16;
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        int64_t x = xa + e;
        ra[e] = (ri >= 0 && x < x_end) ? prod<Tin, Tacc>(__ldg(pa + x), __ldg(pb + x)) : (Tacc)0;
      }
      const int64_t xc = x0 + bp;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        int64_t x = xc + e;
        rc[e] = (bvalid && x < x_end) ? (Tacc)__ldg(pc + x) : (Tacc)0;
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int e = 0; e < 16; ++e) As[buf][ah * 16 + e][ar] = ra[e];
#pragma unroll
      for (int e = 0; e < 4; ++e) Bs[buf][bp + e][bc] = rc[e];
    };

    load(x_begin);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int64_t x0 = x_begin; x0 < x_end; x0 += KC) {
      const bool more = x0 + KC < x_end;
      if (more) load(x0 + KC);
#pragma unroll 8
      for (int k = 0; k < KC && warp_busy; ++k) {
        Tacc a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          a[q] = As[buf][k][ty * 4 + q];
          b[q] = Bs[buf][k][tx * 4 + q];
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p][q] += a[p] * b[q];
      }
      if (more) store(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }

#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int r = ty * 4 + p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = c0 + tx * 4 + q;
        if (c < td.nc) {
          const int t = map[td.map_off + c * ROWS + r];
          if (t >= 0) atomicAdd(out + t, (double)acc[p][q] * scale);
        }
      }
    }
  }
}

// ---------------------------------------------------------------- plain FP32 path
// Work item = (tile of 128 pair rows x up to 64 column shells, 8192-point slice).  Per
// 32-point chunk the block copies the tile's source rows (coalesced) and its column rows
// into shared memory, forms the 128 x 32 pair products P = F1_i F2_j there, and each warp
// runs a 32-row x 32-column block of the outer product, 8 rows x 4 columns per thread
// (two 16-byte loads of P and one of F3 per 32 FMAs).  Warps whose 32 columns lie past the
// tile's nc skip their multiply-adds.  FP32 sums over the slice, FP64 atomics across slices.
namespace f32 {
// The plain-FP32 path: work item = (tile of 128 pair rows x nc <= 64 columns, 8192-point
// slice), one block of 128 threads.  Per 32-point chunk the block forms the 128 x 32 pair
// products once in shared memory and runs a register-tiled outer product
// C[r][c] += P[r][x] F3[c][x]; each thread holds 8 rows x CB columns, CB = 4, 6 or 8 chosen
// per tile (tile widths 32, 48, 64).  The operand loads of the outer product, not the
// multiply-adds, bound this kernel: a warp's 128-bit shared-memory load costs four wavefronts
// whatever its broadcast, so the 8 x 8 thread tile (16 values loaded per 64 multiply-adds)
// is what raises the arithmetic per wavefront.  The next chunk's source and column rows are
// copied global -> shared with cp.async into the other half of a double buffer while the
// current chunk is computed.
constexpr int KC = 32;
constexpr int THREADS = 128;
constexpr int ROWS = 128, COLS = 64, SRC = 64;
constexpr int APITCH = ROWS + 4;    // A[x][r]
constexpr int BPITCH = COLS + 4;    // B[x][c]
constexpr int SPITCH = KC + 1;      // S[row][x]
constexpr int64_t SLICE = 8192;
constexpr int STAGE = SRC * KC / THREADS;  // values per thread and array of one chunk (16)
static_assert(COLS == SRC, "one staging pattern for sources and columns");

struct Smem {
  float A[KC][APITCH];
  float B[2][KC][BPITCH];
  float S1[2][SRC][SPITCH];
  float S2[2][SRC][SPITCH];
};

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool ok) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src),
               "r"(ok ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The outer product of one chunk: thread rows r0 .. r0 + 7, columns c0 .. c0 + CB - 1.
template <int CB>
__device__ __forceinline__ void fma_chunk(const float (&A)[KC][APITCH],
                                          const float (&B)[KC][BPITCH], int r0, int c0,
                                          float (&acc)[8][8]) {
#pragma unroll 4
  for (int k = 0; k < KC; ++k) {
    const float4 a0 = *reinterpret_cast<const float4*>(&A[k][r0]);
    const float4 a1 = *reinterpret_cast<const float4*>(&A[k][r0 + 4]);
    const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
    float bv[8];
    if (CB == 8) {
      const float4 b0 = *reinterpret_cast<const float4*>(&B[k][c0]);
      const float4 b1 = *reinterpret_cast<const float4*>(&B[k][c0 + 4]);
      bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
      bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
    } else if (CB == 6) {  // c0 = 6 m: 8-byte aligned
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float2 b = *reinterpret_cast<const float2*>(&B[k][c0 + 2 * q]);
        bv[2 * q] = b.x;
        bv[2 * q + 1] = b.y;
      }
      bv[6] = bv[7] = 0.f;
    } else {
      const float4 b0 = *reinterpret_cast<const float4*>(&B[k][c0]);
      bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
      bv[4] = bv[5] = bv[6] = bv[7] = 0.f;
    }
#pragma unroll
    for (int p = 0; p < 8; ++p)
#pragma unroll
      for (int q = 0; q < CB; ++q) acc[p][q] = fmaf(av[p], bv[q], acc[p][q]);
  }
}

template <int CB>
__device__ __forceinline__ void run_item(Smem& sm, const TileDesc& td, const int16_t* row_i,
                                         const int16_t* row_j, const int32_t* map,
                                         const float* f1, const float* f2, const float* f3,
                                         int n_shells, int64_t K, int64_t x_begin, int64_t x_end,
                                         bool one_src, double* out, double scale) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // outer-product block of this warp: rows [32 warp, +32), all 8 CB columns
  const int r0 = 32 * warp + 8 * (lane >> 3);
  const int c0 = CB * (lane & 7);
  // pair-product formation: row tid, all points of the chunk
  const int ri = row_i[td.row_off + tid], rj = row_j[td.row_off + tid];
  const int pi = ri >= 0 ? ri - td.i0 : -1, pj = ri >= 0 ? rj - td.j0 : -1;
  // staging: value k of a thread is row (tid >> 5) + 4 k, point tid & 31 of the chunk
  const int sx = tid & 31, srow = tid >> 5;
  auto stage = [&](int buf, int64_t x0) {
    const bool xin = x0 + sx < x_end;
#pragma unroll
    for (int k = 0; k < STAGE; ++k) {
      const int row = srow + 4 * k;
      const int s1 = td.i0 + row, s2 = td.j0 + row, l = td.l0 + row;
      const bool ok1 = row < td.ni && s1 < n_shells && xin;
      cp_async4(&sm.S1[buf][row][sx], f1 + (ok1 ? (int64_t)s1 * K + x0 + sx : 0), ok1);
      if (!one_src) {
        const bool ok2 = row < td.nj && s2 < n_shells && xin;
        cp_async4(&sm.S2[buf][row][sx], f2 + (ok2 ? (int64_t)s2 * K + x0 + sx : 0), ok2);
      }
      const bool okb = row < td.nc && l < n_shells && xin;
      cp_async4(&sm.B[buf][sx][row], f3 + (okb ? (int64_t)l * K + x0 + sx : 0), okb);
    }
    cp_async_commit();
  };
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
  stage(0, x_begin);
  int buf = 0;
  for (int64_t x0 = x_begin; x0 < x_end; x0 += KC) {
    if (x0 + KC < x_end) {
      stage(buf ^ 1, x0 + KC);
      cp_async_wait<1>();  // this chunk's copies are complete, the next chunk's in flight
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    {
      const float(*S1)[SPITCH] = sm.S1[buf];
      const float(*S2)[SPITCH] = one_src ? sm.S1[buf] : sm.S2[buf];
#pragma unroll 8
      for (int xx = 0; xx < KC; ++xx) sm.A[xx][tid] = pi >= 0 ? S1[pi][xx] * S2[pj][xx] : 0.f;
    }
    __syncthreads();
    fma_chunk<CB>(sm.A, sm.B[buf], r0, c0, acc);
    __syncthreads();  // A and this buffer are rewritten next
    buf ^= 1;
  }
#pragma unroll
  for (int p = 0; p < 8; ++p) {
#pragma unroll
    for (int q = 0; q < CB; ++q) {
      const int c = c0 + q;
      if (c < td.nc) {
        const int t = __ldg(map + td.map_off + c * kTileRows + r0 + p);
        if (t >= 0) atomicAdd(out + t, (double)acc[p][q] * scale);
      }
    }
  }
}

__global__ void __launch_bounds__(THREADS, 3)
    contract_f32_kernel(const TileDesc* __restrict__ tiles, int n_tiles,
                        const int16_t* __restrict__ row_i, const int16_t* __restrict__ row_j,
                        const int32_t* __restrict__ map, const float* __restrict__ f1,
                        const float* __restrict__ f2, const float* __restrict__ f3,
                        int n_shells, int64_t K, int64_t k_begin, int64_t k_end,
                        int64_t n_slices, double* __restrict__ out, double scale) {
  extern __shared__ __align__(16) unsigned char f32_smem[];
  Smem& sm = *reinterpret_cast<Smem*>(f32_smem);
  const int64_t n_items = (int64_t)n_tiles * n_slices;
  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int64_t sl = item / n_tiles;
    const TileDesc td = tiles[item % n_tiles];
    const bool one_src = f1 == f2 && td.i0 == td.j0;
    const int64_t x_begin = k_begin + sl * SLICE;
    const int64_t x_end = min(k_end, x_begin + SLICE);
    if (td.nc <= 32)
      run_item<4>(sm, td, row_i, row_j, map, f1, f2, f3, n_shells, K, x_begin, x_end, one_src, out, scale);
    else if (td.nc <= 48)
      run_item<6>(sm, td, row_i, row_j, map, f1, f2, f3, n_shells, K, x_begin, x_end, one_src, out, scale);
    else
      run_item<8>(sm, td, row_i, row_j, map, f1, f2, f3, n_shells, K, x_begin, x_end, one_src, out, scale);
  }
}
}  // namespace f32

template <typename Tin, typename Tacc>
void launch_simt(const DeviceSchedule& s, const Tin* f1, const Tin* f2, const Tin* f3,
                 int n_shells, int64_t K, int64_t k_begin, int64_t k_end, int64_t slice,
                 double* out, int num_sms, cudaStream_t st, double scale) {
  if (s.n_sub == 0 || k_end <= k_begin) return;
  const size_t smem = 2 * sizeof(Tacc) * KC * ((ROWS + APAD) + (COLS + BPAD));
  BSK_CHECK_CUDA(cudaFuncSetAttribute(contract_simt_kernel<Tin, Tacc>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  BSK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, contract_simt_kernel<Tin, Tacc>, THREADS, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t n_slices = (k_end - k_begin + slice - 1) / slice;
  const int64_t n_items = n_slices * s.n_sub;
  int64_t grid = (int64_t)num_sms * per_sm;
  if (grid > n_items) grid = n_items;
  contract_simt_kernel<Tin, Tacc><<<(unsigned)grid, THREADS, smem, st>>>(
      s.tiles, s.subs, s.n_sub, s.row_i, s.row_j, s.map, f1, f2, f3, n_shells, K, k_begin, k_end,
      slice, n_slices, out, scale);
  BSK_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

// FP32 products and tile sums (8192-point slices), FP64 cross-slice sum.
void launch_contract_simt_f32(const DeviceSchedule& s, const float* f1, const float* f2,
                              const float* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale) {
  if (s.n_tiles == 0 || k_end <= k_begin) return;
  const size_t smem = sizeof(f32::Smem);
  BSK_CHECK_CUDA(cudaFuncSetAttribute(f32::contract_f32_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  BSK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, f32::contract_f32_kernel, f32::THREADS, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t n_slices = (k_end - k_begin + f32::SLICE - 1) / f32::SLICE;
  const int64_t n_items = n_slices * s.n_tiles;
  int64_t grid = (int64_t)num_sms * per_sm;
  if (grid > n_items) grid = n_items;
  f32::contract_f32_kernel<<<(unsigned)grid, f32::THREADS, smem, st>>>(
      s.tiles, s.n_tiles, s.row_i, s.row_j, s.map, f1, f2, f3, n_shells, K, k_begin, k_end,
      n_slices, out, scale);
  BSK_CHECK_CUDA(cudaGetLastError());
}

// FP64 products and sums of FP32 fields (the yardstick of the precision study).
void launch_contract_simt_f64(const DeviceSchedule& s, const float* f1, const float* f2,
                              const float* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale) {
  launch_simt<float, double>(s, f1, f2, f3, n_shells, K, k_begin, k_end, 65536, out, num_sms, st,
                             scale);
}

// FP64 fields (grid information).
void launch_contract_simt_d64(const DeviceSchedule& s, const double* f1, const double* f2,
                              const double* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale) {
  launch_simt<double, double>(s, f1, f2, f3, n_shells, K, k_begin, k_end, 65536, out, num_sms, st,
                              scale);
}

}  // namespace bsk
