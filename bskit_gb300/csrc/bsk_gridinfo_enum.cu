// Grid information (triangle counts and mean |k| per bin) by exact lattice enumeration.
//
// bskit's measure_gridinfo_faster (bskit/main.py:1941-2132) computes
//   N_tri(a, b, c) = sum_x n_a n_b n_c / N^3,   n_s = c2r[1{q in shell s}]
//   k_mean_a       = sum_x K_a n_b n_c / N^3 / N_tri,   K_s = c2r[|k| 1{q in shell s}]
// in FP64.  When no triangle of shell modes can wrap around the periodic grid (the grid
// side exceeds three times the largest |q_c| of a shell mode, the condition of the plan's
// reduced grid), these sums are exactly
//   N_tri(a, b, c) = #{(q1, q2, q3) : q1 in a, q2 in b, q3 in c, q1 + q2 + q3 = 0}
//   k_mean_a       = k_f * (sum over those triangles of |q1|) / N_tri,
// the "counting triangles" form of the same estimator (bk_binned, main.py:834-1004).  This
// file evaluates that form directly, in integers, with shell membership read from the plan's
// shell table (the FP64 closed-edge predicate of main.py:1848-1852, so edge ties are the
// plan's).  Nothing here uses floating point except the fixed-point |q1| weights, computed
// once per mode, and the final FP64 divide.
//
// Enumeration.  Let F(q1; y, z) = #{q2 in y : -(q1 + q2) in z}.  Then
//   N_tri(x, y, z) = sum_{q1 in x} F(q1; y, z),   S(x; y, z) = sum_{q1 in x} |q1| F(q1; y, z)
// and, by relabelling the triangle, sum |q2| of bin (a, b, c) = S(b; a, c) and sum |q3| =
// S(c; a, b); F is symmetric in (y, z).
//  * q1 runs over one octant (q1 >= 0 componentwise), each mode weighted by its number of
//    sign images (2^{nonzero components}): flipping the sign of a component of all three
//    vectors maps triangles to triangles and keeps every membership (k_c^2 is unchanged).
//  * For one q1 a CTA sweeps q2 along z-lines (q2_x, q2_y fixed) over the half-lens
//    |q2|^2 <= R2, |q1 + q2|^2 <= R2, |q3| <= |q2|; the half-lens is the set of integer z
//    between bounds that the lanes of a warp compute for 32 lines at once.  The warp then
//    walks each line, every lane on 4 consecutive z (one 4-byte read of the q2 codes, two
//    of the q3 codes, which run the other way and are read from a z-reversed copy of the
//    table).  Pairs with |q3| < |q2| add 2 to H[y][z], pairs with |q3| = |q2| add 1, so
//    that F(q1; y, z) = (H[y][z] + H[z][y]) / 2; a lane's consecutive points with the same
//    membership codes are summed before their shared-memory atomic.
//  * After each q1 the CTA folds F into its running sums for the q1's shell run:
//    G[y >= z] += mult * F and W[y >= z] += mult * F * w(q1), w = |q1| in fixed point with
//    kFrac fractional bits, split at bit 22 into two limbs, so every batch sum is an exact
//    integer in uint64 (for |q| < 256: per-mode counts below 2^28 with the sign images,
//    limbs below 2^30 and 2^22, kMaxBatch modes per batch).
//  * A batch is at most kMaxBatch octant modes of one membership run; at its end the CTA adds
//    its counts to the global uint64 table and its |q| sums, converted to FP64, to the
//    global FP64 table (atomics).  Batches are taken from a counter.
// The finish kernel reads, per triangle, N_tri = G[a][b,c], and the three role sums, and
// divides in FP64.
#include <algorithm>
#include <climits>
#include <cmath>

#include "bsk_internal.cuh"

namespace bsk {
namespace genum {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kWin = 2;                            // 128-point windows whose loads overlap
constexpr int kMaxShells = 64;                     // tables of at most 64 shells
constexpr int kMaxBatch = 32;                      // octant modes per batch
constexpr int kFrac = 44;                          // fractional bits of the |q| weights
constexpr int kLimb = 22;                          // bits of the low limb

// Membership of an integer wavevector in one byte: 0 = no shell, else
// 0x80 | (count - 1) << 6 | first shell (count 1 or 2, first < 64).
__host__ __device__ __forceinline__ int code_first(uint32_t c) { return c & 63; }
__host__ __device__ __forceinline__ int code_last(uint32_t c) { return (c & 63) + ((c >> 6) & 1); }

struct Mode {
  int16_t x, y, z;
  uint16_t code;         // the byte code of the mode
  unsigned long long w;  // |q| * 2^kFrac, rounded (host sqrt, correctly rounded)
};
static_assert(sizeof(HostTriangle) == 3 * sizeof(int32_t), "triangles upload as int32 [T][3]");

struct Batch {
  int begin, end;  // [begin, end) in the mode list, one membership run
};

__host__ __device__ __forceinline__ int pair_index(int y, int z) {  // y >= z
  return y * (y + 1) / 2 + z;
}

__device__ __forceinline__ int isqrt_floor(int t) {
  int s = (int)sqrtf((float)t);
  while (s * s > t) --s;
  while ((s + 1) * (s + 1) <= t) ++s;
  return s;
}

// Plan-table code (first | (count - 1) << 8, 0x00FF none) of the integer wavevector q, all
// |q_c| < Ng / 2: q and -q share it (the predicate squares the components).
__device__ __forceinline__ uint16_t code_of(const uint16_t* __restrict__ table, int Ng, int H,
                                            int qa, int qb, int qc) {
  if (qc < 0) {
    qa = -qa;
    qb = -qb;
    qc = -qc;
  }
  const int a = qa < 0 ? qa + Ng : qa;
  const int b = qb < 0 ? qb + Ng : qb;
  return __ldg(table + ((int64_t)a * Ng + b) * H + qc);
}

// Byte codes of the cube [-r, r]^3 (zero outside |q|^2 <= R2); flag[0] is set when a mode
// lies in more than two shells (not representable: the caller falls back).
__global__ void cube_codes_kernel(const uint16_t* __restrict__ table, int Ng, int r, int R2,
                                  uint8_t* __restrict__ cube, uint8_t* __restrict__ cube_rev,
                                  int* __restrict__ flag) {
  const int S = 2 * r + 1;
  const int64_t total = (int64_t)S * S * S;
  const int HN = Ng / 2 + 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % S) - r;
    const int y = (int)((i / S) % S) - r;
    const int x = (int)(i / ((int64_t)S * S)) - r;
    uint8_t out = 0;
    if (x * x + y * y + z * z <= R2) {
      const uint16_t c = code_of(table, Ng, HN, x, y, z);
      const int first = c & 0xFF, extra = c >> 8;
      if (first != 0xFF) {
        if (extra > 1 || first > 63) atomicOr(flag, 1);
        out = (uint8_t)(0x80 | ((extra & 1) << 6) | (first & 63));
      }
    }
    cube[i] = out;
    cube_rev[i + (int64_t)(-2 * z)] = out;  // (x, y, -z): z runs the other way
  }
}

__device__ __forceinline__ void add_run(uint32_t* H, int n, uint32_t c2, uint32_t c3,
                                        uint32_t cnt) {
  for (int y = code_first(c2); y <= code_last(c2); ++y)
    for (int z = code_first(c3); z <= code_last(c3); ++z) atomicAdd(&H[y * n + z], cnt);
}

// Four consecutive points z = zg .. zg + 3 of a line, their q2 and q3 codes in the bytes of
// w2 and w3: runs of equal (code2, code3) add their count (2 per pair, 1 for the pair with
// |q3| = |q2|) to H with one atomic per run (points outside [lo, hi] count nothing).
__device__ __forceinline__ void count_quad(uint32_t* H, int n, int zg, int lo, int hi,
                                           uint32_t w2, uint32_t w3, int eq_mode, int z_eq) {
  uint32_t run = 0, cnt = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int z = zg + j;
    const uint32_t c2 = (w2 >> (8 * j)) & 0xFFu, c3 = (w3 >> (8 * j)) & 0xFFu;
    const uint32_t key = (z >= lo && z <= hi && (c2 & c3 & 0x80u)) ? ((c2 << 8) | c3) : 0u;
    if (key != run) {
      if (run) add_run(H, n, run >> 8, run & 0xFFu, cnt);
      run = key;
      cnt = 0;
    }
    cnt += eq_mode == 1 ? 1u : (eq_mode == 2 && z == z_eq ? 1u : 2u);
  }
  if (run) add_run(H, n, run >> 8, run & 0xFFu, cnt);
}

// Dynamic shared memory: G, Whi, Wlo (n (n + 1) / 2 uint64 each), then H (n * n uint32).
__global__ void __launch_bounds__(kThreads, 2)
    enum_kernel(const Mode* __restrict__ modes, const Batch* __restrict__ batches, int n_batches,
                int* __restrict__ next_batch, const uint8_t* __restrict__ cube,
                const uint8_t* __restrict__ cube_rev, int r, int R2,
                int n, unsigned long long* __restrict__ g_cnt, double* __restrict__ g_w) {
  extern __shared__ unsigned long long smem_u64[];
  __shared__ int s_batch;
  const int np = n * (n + 1) / 2;
  unsigned long long* G = smem_u64;
  unsigned long long* Whi = G + np;
  unsigned long long* Wlo = Whi + np;
  uint32_t* H = reinterpret_cast<uint32_t*>(Wlo + np);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = 2 * r + 1;
  for (int i = threadIdx.x; i < n * n; i += kThreads) H[i] = 0u;
  while (true) {
    __syncthreads();  // the previous batch's flush has read G / W
    if (threadIdx.x == 0) s_batch = atomicAdd(next_batch, 1);
    for (int i = threadIdx.x; i < np; i += kThreads) G[i] = Whi[i] = Wlo[i] = 0ull;
    __syncthreads();
    const int bi = s_batch;
    if (bi >= n_batches) break;
    const Batch bt = batches[bi];
    for (int m = bt.begin; m < bt.end; ++m) {
      const Mode q1 = modes[m];
      const int x1 = q1.x, y1 = q1.y, z1 = q1.z;
      const int n1 = x1 * x1 + y1 * y1 + z1 * z1;
      // lines (x2, y2) with both |q2| <= r and |q1 + q2| <= r possible
      const int xa = max(-r, -r - x1), xb = min(r, r - x1);
      const int ya = max(-r, -r - y1), yb = min(r, r - y1);
      const int ny = yb - ya + 1;
      const int lines = (xb - xa + 1) * ny;
      for (int l0 = warp * 32; l0 < lines; l0 += kWarps * 32) {
        // each lane sets up one line of the block of 32: the z-interval of the half-lens
        //   |q2|^2 <= R2: |z| <= r1;   |q3|^2 <= R2: |z1 + z| <= r2;
        //   |q3|^2 <= |q2|^2  <=>  2 z1 z <= -(n1 + 2 (x1 x2 + y1 y2)) = D
        int lo = 1, hi = 0, b2 = 0, b3 = 0, eq_mode = 0, z_eq = 0;
        const int li = l0 + lane;
        if (li < lines) {
          const int x2 = xa + li / ny, y2 = ya + li % ny;
          const int x3 = -(x1 + x2), y3 = -(y1 + y2);
          const int t1 = R2 - x2 * x2 - y2 * y2;
          const int t2 = R2 - x3 * x3 - y3 * y3;
          if (t1 >= 0 && t2 >= 0) {
            const int r1 = isqrt_floor(t1), r2 = isqrt_floor(t2);
            lo = max(-r1, -z1 - r2);
            hi = min(r1, -z1 + r2);
            const int D = -(n1 + 2 * (x1 * x2 + y1 * y2));
            if (z1 == 0) {
              if (D < 0) hi = lo - 1;
              eq_mode = D == 0 ? 1 : 0;
            } else {
              const int den = 2 * z1;  // z1 > 0: z <= floor(D / den)
              hi = min(hi, D >= 0 ? D / den : -((-D + den - 1) / den));
              if (D % den == 0) {
                eq_mode = 2;
                z_eq = D / den;
              }
            }
            b2 = ((x2 + r) * S + (y2 + r)) * S + r;        // cube index of (x2, y2, z) - z
            b3 = ((x3 + r) * S + (y3 + r)) * S + r + z1;   // cube_rev index of q3 - z
          }
        }
        uint32_t todo = __ballot_sync(0xFFFFFFFFu, lo <= hi);
        while (todo) {
          const int k = __ffs(todo) - 1;
          todo &= todo - 1;
          const int klo = __shfl_sync(0xFFFFFFFFu, lo, k);
          const int khi = __shfl_sync(0xFFFFFFFFu, hi, k);
          const int kb2 = __shfl_sync(0xFFFFFFFFu, b2, k);
          const int kb3 = __shfl_sync(0xFFFFFFFFu, b3, k);
          const int kmode = __shfl_sync(0xFFFFFFFFu, eq_mode, k);
          const int kzeq = __shfl_sync(0xFFFFFFFFu, z_eq, k);
          // lane l takes the 4 points zs + 128 u + 4 l .. + 3; zs makes the q2 reads 4-byte
          // aligned, the q3 reads (the other direction, in cube_rev) are two aligned words
          // and a funnel shift by the line's offset
          const int zs = klo - ((kb2 + klo) & 3);
          const int m3 = (kb3 + zs) & 3;
          for (int z0 = zs; z0 <= khi; z0 += 128 * kWin) {
            uint32_t w2[kWin], w3[kWin];
#pragma unroll
            for (int u = 0; u < kWin; ++u) {
              const int zg = z0 + 128 * u + 4 * lane;
              w2[u] = w3[u] = 0u;
              if (zg <= khi) {
                w2[u] = __ldg(reinterpret_cast<const uint32_t*>(cube + kb2 + zg));
                const uint32_t* p3 = reinterpret_cast<const uint32_t*>(cube_rev + kb3 + zg - m3);
                w3[u] = __funnelshift_r(__ldg(p3), __ldg(p3 + 1), 8 * m3);
              }
            }
#pragma unroll
            for (int u = 0; u < kWin; ++u) {
              const int zg = z0 + 128 * u + 4 * lane;
              if (zg <= khi) count_quad(H, n, zg, klo, khi, w2[u], w3[u], kmode, kzeq);
            }
          }
        }
      }
      __syncthreads();
      // fold F(q1; y, z) = (H[y][z] + H[z][y]) / 2 into the batch sums, weighted by the
      // mode's sign images and its fixed-point |q1|
      const unsigned long long mult = 1ull << ((x1 != 0) + (y1 != 0) + (z1 != 0));
      const unsigned long long w_hi = q1.w >> kLimb, w_lo = q1.w & ((1ull << kLimb) - 1);
      for (int i = threadIdx.x; i < n * n; i += kThreads) {
        const int y = i / n, z = i - y * n;
        if (z > y) continue;
        const unsigned long long f =
            ((unsigned long long)H[y * n + z] + (unsigned long long)H[z * n + y]) >> 1;
        if (f) {
          const int p = pair_index(y, z);
          const unsigned long long fm = f * mult;
          G[p] += fm;
          Whi[p] += fm * w_hi;
          Wlo[p] += fm * w_lo;
        }
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n * n; i += kThreads) H[i] = 0u;
      __syncthreads();
    }
    // add the batch sums to every shell of the batch's membership run
    const uint32_t code = modes[bt.begin].code;
    for (int x = code_first(code); x <= code_last(code); ++x) {
      for (int p = threadIdx.x; p < np; p += kThreads) {
        if (G[p]) {
          const size_t o = (size_t)x * np + p;
          atomicAdd(g_cnt + o, G[p]);
          atomicAdd(g_w + o, (double)Whi[p] * (1.0 / (double)(1ull << (kFrac - kLimb))) +
                                 (double)Wlo[p] * (1.0 / (double)(1ull << kFrac)));
        }
      }
    }
  }
}

size_t enum_smem_bytes(int n) {
  return 3 * sizeof(unsigned long long) * (size_t)(n * (n + 1) / 2) +
         sizeof(uint32_t) * (size_t)n * n;
}

// Per triangle t = (a, b, c): N_tri = G[a][b, c]; k_mean of each role from the role sums.
__global__ void enum_finish_kernel(int64_t T, const int32_t* __restrict__ tri, int n,
                                   const unsigned long long* __restrict__ g_cnt,
                                   const double* __restrict__ g_w, double kf,
                                   double* __restrict__ ntri, double* __restrict__ kmean) {
  const int np = n * (n + 1) / 2;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int s[3] = {tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]};
    auto idx = [&](int x, int y, int z) {
      return (size_t)x * np + (y >= z ? pair_index(y, z) : pair_index(z, y));
    };
    const unsigned long long cnt = g_cnt[idx(s[0], s[1], s[2])];
    ntri[t] = (double)cnt;
    for (int role = 0; role < 3; ++role) {
      const int x = s[role], y = s[(role + 1) % 3], z = s[(role + 2) % 3];
      const size_t o = idx(x, y, z);
      kmean[3 * t + role] = cnt ? g_w[o] / (double)cnt * kf : nan("");
    }
  }
}

}  // namespace genum

// The enumeration counts exactly what the FFT sums give when no triangle of shell modes can
// wrap around the grid (Ng > 3 qmax); its shared-memory tables hold up to 64 shells, and the
// fixed-point |q| sums stay below 2^64 for |q| < 256.
bool gridinfo_enum_supported(const bsk_plan* p) {
  return p->n <= genum::kMaxShells && p->Ng > 3 * p->qmax && p->qmax < 255;
}

void gridinfo_enum(bsk_plan* p, const std::vector<HostTriangle>& tri, double* ntri,
                   double* kmean, cudaStream_t st) {
  using namespace genum;
  const int64_t T = (int64_t)tri.size();
  BSK_REQUIRE(gridinfo_enum_supported(p), BSK_ERR_STATE, "internal: enumeration unsupported");
  const int r = p->qmax;
  const int R2 = (r + 1) * (r + 1) - 1;  // every shell mode has |q| < qmax + 1
  const int S = 2 * r + 1;
  const size_t n_cube = (size_t)S * S * S;
  // byte codes of the cube [-r, r]^3, kept on the device for the enumeration; the octant
  // part is read back to list the q1 modes
  // [pad][cube][pad][cube_rev][pad][flag]: the pads hold the few bytes that the 4-byte reads
  // of a line's first and last points take from before and after the cube
  const size_t pad = 64, span = (n_cube + 15) / 16 * 16;
  char* cube_mem = nullptr;
  BSK_CHECK_CUDA(cudaMallocAsync((void**)&cube_mem, 3 * pad + 2 * span + 16, st));
  struct FreeCube {
    char* w;
    cudaStream_t s;
    ~FreeCube() { cudaFreeAsync(w, s); }
  } free_cube{cube_mem, st};
  BSK_CHECK_CUDA(cudaMemsetAsync(cube_mem, 0, 3 * pad + 2 * span + 16, st));
  uint8_t* d_cube = (uint8_t*)cube_mem + pad;
  uint8_t* d_cube_rev = d_cube + span + pad;
  int* d_flag = (int*)(d_cube_rev + span + pad);
  std::vector<uint8_t> cube(n_cube);
  int flag = 0;
  cube_codes_kernel<<<p->num_sms * 8, 256, 0, st>>>(p->table, p->Ng, r, R2, d_cube, d_cube_rev,
                                                    d_flag);
  BSK_CHECK_CUDA(cudaGetLastError());
  BSK_CHECK_CUDA(cudaMemcpyAsync(cube.data(), d_cube, n_cube, cudaMemcpyDeviceToHost, st));
  BSK_CHECK_CUDA(cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  BSK_CHECK_CUDA(cudaStreamSynchronize(st));
  BSK_REQUIRE(flag == 0, BSK_ERR_STATE, "internal: a mode lies in more than two shells");
  std::vector<Mode> modes;
  for (int x = 0; x <= r; ++x)
    for (int y = 0; y <= r; ++y)
      for (int z = 0; z <= r; ++z) {
        const uint8_t c = cube[((size_t)(x + r) * S + (y + r)) * S + (z + r)];
        if (c & 0x80) {
          const double w = std::sqrt((double)(x * x + y * y + z * z)) * std::ldexp(1.0, kFrac);
          modes.push_back(Mode{(int16_t)x, (int16_t)y, (int16_t)z, (uint16_t)c,
                               (unsigned long long)std::llround(w)});
        }
      }
  std::stable_sort(modes.begin(), modes.end(),
                   [](const Mode& a, const Mode& b) { return a.code < b.code; });
  // a mode adds at most 8 * (largest shell count) * 2^30 to a high-limb sum: the batch is
  // short enough that kMaxBatch such terms stay below 2^63
  int64_t max_count = 1;
  for (int64_t c : p->counts) max_count = std::max(max_count, c);
  const size_t batch_len = (size_t)std::max<int64_t>(
      1, std::min<int64_t>(kMaxBatch, (INT64_MAX >> 33) / max_count));
  std::vector<Batch> batches;
  for (size_t i = 0; i < modes.size();) {
    size_t j = i;
    while (j < modes.size() && modes[j].code == modes[i].code && j - i < batch_len) ++j;
    batches.push_back(Batch{(int)i, (int)j});
    i = j;
  }
  const int n = p->n;
  const size_t np = (size_t)n * (n + 1) / 2;
  const size_t tab = (size_t)n * np;
  const size_t bytes_modes = std::max<size_t>(1, modes.size()) * sizeof(Mode);
  const size_t bytes_batches = std::max<size_t>(1, batches.size()) * sizeof(Batch);
  const size_t bytes_tab = tab * (sizeof(unsigned long long) + sizeof(double));
  const size_t bytes_tri = (size_t)T * 3 * sizeof(int32_t);
  char* work = nullptr;
  BSK_CHECK_CUDA(cudaMallocAsync((void**)&work,
                                 bytes_modes + bytes_batches + bytes_tab + 256 + bytes_tri, st));
  struct Free {
    char* w;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(w, s); }
  } free_work{work, st};
  Mode* d_modes = (Mode*)work;
  Batch* d_batches = (Batch*)(work + bytes_modes);
  unsigned long long* g_cnt = (unsigned long long*)(work + bytes_modes + bytes_batches);
  double* g_w = (double*)(g_cnt + tab);
  int* d_next = (int*)(g_w + tab);
  int32_t* d_tri = (int32_t*)((char*)d_next + 256);
  BSK_CHECK_CUDA(cudaMemsetAsync(g_cnt, 0, bytes_tab + 256, st));
  BSK_CHECK_CUDA(cudaMemcpyAsync(d_tri, tri.data(), bytes_tri, cudaMemcpyHostToDevice, st));
  if (!modes.empty()) {
    BSK_CHECK_CUDA(cudaMemcpyAsync(d_modes, modes.data(), modes.size() * sizeof(Mode),
                                   cudaMemcpyHostToDevice, st));
    BSK_CHECK_CUDA(cudaMemcpyAsync(d_batches, batches.data(), batches.size() * sizeof(Batch),
                                   cudaMemcpyHostToDevice, st));
    const size_t smem = enum_smem_bytes(n);
    BSK_CHECK_CUDA(cudaFuncSetAttribute(enum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    int per_sm = 0;
    BSK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, enum_kernel, kThreads,
                                                                 smem));
    const int grid = std::max(1, std::min<int>((int)batches.size(), per_sm * p->num_sms));
    enum_kernel<<<grid, kThreads, smem, st>>>(d_modes, d_batches, (int)batches.size(), d_next,
                                              d_cube, d_cube_rev, r, R2, n, g_cnt, g_w);
    BSK_CHECK_CUDA(cudaGetLastError());
  }
  const double kf = 2.0 * 3.14159265358979323846 / p->L;
  enum_finish_kernel<<<(int)std::min<int64_t>((T + 255) / 256, 65535), 256, 0, st>>>(
      T, d_tri, n, g_cnt, g_w, kf, ntri, kmean);
  BSK_CHECK_CUDA(cudaGetLastError());
  // the host mode list, batches and triangles must outlive their copies
  BSK_CHECK_CUDA(cudaStreamSynchronize(st));
}

}  // namespace bsk
