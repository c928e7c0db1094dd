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
//  * For one q1 a CTA sweeps q2 along z-lines (q2_x, q2_y fixed, one line per thread) over
//    the half-lens |q2|^2 <= R2, |q1 + q2|^2 <= R2, |q3| <= |q2|; the half-lens is the set
//    of integer z between bounds computed per line.  Pairs with |q3| < |q2| add 2 to
//    H[y][z], pairs with |q3| = |q2| add 1, so that F(q1; y, z) = (H[y][z] + H[z][y]) / 2.
//    Consecutive points of a line with the same membership codes are summed in a register
//    before their shared-memory atomic.
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

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxShells = 64;                     // tables of at most 64 shells
constexpr int kMaxBatch = 32;                      // octant modes per batch
constexpr int kFrac = 44;                          // fractional bits of the |q| weights
constexpr int kLimb = 22;                          // bits of the low limb

struct Mode {
  int16_t x, y, z;
  uint16_t code;         // first shell | (count - 1) << 8, as the plan's table
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

// Membership code of the integer wavevector q (all |q_c| < Ng / 2) from the plan's
// half-complex table: q and -q share it (the predicate squares the components).
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

__device__ __forceinline__ void add_run(uint32_t* H, int n, uint16_t c2, uint16_t c3,
                                        uint32_t acc) {
  if (!acc || (c2 & 0xFF) == 0xFF || (c3 & 0xFF) == 0xFF) return;
  const int f2 = c2 & 0xFF, e2 = f2 + (c2 >> 8);
  const int f3 = c3 & 0xFF, e3 = f3 + (c3 >> 8);
  for (int y = f2; y <= e2; ++y)
    for (int z = f3; z <= e3; ++z) atomicAdd(&H[y * n + z], acc);
}

// Dynamic shared memory: G, Whi, Wlo (n (n + 1) / 2 uint64 each), then H (n * n uint32).
__global__ void __launch_bounds__(kThreads)
    enum_kernel(const Mode* __restrict__ modes, const Batch* __restrict__ batches, int n_batches,
                int* __restrict__ next_batch, const uint16_t* __restrict__ table, int Ng,
                int R2, int n, unsigned long long* __restrict__ g_cnt,
                double* __restrict__ g_w) {
  extern __shared__ unsigned long long smem_u64[];
  __shared__ int s_batch;
  const int np = n * (n + 1) / 2;
  unsigned long long* G = smem_u64;
  unsigned long long* Whi = G + np;
  unsigned long long* Wlo = Whi + np;
  uint32_t* H = reinterpret_cast<uint32_t*>(Wlo + np);
  const int HN = Ng / 2 + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = isqrt_floor(R2);
  const int side = 2 * r + 1;
  const int lines = side * side;
  auto row_base = [&](int qa, int qb) {  // table offset of (qa, qb, 0)
    const int a = qa < 0 ? qa + Ng : qa;
    const int b = qb < 0 ? qb + Ng : qb;
    return ((int64_t)a * Ng + b) * HN;
  };
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
      // one warp per z-line of q2 = (x2, y2, z), its lanes on 32 consecutive z: the table
      // reads of q2 and q3 are contiguous, and lanes whose (q2, q3) memberships agree add
      // their count with one shared-memory atomic (the lowest lane of each group)
      for (int li = warp; li < lines; li += kWarps) {
        const int x2 = li / side - r, y2 = li % side - r;
        const int t1 = R2 - x2 * x2 - y2 * y2;
        const int x3 = -(x1 + x2), y3 = -(y1 + y2);
        const int t2 = R2 - x3 * x3 - y3 * y3;
        if (t1 < 0 || t2 < 0) continue;  // warp-uniform
        const int r1 = isqrt_floor(t1), r2 = isqrt_floor(t2);
        // |q2|^2 <= R2: |z| <= r1;  |q3|^2 <= R2: |z1 + z| <= r2
        const int lo = max(-r1, -z1 - r2);
        int hi = min(r1, -z1 + r2);
        // |q3|^2 <= |q2|^2  <=>  2 z1 z <= -(n1 + 2 (x1 x2 + y1 y2)) = D
        const int D = -(n1 + 2 * (x1 * x2 + y1 * y2));
        if (z1 == 0) {
          if (D < 0) continue;
        } else {
          const int den = 2 * z1;  // z1 > 0: z <= floor(D / den)
          hi = min(hi, D >= 0 ? D / den : -((-D + den - 1) / den));
        }
        // the one z with |q3| = |q2| (counted once, every other pair twice): 2 z1 z = D
        const int z_eq = (z1 == 0) ? (D == 0 ? INT_MIN + 1 : INT_MIN)
                                   : (D % (2 * z1) == 0 ? D / (2 * z1) : INT_MIN);
        const int64_t b2p = row_base(x2, y2), b2n = row_base(-x2, -y2);
        const int64_t b3p = row_base(x3, y3), b3n = row_base(-x3, -y3);
        for (int z0 = lo; z0 <= hi; z0 += 32) {
          const int z = z0 + lane;
          uint32_t key = 0xFFFFFFFFu;
          if (z <= hi) {
            const int z3 = -(z1 + z);
            const uint32_t c2 = __ldg(table + (z >= 0 ? b2p + z : b2n - z));
            const uint32_t c3 = __ldg(table + (z3 >= 0 ? b3p + z3 : b3n - z3));
            if ((c2 & 0xFF) != 0xFF && (c3 & 0xFF) != 0xFF) key = c2 | (c3 << 16);
          }
          const uint32_t group = __match_any_sync(0xFFFFFFFFu, key);
          if (key != 0xFFFFFFFFu && lane == __ffs(group) - 1) {
            // with z1 == 0 every pair of the half-lens has |q3| = |q2| when D == 0
            uint32_t cnt = 2u * __popc(group);
            if (z1 == 0) {
              if (z_eq == INT_MIN + 1) cnt = __popc(group);
            } else if (z_eq >= z0 && z_eq < z0 + 32 && ((group >> (z_eq - z0)) & 1u)) {
              cnt -= 1u;
            }
            add_run(H, n, (uint16_t)(key & 0xFFFF), (uint16_t)(key >> 16), cnt);
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
    const uint16_t code = modes[bt.begin].code;
    const int f1 = code & 0xFF, e1 = f1 + (code >> 8);
    for (int x = f1; x <= e1; ++x) {
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

// One thread per octant point (x, y, z) in [0, r]^3: its membership code (0x00FF = none).
__global__ void octant_codes_kernel(const uint16_t* __restrict__ table, int Ng, int r, int R2,
                                    uint16_t* __restrict__ out) {
  const int side = r + 1;
  const int64_t total = (int64_t)side * side * side;
  const int HN = Ng / 2 + 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % side);
    const int y = (int)((i / side) % side);
    const int x = (int)(i / ((int64_t)side * side));
    out[i] = x * x + y * y + z * z <= R2 ? code_of(table, Ng, HN, x, y, z) : (uint16_t)0x00FF;
  }
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
  const int64_t T = (int64_t)tri.size();
  using namespace genum;
  BSK_REQUIRE(gridinfo_enum_supported(p), BSK_ERR_STATE, "internal: enumeration unsupported");
  const int r = p->qmax;
  const int R2 = (r + 1) * (r + 1) - 1;  // every shell mode has |q| < qmax + 1
  // octant modes of the plan's shells, sorted by membership run, then batched
  const int side = r + 1;
  const size_t n_oct = (size_t)side * side * side;
  std::vector<uint16_t> codes(n_oct);
  {
    void* d = nullptr;
    BSK_CHECK_CUDA(cudaMallocAsync(&d, n_oct * sizeof(uint16_t), st));
    octant_codes_kernel<<<p->num_sms * 8, 256, 0, st>>>(p->table, p->Ng, r, R2, (uint16_t*)d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(codes.data(), d, n_oct * sizeof(uint16_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(d, st);
    BSK_REQUIRE(e == cudaSuccess, BSK_ERR_CUDA,
                std::string("grid information: octant codes: ") + cudaGetErrorString(e));
  }
  std::vector<Mode> modes;
  for (int x = 0; x <= r; ++x)
    for (int y = 0; y <= r; ++y)
      for (int z = 0; z <= r; ++z) {
        const uint16_t c = codes[((size_t)x * side + y) * side + z];
        if ((c & 0xFF) != 0xFF) {
          const double w = std::sqrt((double)(x * x + y * y + z * z)) * std::ldexp(1.0, kFrac);
          modes.push_back(Mode{(int16_t)x, (int16_t)y, (int16_t)z, c,
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
                                              p->table, p->Ng, R2, n, g_cnt, g_w);
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
