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
//  * q1 runs over x >= y >= 0, z >= 0, each mode weighted by the size of its orbit under
//    sign flips and the x <-> y swap (2^{nonzero components}, times 2 when x != y): applied
//    to all three vectors these map triangles to triangles and keep every membership, since
//    k_c^2 does not change under a sign flip and (kx*kx + ky*ky) is the same sum either
//    way (floating-point addition commutes).  z is not swapped with x or y: it is added last,
//    and at edge ties the rounded sum depends on that order.
//  * For one q1 a CTA sweeps q2 along z-lines (q2_x, q2_y fixed) over the half-lens
//    |q2|^2 <= R2, |q1 + q2|^2 <= R2, |q3| <= |q2|; the half-lens is the set of integer z
//    between bounds that the lanes of a warp compute for 32 lines at once.  The warp then
//    walks those lines as one packed stream of 8-point groups, a group per lane (one 8-byte
//    read of the q2 codes, two of the q3 codes, which run the other way and are read from a
//    z-reversed copy of the table).  Pairs with |q3| < |q2| add 2 to H[y][z], pairs with
//    |q3| = |q2| add 1, so that F(q1; y, z) = (H[y][z] + H[z][y]) / 2; lanes whose points
//    have the same membership codes add their counts with one shared-memory atomic.
//  * After each q1 the CTA folds F into its running sums for the q1's shell run:
//    G[y >= z] += mult * F and W[y >= z] += mult * F * w(q1), w = |q1| in fixed point with
//    kFrac fractional bits, split at bit 22 into two limbs, so every batch sum is an exact
//    integer in uint64 (for |q| < 256: per-mode counts below 2^29 with the orbit weights,
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

// Bits 7, 15, 23, 31 of m (and no others) -> bits 0..3.  The multiplier moves bit 8j + 7 to
// bit 28 + j; every other product term lands outside bits 24..31 (8j - 7k is distinct for
// j, k in 0..3), so no carry reaches them.
__device__ __forceinline__ uint32_t high_bits4(uint32_t m) { return (m * 0x00204081u) >> 28; }

// 0x80 in each byte of x that is zero (the per-byte carry stays inside its byte).
__device__ __forceinline__ uint32_t zero_bytes(uint32_t x) {
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
}

// The warp's 256 points of one iteration of the packed line stream: lane l holds the 8
// consecutive points zg .. zg + 7 of one line, their q2 and q3 codes in the bytes of w2 and
// (w3lo, w3hi), and in8: which of them count (inside the line's z-interval, both codes
// valid).  A run is a maximal stretch of counted points of the stream with equal (code2,
// code3); runs may cross lanes (neighbouring lanes hold neighbouring groups, mostly of one
// line) and even lines, which only merges counts of one (y, z) bin.  The lane holding a
// run's first point adds 2 per point of the run to H with one atomic (pairs with
// |q3| = |q2| are corrected per line by the caller).
__device__ __forceinline__ void count_group(uint32_t* H, int n, int lane, uint32_t in8,
                                            uint2 w2, uint32_t w3lo, uint32_t w3hi) {
  // the previous point of the stream: its two codes and whether it counts
  uint32_t prev = __shfl_up_sync(
      0xFFFFFFFFu, (__byte_perm(w2.y, w3hi, 0x3700) & 0xFFFF0000u) | (in8 >> 7), 1);
  if (lane == 0) prev = 0u;
  // codes shifted by one point: byte i holds point i - 1's code
  const uint32_t p2lo = __funnelshift_l(prev, w2.x, 8), p3lo = __byte_perm(prev, w3lo, 0x6542);
  const uint32_t p2hi = __funnelshift_l(w2.x, w2.y, 8), p3hi = __funnelshift_l(w3lo, w3hi, 8);
  const uint32_t same8 = high_bits4(zero_bytes((w2.x ^ p2lo) | (w3lo ^ p3lo))) |
                         (high_bits4(zero_bytes((w2.y ^ p2hi) | (w3hi ^ p3hi))) << 4);
  const uint32_t prev_in8 = ((in8 << 1) | (prev & 1u)) & 0xFFu;
  const uint32_t st8 = in8 & ~(same8 & prev_in8);  // run starts
  const uint32_t brk = st8 | (~in8 & 0xFFu);       // points where no run continues
  const uint32_t brk_lanes = __ballot_sync(0xFFFFFFFFu, brk != 0u);
  // the end of a run that no later point of this lane ends: the first break of a later
  // lane (position 256 when none)
  const uint32_t later = brk_lanes & (lane == 31 ? 0u : ~((2u << lane) - 1u));
  const int nl = later ? __ffs(later) - 1 : 32;
  const uint32_t nbrk = __shfl_sync(0xFFFFFFFFu, brk, nl & 31);
  const int far_pos = nl < 32 ? 8 * nl + __ffs(nbrk) - 1 : 256;
  uint32_t s8 = st8;
  while (s8) {
    const int j = __ffs(s8) - 1;
    s8 &= s8 - 1;
    const uint32_t after = brk >> (j + 1);
    const int s_pos = 8 * lane + j;
    const int e_pos = after ? s_pos + __ffs(after) : far_pos;
    const uint32_t cnt = 2u * (uint32_t)(e_pos - s_pos);
    const uint32_t c2 = __byte_perm(w2.x, w2.y, j) & 0xFFu;
    const uint32_t c3 = __byte_perm(w3lo, w3hi, j) & 0xFFu;
    if (((c2 | c3) & 0x40u) == 0u)  // both points in one shell: code = 0x80 | shell
      atomicAdd(&H[(int)(c2 * n + c3) - 0x80 * (n + 1)], cnt);
    else
      add_run(H, n, c2, c3, cnt);
  }
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
        // The stream below counts 2 for every pair; the pairs with |q3| = |q2| count once:
        // the point z_eq of an eq_mode 2 line, every point of an eq_mode 1 line (z1 = 0, rare)
        if (eq_mode == 2 && z_eq >= lo && z_eq <= hi) {
          const uint32_t c2 = cube[b2 + z_eq], c3 = cube_rev[b3 + z_eq];
          if (c2 & c3 & 0x80u) add_run(H, n, c2, c3, 0xFFFFFFFFu);
        } else if (eq_mode == 1) {
          for (int z = lo; z <= hi; ++z) {
            const uint32_t c2 = cube[b2 + z], c3 = cube_rev[b3 + z];
            if (c2 & c3 & 0x80u) add_run(H, n, c2, c3, 0xFFFFFFFFu);
          }
        }
        // The block's lines as one stream of 8-point groups: line k (lane k's) has g_k
        // groups from zs_k (zs_k <= lo_k, q2 reads 8-byte aligned); lane l of an iteration
        // takes group t = t0 + l, whose line it finds by a binary search over the inclusive
        // prefix sums of g, and whose points start at zg = base_k + 8 t.
        const int zs = lo - ((b2 + lo) & 7);
        const int g = lo <= hi ? (hi - zs) / 8 + 1 : 0;
        int incl = g;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
          if (lane >= d) incl += v;
        }
        const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const int base = zs - 8 * (incl - g);
        const int a2 = b2 + base, a3 = b3 + base, zlo = lo - base, zhi = hi - base;
        for (int t0 = 0; t0 < total; t0 += 32) {
          const int t = t0 + lane;
          int k = 0;  // the number of lines whose groups all come before t
#pragma unroll
          for (int step = 16; step >= 1; step >>= 1)
            if (__shfl_sync(0xFFFFFFFFu, incl, k + step - 1) <= t) k += step;
          const bool valid = t < total;
          k = min(k, 31);
          const int o = 8 * t;
          const int ka2 = __shfl_sync(0xFFFFFFFFu, a2, k) + o;
          const int ka3 = __shfl_sync(0xFFFFFFFFu, a3, k) + o;
          const int klo = __shfl_sync(0xFFFFFFFFu, zlo, k) - o;
          const int khi = __shfl_sync(0xFFFFFFFFu, zhi, k) - o;
          uint2 w2 = make_uint2(0u, 0u);
          uint32_t w3lo = 0u, w3hi = 0u, in8 = 0u;
          if (valid) {
            w2 = __ldg(reinterpret_cast<const uint2*>(cube + ka2));
            // q3's codes run the other way: read from cube_rev, 16 aligned bytes and funnel
            // shifts by the group's offset
            const int m3 = ka3 & 7;
            const uint2* p3 = reinterpret_cast<const uint2*>(cube_rev + ka3 - m3);
            const uint2 x = __ldg(p3), y = __ldg(p3 + 1);
            const int sh = 8 * (m3 & 3);
            if (m3 < 4) {
              w3lo = __funnelshift_r(x.x, x.y, sh);
              w3hi = __funnelshift_r(x.y, y.x, sh);
            } else {
              w3lo = __funnelshift_r(x.y, y.x, sh);
              w3hi = __funnelshift_r(y.x, y.y, sh);
            }
            // points lo - zg .. hi - zg of the group (the first group starts at most 7 before
            // lo, every group starts at or before hi), with both codes valid
            const int za = max(klo, 0), zb = min(khi, 7);
            const uint32_t ok8 = high_bits4(w2.x & w3lo & 0x80808080u) |
                                 (((w2.y & w3hi & 0x80808080u) * 0x00204081u) >> 24);
            in8 = ok8 & (0xFFu << za) & (0xFFu >> (7 - zb));
          }
          count_group(H, n, lane, in8, w2, w3lo, w3hi);
        }
      }
      __syncthreads();
      // fold F(q1; y, z) = (H[y][z] + H[z][y]) / 2 into the batch sums, weighted by the
      // mode's sign images and its fixed-point |q1|
      const unsigned long long mult = (1ull << ((x1 != 0) + (y1 != 0) + (z1 != 0)))
                                      << (x1 != y1 ? 1 : 0);
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
    for (int y = 0; y <= x; ++y)  // x >= y: the x <-> y swap is a symmetry too
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
  // a mode adds at most 16 * (largest shell count) * 2^30 to a high-limb sum: the batch is
  // short enough that kMaxBatch such terms stay below 2^63
  int64_t max_count = 1;
  for (int64_t c : p->counts) max_count = std::max(max_count, c);
  const size_t batch_len = (size_t)std::max<int64_t>(
      1, std::min<int64_t>(kMaxBatch, (INT64_MAX >> 34) / max_count));
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
