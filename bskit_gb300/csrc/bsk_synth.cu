// Shell-field synthesis: I_s(x) = c2r[ dhat_k 1{k in shell s} ] for a batch of shells,
// as three pruned passes of length-Ng inverse FFTs written for this problem.
//
// A shell of radius r occupies |q_a|, |q_b|, q_c <= r of the half spectrum, so:
//   X pass: for every column (q_b, q_c) with |q_b|, q_c <= r, the masked spectrum along
//           q_a (only |q_a| <= r nonzero) -> G[s][x][q_b][q_c]   (reads the slot spectrum
//           and the shell table once for all shells of the batch);
//   Y pass: for every (x, q_c <= r), G along q_b -> Hh[s][x][y][q_c];
//   Z pass: for every two rows (x, y), (x, y+1), the Hermitian-extended sequences along
//           q_c packed as Z1 + i Z2 -> one complex inverse FFT whose real and imaginary
//           parts are the two real output rows; the rows are written as FP32 fields and,
//           when asked, as the bf16 hi / lo planes of the tensor-core contraction.
// Every array keeps q_c fastest, so the passes read and write 8- or 16-wide (64- or 128-byte)
// runs of it.
// The FFTs are radix-16/24/12/8/6/4/2/3/5 Stockham passes in shared memory (twiddles from a
// table computed in double precision on the host); unnormalised, sign +1, as cuFFT's C2R.
#include <atomic>
#include <cmath>

#include "bsk_internal.cuh"

namespace bsk {
namespace {

constexpr int kLines = 16;   // lines (one 16-wide q_c run) per block of the Y pass
constexpr int kXLines = 8;   // X pass: half a q_c run per block (its staged spectrum columns
                             // need shared memory too; 8 lines let three blocks share an SM)
constexpr int kZLines = 16;  // lines (two output rows each) per block of the Z pass
constexpr int kThreads = 256;

__device__ __forceinline__ int fft_freq(int a, int n) { return a < (n + 1) / 2 ? a : a - n; }

__device__ __forceinline__ bool in_shell(uint16_t code, int s) {
  const int first = code & 0xFF;
  const int cnt = (code >> 8) + 1;
  return first != 0xFF && s >= first && s < first + cnt;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by +i
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }

// Unnormalised R-point DFT with sign +1 in registers: v[q] <- sum_r v[r] e^{+2 pi i r q / R}.
// roots[R][k] = e^{+2 pi i k / R}.
__device__ __forceinline__ void dft2(float2* v) {
  const float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
__device__ __forceinline__ void dft4(float2* v) {
  const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
  const float2 s13 = cadd(v[1], v[3]), d13 = mul_i(csub(v[1], v[3]));
  v[0] = cadd(s02, s13);
  v[2] = csub(s02, s13);
  v[1] = cadd(d02, d13);
  v[3] = csub(d02, d13);
}
__device__ __forceinline__ void dft8(float2* v) {
  // two 4-point DFTs of the even and odd samples, combined with e^{+2 pi i k / 8}
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e);
  dft4(o);
  const float h = 0.70710678118654752f;
  const float2 w1 = make_float2(h, h), w3 = make_float2(-h, h);
  const float2 t0 = o[0], t1 = cmul(o[1], w1), t2 = mul_i(o[2]), t3 = cmul(o[3], w3);
  v[0] = cadd(e[0], t0);
  v[4] = csub(e[0], t0);
  v[1] = cadd(e[1], t1);
  v[5] = csub(e[1], t1);
  v[2] = cadd(e[2], t2);
  v[6] = csub(e[2], t2);
  v[3] = cadd(e[3], t3);
  v[7] = csub(e[3], t3);
}
__device__ __forceinline__ void dft16(float2* v) {
  // 16 = 4 x 4: DFT4 over a of v[4a + b], twiddle e^{2 pi i b c / 16}, DFT4 over b
  float2 y[4][4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    float2 t[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
    dft4(t);
#pragma unroll
    for (int c = 0; c < 4; ++c) y[b][c] = t[c];
  }
  const float c1 = 0.92387953251128676f, s1 = 0.38268343236508977f;  // cos, sin(pi/8)
  const float h = 0.70710678118654752f;
  // e^{2 pi i k / 16} for k = b c: k = 1, 2, 3, 4, 6, 9
  y[1][1] = cmul(y[1][1], make_float2(c1, s1));
  y[1][2] = cmul(y[1][2], make_float2(h, h));
  y[1][3] = cmul(y[1][3], make_float2(s1, c1));
  y[2][1] = cmul(y[2][1], make_float2(h, h));
  y[2][2] = mul_i(y[2][2]);
  y[2][3] = cmul(y[2][3], make_float2(-h, h));
  y[3][1] = cmul(y[3][1], make_float2(s1, c1));
  y[3][2] = cmul(y[3][2], make_float2(-h, h));
  y[3][3] = cmul(y[3][3], make_float2(-c1, -s1));
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float2 t[4] = {y[0][c], y[1][c], y[2][c], y[3][c]};
    dft4(t);
#pragma unroll
    for (int d = 0; d < 4; ++d) v[c + 4 * d] = t[d];
  }
}
template <int R>
__device__ __forceinline__ void dft_generic(float2* v, const float2* roots) {
  float2 out[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float2 acc = v[0];
#pragma unroll
    for (int r = 1; r < R; ++r) acc = cadd(acc, cmul(v[r], roots[(r * q) % R]));
    out[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = out[q];
}

struct FftPlan {
  int n;
  int np;
  int radix[8];  // 16, 24, 12, 8, 6, 4, 2, 3 or 5
  float2 root3[3];
  float2 root5[5];
  float2 rootc[24];  // e^{+2 pi i k / Rc} of the plan's composite radix Rc (24, 12 or 6)
};

template <int R>
__device__ __forceinline__ void dft_small(float2* v, const FftPlan& pl) {
  if (R == 8) dft8(v);
  else if (R == 4) dft4(v);
  else if (R == 2) dft2(v);
  else if (R == 3) dft_generic<3>(v, pl.root3);
  else dft_generic<5>(v, pl.root5);
}

// R = R1 R2 point DFT: input r = R2 a + b, output q = c + R1 d:
// X[c + R1 d] = sum_b e^{2 pi i b d / R2} e^{2 pi i b c / R} sum_a v[R2 a + b] e^{2 pi i a c / R1}.
template <int R1, int R2>
__device__ __forceinline__ void dft_comp(float2* v, const FftPlan& pl) {
  float2 y[R2][R1];
#pragma unroll
  for (int b = 0; b < R2; ++b) {
    float2 t[R1];
#pragma unroll
    for (int a = 0; a < R1; ++a) t[a] = v[R2 * a + b];
    dft_small<R1>(t, pl);
#pragma unroll
    for (int c = 0; c < R1; ++c) y[b][c] = b && c ? cmul(t[c], pl.rootc[b * c]) : t[c];
  }
#pragma unroll
  for (int c = 0; c < R1; ++c) {
    float2 t[R2];
#pragma unroll
    for (int b = 0; b < R2; ++b) t[b] = y[b][c];
    dft_small<R2>(t, pl);
#pragma unroll
    for (int d = 0; d < R2; ++d) v[c + R1 * d] = t[d];
  }
}

// Radix plan of a length: 16s, then one of 24 / 12 / 8 / 6 / 4 / 2, then 3s and 5s (constexpr, so that a
// compile-time length gets a fully unrolled pass sequence).
// The p-th radix of a length's plan (0 past the end, -1 when the length does not factor).
__host__ __device__ constexpr int plan_radix(int n, int p) {
  int k = 0;
  while (n % 16 == 0) { n /= 16; if (k++ == p) return 16; }
  const int comp[6] = {24, 12, 8, 6, 4, 2};  // at most one of these, 2^a 3 first
  for (int c : comp)
    if (n % c == 0) { n /= c; if (k++ == p) return c; break; }
  while (n % 3 == 0) { n /= 3; if (k++ == p) return 3; }
  while (n % 5 == 0) { n /= 5; if (k++ == p) return 5; }
  return n == 1 ? 0 : -1;
}
__host__ __device__ constexpr int plan_np(int n) {
  int p = 0;
  while (plan_radix(n, p) > 0) ++p;
  return plan_radix(n, p) == 0 ? p : -1;
}

// Lines are kept in shared memory with a stride of n + 1 complex values, and consecutive
// threads take the same butterfly of consecutive lines: both keep the Stockham reads and
// writes of a warp on distinct banks.
__host__ __device__ constexpr int line_stride(int n) { return n + 1; }

template <int R>
__device__ __forceinline__ void dft_radix(float2* v, const FftPlan& pl) {
  if (R == 16) dft16(v);
  else if (R == 24) dft_comp<8, 3>(v, pl);
  else if (R == 12) dft_comp<4, 3>(v, pl);
  else if (R == 6) dft_comp<2, 3>(v, pl);
  else dft_small<R>(v, pl);
}

// One Stockham pass of radix R over `lines` sequences of length n (src -> dst).  Input
// positions zlo .. zhi are known to be zero: they are neither read nor need to be written
// (the first pass of a pruned transform, whose inputs outside the kept frequencies are zero).
template <int R>
__device__ __forceinline__ void fft_pass(const float2* __restrict__ src, float2* __restrict__ dst,
                                         int lines, int n, int Ns, const float2* __restrict__ tw,
                                         const FftPlan& pl, int zlo = 1 << 30, int zhi = -1) {
  const int m = n / R;
  const int step = n / (Ns * R);
  const int ls = line_stride(n);
  for (int t = threadIdx.x; t < lines * m; t += blockDim.x) {
    const int j = t / lines;
    const int line = t - j * lines;
    const int k = j % Ns;
    const float2* in = src + line * ls;
    float2* o = dst + line * ls;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int q = j + r * m;
      v[r] = (q >= zlo && q <= zhi) ? make_float2(0.f, 0.f) : in[q];
    }
    if (Ns > 1) {  // the first pass has k = 0: unit twiddles
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * k * step]);
    }
    dft_radix<R>(v, pl);
    const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) o[idx + r * Ns] = v[r];
  }
}

// Compile-time length: the pass sequence unrolled, every divisor a constant.
template <int N, int L, int P, int Ns>
__device__ __forceinline__ void run_passes(float2*& src, float2*& dst,
                                           const float2* __restrict__ tw, const FftPlan& pl,
                                           int zlo = 1 << 30, int zhi = -1) {
  if constexpr (P < plan_np(N)) {
    constexpr int R = plan_radix(N, P);
    if (P == 0) fft_pass<R>(src, dst, L, N, Ns, tw, pl, zlo, zhi);
    else fft_pass<R>(src, dst, L, N, Ns, tw, pl);
    __syncthreads();
    float2* t2 = src;
    src = dst;
    dst = t2;
    run_passes<N, L, P + 1, Ns * R>(src, dst, tw, pl);
  }
}

// All passes but the last (the Z pass fuses the last one with its stores).
template <int N, int L, int P, int Ns>
__device__ __forceinline__ void run_passes_but_last(float2*& src, float2*& dst,
                                                    const float2* __restrict__ tw,
                                                    const FftPlan& pl, int zlo = 1 << 30,
                                                    int zhi = -1) {
  if constexpr (P + 1 < plan_np(N)) {
    constexpr int R = plan_radix(N, P);
    if (P == 0) fft_pass<R>(src, dst, L, N, Ns, tw, pl, zlo, zhi);
    else fft_pass<R>(src, dst, L, N, Ns, tw, pl);
    __syncthreads();
    float2* t2 = src;
    src = dst;
    dst = t2;
    run_passes_but_last<N, L, P + 1, Ns * R>(src, dst, tw, pl);
  }
}

// Inverse FFT (sign +1, unnormalised) of L sequences of length n stored with line
// stride n + 1 in `a`; `b` is scratch of the same size.  Returns the buffer holding the
// result.  NC = n at compile time, or 0.
template <int NC, int L>
__device__ float2* fft_lines(float2* a, float2* b, const FftPlan& pl,
                             const float2* __restrict__ tw, int zlo = 1 << 30, int zhi = -1) {
  float2* src = a;
  float2* dst = b;
  if constexpr (NC != 0) {
    run_passes<NC, L, 0, 1>(src, dst, tw, pl, zlo, zhi);
  } else {
    const int n = pl.n;
    int Ns = 1;
    for (int p = 0; p < pl.np; ++p) {
      const int R = pl.radix[p];
      const int zl = p == 0 ? zlo : 1 << 30, zh = p == 0 ? zhi : -1;
      switch (R) {
        case 16: fft_pass<16>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 24: fft_pass<24>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 12: fft_pass<12>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 6: fft_pass<6>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 8: fft_pass<8>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 4: fft_pass<4>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 2: fft_pass<2>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        case 3: fft_pass<3>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
        default: fft_pass<5>(src, dst, L, n, Ns, tw, pl, zl, zh); break;
      }
      __syncthreads();
      float2* t2 = src;
      src = dst;
      dst = t2;
      Ns *= R;
    }
  }
  return src;
}

// Index of the i-th kept frequency of an axis: the `nk` frequencies |q| <= R around 0
// (all n of them when 2R + 1 >= n).
__device__ __forceinline__ int kept_index(int i, int nk, int R, int n) {
  return nk == n ? i : (i - R + n) % n;
}

struct SynthArgs {
  int N, H, R, nk, Cp, s0, ns;
  int out0;                // shell written at fields[0] (and hi/lo[0])
  int fields_from;         // the FP32 field is written for shells s0 + s >= fields_from only
  const float2* spec;      // [a][b][c] slot spectrum
  const uint16_t* table;   // [a][b][c] shell codes
  float2* G;               // [s][x][bk][c]   (c < Cp)
  float2* Hh;              // [s][x][y][c]
  float* fields;           // [shell][N^3], shell index s0 + s
  __nv_bfloat16* split;    // optional chunk-major hi / lo split of split_shells shells
  int split_shells;
  const float2* tw;        // [N] e^{+2 pi i k / N}
};

// X pass: block (bk, c-run).  Spectrum and table columns are read once for all shells.
template <int NC>
__global__ void __launch_bounds__(kThreads) synth_x_kernel(SynthArgs A, FftPlan pl) {
  extern __shared__ float2 sm[];
  const int N = NC ? NC : A.N, nk = A.nk;
  const int ls = line_stride(N);
  float2* buf0 = sm;                       // kXLines lines
  float2* buf1 = buf0 + kXLines * ls;       // kXLines lines
  float2* tw = buf1 + kXLines * ls;         // N
  float2* sS = tw + N;                     // nk * kXLines
  uint16_t* sT = reinterpret_cast<uint16_t*>(sS + nk * kXLines);  // nk * kXLines
  const int bk = blockIdx.x;
  const int c0 = blockIdx.y * kXLines;
  const int b = kept_index(bk, nk, A.R, N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = A.tw[i];
  for (int i = threadIdx.x; i < nk * kXLines; i += blockDim.x) {
    const int ak = i / kXLines, l = i - ak * kXLines;
    const int a = kept_index(ak, nk, A.R, N);
    const int c = c0 + l;
    float2 v = make_float2(0.f, 0.f);
    uint16_t code = 0xFF;
    if (c < A.H && c <= A.R) {
      const int64_t m = ((int64_t)a * N + b) * A.H + c;
      v = A.spec[m];
      code = A.table[m];
    }
    sS[i] = v;
    sT[i] = code;
  }
  __syncthreads();
  // positions R + 1 .. N - R - 1 of a line (|q_a| > R) are zero: not written, not read
  const int zlo = nk == N ? 1 << 30 : A.R + 1, zhi = nk == N ? -1 : N - A.R - 1;
  for (int s = 0; s < A.ns; ++s) {
    for (int i = threadIdx.x; i < kXLines * nk; i += blockDim.x) {
      const int ak = i / kXLines, l = i - ak * kXLines;
      // kept frequency ak sits at position a of line l (frequency index a)
      const int a = kept_index(ak, nk, A.R, N);
      const float2 v = in_shell(sT[ak * kXLines + l], A.s0 + s) ? sS[ak * kXLines + l]
                                                                 : make_float2(0.f, 0.f);
      buf0[l * ls + a] = v;
    }
    __syncthreads();
    const float2* res = fft_lines<NC, kXLines>(buf0, buf1, pl, tw, zlo, zhi);
    // G[s][x][bk][c0 + l]
    float2* g = A.G + (((int64_t)s * N) * nk + bk) * A.Cp + c0;
    for (int i = threadIdx.x; i < kXLines * N; i += blockDim.x) {
      const int x = i / kXLines, l = i - x * kXLines;
      g[(int64_t)x * nk * A.Cp + l] = res[l * ls + x];
    }
    __syncthreads();
  }
}

// The Y and Z passes are persistent: a block walks units (u, u + gridDim.x, ...) and,
// while the FFT of one unit runs, the global loads of its share of the next unit's input
// are already in flight into registers (kYPf / kZPf values per thread; inputs beyond
// that, only possible for the largest shells, are read when the unit starts).
constexpr int kYPf = 16;  // Y pass: kYPf * kThreads / kLines kept q_b per line
constexpr int kZPf = 8;   // Z pass: kZPf * kThreads / kZLines nonzero q_c per line

// Y pass: unit (x, c-run, shell).
template <int NC>
__global__ void __launch_bounds__(kThreads, 2) synth_y_kernel(SynthArgs A, FftPlan pl, int units) {
  extern __shared__ float2 sm[];
  const int N = NC ? NC : A.N, nk = A.nk;
  const int ls = line_stride(N);
  float2* buf0 = sm;
  float2* buf1 = buf0 + kLines * ls;
  float2* tw = buf1 + kLines * ls;
  const int nrun = A.Cp / kLines;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = A.tw[i];
  // thread's inputs: i = threadIdx.x + k kThreads -> (bk = i / kLines, l = i % kLines)
  float2 pre[kYPf];
  auto src = [&](int u) {
    const int s = u / (N * nrun), r = u - s * (N * nrun);
    const int x = r / nrun, c0 = (r - x * nrun) * kLines;
    return A.G + (((int64_t)s * N + x) * nk) * A.Cp + c0;
  };
  auto fetch = [&](int u) {
    const float2* g = src(u);
#pragma unroll
    for (int k = 0; k < kYPf; ++k) {
      const int i = threadIdx.x + k * kThreads;
      const int bk = i / kLines, l = i - bk * kLines;
      pre[k] = bk < nk ? g[(int64_t)bk * A.Cp + l] : make_float2(0.f, 0.f);
    }
  };
  int u = blockIdx.x;
  if (u < units) fetch(u);
  for (; u < units; u += gridDim.x) {
    const float2* g = src(u);
    // kept frequencies (|q_b| <= R, or all) from the prefetch, the rest of the line zero
#pragma unroll
    for (int k = 0; k < kYPf; ++k) {
      const int i = threadIdx.x + k * kThreads;
      const int bk = i / kLines, l = i - bk * kLines;
      if (bk < nk) buf0[l * ls + kept_index(bk, nk, A.R, N)] = pre[k];
    }
    for (int i = threadIdx.x + kYPf * kThreads; i < nk * kLines; i += kThreads) {
      const int bk = i / kLines, l = i - bk * kLines;
      buf0[l * ls + kept_index(bk, nk, A.R, N)] = g[(int64_t)bk * A.Cp + l];
    }
    // positions R + 1 .. N - R - 1 (|q_b| > R) are zero: not written, not read
    __syncthreads();
    if (u + (int)gridDim.x < units) fetch(u + gridDim.x);
    const float2* res = nk < N ? fft_lines<NC, kLines>(buf0, buf1, pl, tw, A.R + 1, N - A.R - 1)
                               : fft_lines<NC, kLines>(buf0, buf1, pl, tw);
    const int s = u / (N * nrun), r = u - s * (N * nrun);
    const int x = r / nrun, c0 = (r - x * nrun) * kLines;
    float2* h = A.Hh + (((int64_t)s * N + x) * N) * A.Cp + c0;
    for (int i = threadIdx.x; i < kLines * N; i += kThreads) {
      const int y = i / kLines, l = i - y * kLines;
      h[(int64_t)y * A.Cp + l] = res[l * ls + y];
    }
    __syncthreads();
  }
}

// Radix of the last pass of a compile-time length, and the size of its twiddle table twl.
template <int NC>
__host__ __device__ constexpr int z_last_radix() { return plan_radix(NC, plan_np(NC) - 1); }
template <int NC>
__host__ __device__ constexpr int z_twl_size() { return NC - NC / z_last_radix<NC>(); }

// Last FFT pass of the Z pass fused with its stores.  Butterfly j of a line yields the
// outputs z = j + M r (M = n / R); lanes j (even) and j + 1 hold z and z + 1, so one
// exchange gives the even lane row y1's pair (z, z + 1) (real parts) and the odd lane row
// y2's (imaginary parts): 8-byte field stores, 4-byte hi / lo stores, 32-byte sectors.
// Consecutive lanes take consecutive j, so the twiddles come from a table twl[(r - 1) M + j]
// = e^{+2 pi i r j / n}: a warp reads consecutive entries (tw[r j] would be r apart, a
// gcd(r, 16)-way bank conflict).
template <int NC>
__device__ __forceinline__ void z_last_pass(const float2* __restrict__ src,
                                            const float2* __restrict__ twl, const FftPlan& pl,
                                            const SynthArgs& A, int sh, int64_t row0, int y0,
                                            bool fp32) {
  constexpr int np = plan_np(NC);
  constexpr int R = z_last_radix<NC>();
  constexpr int M = NC / R;
  static_assert(np >= 2 && M % 2 == 0 && (kZLines * M) % kThreads == 0,
                "the fused last pass wants full warps of line-ordered butterfly pairs");
  constexpr int ls = line_stride(NC);
  for (int t = threadIdx.x; t < kZLines * M; t += kThreads) {
    const int line = t / M, j = t - line * M;
    const float2* in = src + line * ls;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[j + r * M];
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], twl[(r - 1) * M + j]);
    dft_radix<R>(v, pl);
    const bool odd = j & 1;
    const int y = y0 + 2 * line + (odd ? 1 : 0);
    const int64_t K = (int64_t)NC * NC * NC;
    const int64_t o = row0 + (int64_t)y * NC + (j & ~1);  // point index within the shell
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float got = __shfl_xor_sync(0xffffffffu, odd ? v[r].x : v[r].y, 1);
      const float2 f = odd ? make_float2(got, v[r].y) : make_float2(v[r].x, got);
      if (y < NC) {
        const int64_t pt = o + (int64_t)M * r;
        if (fp32) *reinterpret_cast<float2*>(A.fields + (int64_t)sh * K + pt) = f;
        if (A.split) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(f.x, f.y);
          const float2 fb = __bfloat1622float2(h);
          const __nv_bfloat162 lw = __floats2bfloat162_rn(f.x - fb.x, f.y - fb.y);
          *reinterpret_cast<__nv_bfloat162*>(A.split + split_index(0, sh, pt, A.split_shells)) = h;
          *reinterpret_cast<__nv_bfloat162*>(A.split + split_index(1, sh, pt, A.split_shells)) = lw;
        }
      }
    }
  }
}

// Z pass: unit (x, run of 2 kZLines rows y, shell).  Line l packs rows y0 + 2l, y0 + 2l + 1.
template <int NC>
__global__ void __launch_bounds__(kThreads, 2) synth_z_kernel(SynthArgs A, FftPlan pl, int units) {
  extern __shared__ float2 sm[];
  const int N = NC ? NC : A.N;
  const int ls = line_stride(N);
  float2* buf0 = sm;
  float2* buf1 = buf0 + kZLines * ls;
  float2* tw = buf1 + kZLines * ls;
  float2* twl = tw + N;  // the last pass's twiddles (compile-time lengths)
  const int ny = (N + 2 * kZLines - 1) / (2 * kZLines);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = A.tw[i];
  if constexpr (NC != 0) {
    constexpr int M = NC / z_last_radix<NC>();
    for (int i = threadIdx.x; i < z_twl_size<NC>(); i += blockDim.x)
      twl[i] = A.tw[(i / M + 1) * (i % M)];  // r j < R M = n
  }
  const int cn = min(A.R, N / 2) + 1;  // q_c = 0 .. cn - 1 can be nonzero
  // kThreads / kZLines threads per line, q_c strided by that
  constexpr int tpl = kThreads / kZLines;
  const int l = threadIdx.x / tpl, cl = threadIdx.x % tpl;
  float2 p1[kZPf], p2[kZPf];
  auto fetch = [&](int u) {
    const int s = u / (N * ny), r = u - s * (N * ny);
    const int x = r / ny, y1 = (r - x * ny) * 2 * kZLines + 2 * l;
    const float2* h = A.Hh + (((int64_t)s * N + x) * N + y1) * A.Cp;
#pragma unroll
    for (int k = 0; k < kZPf; ++k) {
      const int c = cl + k * tpl;
      p1[k] = (y1 < N && c < cn) ? h[c] : make_float2(0.f, 0.f);
      p2[k] = (y1 + 1 < N && c < cn) ? h[A.Cp + c] : make_float2(0.f, 0.f);
    }
  };
  // line value at q_c = c and its Hermitian partner at N - c
  auto put = [&](float2* line, int c, float2 z1, float2 z2) {
    if (c == 0 || 2 * c == N) {
      line[c] = make_float2(z1.x, z2.x);
    } else {
      line[c] = make_float2(z1.x - z2.y, z1.y + z2.x);       // Z1 + i Z2
      line[N - c] = make_float2(z1.x + z2.y, -z1.y + z2.x);  // conj(Z1) + i conj(Z2)
    }
  };
  int u = blockIdx.x;
  if (u < units) fetch(u);
  for (; u < units; u += gridDim.x) {
    const int s = u / (N * ny), r = u - s * (N * ny);
    const int x = r / ny, y0 = (r - x * ny) * 2 * kZLines;
    const int y1 = y0 + 2 * l;
    float2* line = buf0 + l * ls;
#pragma unroll
    for (int k = 0; k < kZPf; ++k) {
      const int c = cl + k * tpl;
      if (c < cn) put(line, c, p1[k], p2[k]);
    }
    if (cn > kZPf * tpl) {
      const float2* h = A.Hh + (((int64_t)s * N + x) * N + y1) * A.Cp;
      for (int c = cl + kZPf * tpl; c < cn; c += tpl) {
        const float2 z1 = y1 < N ? h[c] : make_float2(0.f, 0.f);
        const float2 z2 = y1 + 1 < N ? h[A.Cp + c] : make_float2(0.f, 0.f);
        put(line, c, z1, z2);
      }
    }
    // positions cn .. N - cn (|q_c| >= cn) are zero: not written, not read
    __syncthreads();
    if (u + (int)gridDim.x < units) fetch(u + gridDim.x);
    const int64_t K = (int64_t)N * N * N;
    const int sh = A.s0 + s - A.out0;  // shell index in the output arrays
    const int64_t row0 = ((int64_t)x * N) * N;
    if constexpr (NC != 0) {
      float2* src = buf0;
      float2* dst = buf1;
      run_passes_but_last<NC, kZLines, 0, 1>(src, dst, tw, pl, cn, N - cn);
      z_last_pass<NC>(src, twl, pl, A, sh, row0, y0, A.s0 + s >= A.fields_from);
    } else {
      const float2* res = fft_lines<NC, kZLines>(buf0, buf1, pl, tw, cn, N - cn);
      // four consecutive z per thread: 16-byte field stores, 8-byte hi / lo stores (N % 4 == 0)
      const int nq = N / 4;
      for (int i = threadIdx.x; i < 2 * kZLines * nq; i += kThreads) {
        const int rr = i / nq, z = (i - rr * nq) * 4;  // output row y0 + rr
        const int y = y0 + rr;
        if (y >= N) continue;
        const float2* w = res + (rr >> 1) * ls + z;
        float4 v;
        if (rr & 1) v = make_float4(w[0].y, w[1].y, w[2].y, w[3].y);
        else v = make_float4(w[0].x, w[1].x, w[2].x, w[3].x);
        const int64_t pt = row0 + (int64_t)y * N + z;
        if (A.s0 + s >= A.fields_from)
          *reinterpret_cast<float4*>(A.fields + (int64_t)sh * K + pt) = v;
        if (A.split) {
          const __nv_bfloat162 h01 = __floats2bfloat162_rn(v.x, v.y);
          const __nv_bfloat162 h23 = __floats2bfloat162_rn(v.z, v.w);
          const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
          const __nv_bfloat162 l01 = __floats2bfloat162_rn(v.x - f01.x, v.y - f01.y);
          const __nv_bfloat162 l23 = __floats2bfloat162_rn(v.z - f23.x, v.w - f23.y);
          uint2 hv, lv;
          hv.x = *reinterpret_cast<const uint32_t*>(&h01);
          hv.y = *reinterpret_cast<const uint32_t*>(&h23);
          lv.x = *reinterpret_cast<const uint32_t*>(&l01);
          lv.y = *reinterpret_cast<const uint32_t*>(&l23);
          *reinterpret_cast<uint2*>(A.split + split_index(0, sh, pt, A.split_shells)) = hv;
          *reinterpret_cast<uint2*>(A.split + split_index(1, sh, pt, A.split_shells)) = lv;
        }
      }
    }
    __syncthreads();
  }
}

template <int NC>
void run_synth(const SynthArgs& A, const FftPlan& pl, int nk, int Cp, int ns, size_t fft_smem,
               size_t x_smem, cudaStream_t st) {
  static std::atomic<bool> attr_done[64];  // zero-initialised: false
  int dev = 0;
  BSK_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !attr_done[dev]) {
    const int maxs = 227 * 1024;
    BSK_CHECK_CUDA(cudaFuncSetAttribute(synth_x_kernel<NC>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
    BSK_CHECK_CUDA(cudaFuncSetAttribute(synth_y_kernel<NC>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
    BSK_CHECK_CUDA(cudaFuncSetAttribute(synth_z_kernel<NC>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
    attr_done[dev] = true;
  }
  const int N = A.N;
  synth_x_kernel<NC><<<dim3(nk, Cp / kXLines), kThreads, x_smem, st>>>(A, pl);
  BSK_CHECK_CUDA(cudaGetLastError());
  // persistent Y and Z passes: as many blocks as are resident at once
  int nsm = 0, by = 0, bz = 0;
  BSK_CHECK_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  size_t z_smem = (2 * (size_t)kZLines * (N + 1) + N) * sizeof(float2);
  if constexpr (NC != 0) z_smem += z_twl_size<NC>() * sizeof(float2);
  BSK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&by, synth_y_kernel<NC>, kThreads,
                                                               fft_smem));
  BSK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bz, synth_z_kernel<NC>, kThreads,
                                                               z_smem));
  const int y_units = N * (Cp / kLines) * ns;
  const int z_units = N * ((N + 2 * kZLines - 1) / (2 * kZLines)) * ns;
  const int y_grid = std::max(1, std::min(y_units, std::max(by, 1) * nsm));
  const int z_grid = std::max(1, std::min(z_units, std::max(bz, 1) * nsm));
  synth_y_kernel<NC><<<y_grid, kThreads, fft_smem, st>>>(A, pl, y_units);
  BSK_CHECK_CUDA(cudaGetLastError());
  synth_z_kernel<NC><<<z_grid, kThreads, z_smem, st>>>(A, pl, z_units);
  BSK_CHECK_CUDA(cudaGetLastError());
}

bool make_plan(int n, FftPlan& pl) {
  pl.n = n;
  pl.np = plan_np(n);
  if (pl.np <= 0 || pl.np > 8) return false;
  int rc = 0;
  for (int p = 0; p < pl.np; ++p) {
    pl.radix[p] = plan_radix(n, p);
    if (pl.radix[p] == 24 || pl.radix[p] == 12 || pl.radix[p] == 6) rc = pl.radix[p];
  }
  for (int k = 0; k < 3; ++k)
    pl.root3[k] = make_float2((float)std::cos(2 * M_PI * k / 3), (float)std::sin(2 * M_PI * k / 3));
  for (int k = 0; k < 5; ++k)
    pl.root5[k] = make_float2((float)std::cos(2 * M_PI * k / 5), (float)std::sin(2 * M_PI * k / 5));
  for (int k = 0; k < 24; ++k)
    pl.rootc[k] = rc ? make_float2((float)std::cos(2 * M_PI * k / rc), (float)std::sin(2 * M_PI * k / rc))
                     : make_float2(1.f, 0.f);
  return true;
}

}  // namespace

bool synth_fast_size(int n) {
  switch (n) {
    case 48: case 96: case 128: case 160: case 192: case 240: case 256: case 288: case 320:
    case 384: case 480:
      return true;
    default:
      return false;
  }
}

bool synth_supported(int n) {
  FftPlan pl;
  return n >= 8 && n <= 512 && n % 4 == 0 && make_plan(n, pl);
}

size_t synth_workspace_bytes(int n, int max_r, int batch) {
  const int nk = std::min(2 * max_r + 1, n);
  const int Cp = (max_r + 1 + kLines - 1) / kLines * kLines;
  return ((size_t)batch * n * nk * Cp + (size_t)batch * n * n * Cp) * sizeof(float2) +
         (size_t)n * sizeof(float2);
}

void synth_init_workspace(int N, void* work) {
  std::vector<float2> htw(N);
  for (int k = 0; k < N; ++k)
    htw[k] = make_float2((float)std::cos(2 * M_PI * k / N), (float)std::sin(2 * M_PI * k / N));
  BSK_CHECK_CUDA(cudaMemcpy(work, htw.data(), N * sizeof(float2), cudaMemcpyHostToDevice));
}

void launch_synth(int N, const cufftComplex* spec, const uint16_t* table, int s0, int ns, int R,
                  void* work, float* fields, __nv_bfloat16* split, int split_shells,
                  cudaStream_t st, int out_s0, int fields_from) {
  FftPlan pl;
  BSK_REQUIRE(make_plan(N, pl), BSK_ERR_UNSUPPORTED, "no FFT plan for this grid size");
  R = std::min(R, N / 2);
  const int nk = std::min(2 * R + 1, N);
  const int Cp = (R + 1 + kLines - 1) / kLines * kLines;
  SynthArgs A;
  A.N = N;
  A.H = N / 2 + 1;
  A.R = R;
  A.nk = nk;
  A.Cp = Cp;
  A.s0 = s0;
  A.ns = ns;
  A.out0 = out_s0;
  A.fields_from = fields_from;
  A.spec = reinterpret_cast<const float2*>(spec);
  A.table = table;
  float2* tw = reinterpret_cast<float2*>(work);
  A.G = tw + N;
  A.Hh = A.G + (size_t)ns * N * nk * Cp;
  A.fields = fields;
  A.split = split;
  A.split_shells = split_shells;
  A.tw = tw;
  const size_t fft_smem = (2 * (size_t)kLines * (N + 1) + N) * sizeof(float2);
  const size_t x_smem = (2 * (size_t)kXLines * (N + 1) + N) * sizeof(float2) +
                        (size_t)nk * kXLines * (sizeof(float2) + sizeof(uint16_t));
  BSK_REQUIRE(x_smem <= 227 * 1024, BSK_ERR_UNSUPPORTED, "grid too large for the field synthesis");
  switch (N) {
    case 48: run_synth<48>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 96: run_synth<96>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 128: run_synth<128>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 160: run_synth<160>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 192: run_synth<192>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 240: run_synth<240>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 256: run_synth<256>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 288: run_synth<288>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 320: run_synth<320>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 384: run_synth<384>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    case 480: run_synth<480>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
    default: run_synth<0>(A, pl, nk, Cp, ns, fft_smem, x_smem, st); break;
  }
}

}  // namespace bsk
