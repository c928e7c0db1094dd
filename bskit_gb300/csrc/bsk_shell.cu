// Shell membership table, spectrum extraction, shell filter and small
// elementwise kernels.
//
// Every kernel here is HBM-bound: one pass over the half-complex spectrum
// (or a field), 16-byte vector accesses, grid sized from the SM count.
#include "bsk_internal.cuh"

namespace bsk {
namespace {

__device__ __forceinline__ int fft_freq(int a, int n) { return a < (n + 1) / 2 ? a : a - n; }

// |k| of integer frequency (qa, qb, qc) exactly as sqrt((kx*kx + ky*ky) + kz*kz)
// with k = q * kf, every operation correctly rounded (no FMA contraction).
__device__ __forceinline__ double mode_kk(int qa, int qb, int qc, double kf) {
  double kx = __dmul_rn((double)qa, kf);
  double ky = __dmul_rn((double)qb, kf);
  double kz = __dmul_rn((double)qc, kf);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
  return __dsqrt_rn(s);
}

// One thread per half-complex mode of the Ng grid.  code = first shell | (count-1) << 8,
// 0x00FF when the mode is in no shell.  Counts are weighted by the number of full-grid
// modes the half-complex entry stands for.
__global__ void shell_table_kernel(int Ng, int reduced, double kf, int n,
                                   const double* __restrict__ edges, uint16_t* __restrict__ table,
                                   unsigned long long* __restrict__ counts, int* __restrict__ flag) {
  extern __shared__ unsigned long long s_counts[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_counts[i] = 0ull;
  __syncthreads();
  const int H = Ng / 2 + 1;
  const int64_t Mh = (int64_t)Ng * Ng * H;
  int local_qmax = 0;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < Mh;
       m += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(m % H);
    int64_t r = m / H;
    int b = (int)(r % Ng);
    int a = (int)(r / Ng);
    int qa = fft_freq(a, Ng), qb = fft_freq(b, Ng), qc = c;
    uint16_t code = 0x00FF;
    bool nyq = reduced && ((Ng % 2 == 0) && (qa == -Ng / 2 || qb == -Ng / 2 || qc == Ng / 2));
    if (!nyq) {
      double kk = mode_kk(qa, qb, qc, kf);
      int first = -1, last = -1, cnt = 0;
      for (int i = 0; i < n; ++i) {
        if (kk <= edges[2 * i + 1] && kk >= edges[2 * i]) {
          if (first < 0) first = i;
          last = i;
          ++cnt;
        }
      }
      if (cnt > 0) {
        if (last - first + 1 != cnt || first > 254) atomicOr(flag, 1);
        code = (uint16_t)(first | ((cnt - 1) << 8));
        unsigned long long w = (qc == 0 || (Ng % 2 == 0 && qc == Ng / 2)) ? 1ull : 2ull;
        for (int i = first; i <= last; ++i) atomicAdd(&s_counts[i], w);
        int aq = max(abs(qa), max(abs(qb), qc));
        local_qmax = max(local_qmax, aq);
      }
    }
    table[m] = code;
  }
  if (local_qmax > 0) atomicMax(flag + 1, local_qmax);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (s_counts[i]) atomicAdd(&counts[i], s_counts[i]);
}

// coarse[a][b][c] = fine[qa mod N][qb mod N][c] / N^3 for modes strictly below the coarse
// Nyquist frequency; zero elsewhere.  When Ng == N it is a scaled copy.
// Optional window compensation: per-axis factor table w[q + N/2], the mode's value
// is multiplied by w[qa] w[qb] w[qc].
__global__ void extract_kernel(int N, int Ng, float scale, const float2* __restrict__ fine,
                               float2* __restrict__ coarse, const float* __restrict__ axis_w) {
  const int H = Ng / 2 + 1, HN = N / 2 + 1;
  const int64_t Mh = (int64_t)Ng * Ng * H;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < Mh;
       m += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(m % H);
    int64_t r = m / H;
    int b = (int)(r % Ng);
    int a = (int)(r / Ng);
    float2 v = make_float2(0.f, 0.f);
    const int qa = fft_freq(a, Ng), qb = fft_freq(b, Ng);
    float f = scale;
    if (axis_w) f *= axis_w[qa + N / 2] * axis_w[qb + N / 2] * axis_w[c + N / 2];
    if (Ng == N) {
      v = fine[m];
      v.x *= f;
      v.y *= f;
    } else {
      bool nyq = (Ng % 2 == 0) && (qa == -Ng / 2 || qb == -Ng / 2 || c == Ng / 2);
      if (!nyq) {
        int fa = qa < 0 ? qa + N : qa;
        int fb = qb < 0 ? qb + N : qb;
        v = fine[((int64_t)fa * N + fb) * HN + c];
        v.x *= f;
        v.y *= f;
      }
    }
    coarse[m] = v;
  }
}

// spec[m] *= scale * w[qa] w[qb] w[qc] over an N^3 half spectrum (N/2+1 last axis).
__global__ void window_kernel(int N, float scale, float2* __restrict__ spec,
                              const float* __restrict__ axis_w) {
  const int H = N / 2 + 1;
  const int64_t Mh = (int64_t)N * N * H;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < Mh;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(m % H);
    const int64_t r = m / H;
    const int qb = fft_freq((int)(r % N), N), qa = fft_freq((int)(r / N), N);
    const float f = scale * axis_w[qa + N / 2] * axis_w[qb + N / 2] * axis_w[c + N / 2];
    float2 v = spec[m];
    v.x *= f;
    v.y *= f;
    spec[m] = v;
  }
}

__device__ __forceinline__ bool in_shell(uint16_t code, int s) {
  int first = code & 0xFF;
  int cnt = (code >> 8) + 1;
  return first != 0xFF && s >= first && s < first + cnt;
}

// out[s][m] = spec[m] if mode m is in shell s0+s else 0.  Two modes per thread (16 B).
__global__ void filter_kernel(int64_t Mh, const float4* __restrict__ spec,
                              const uint32_t* __restrict__ table2, int s0, int ns,
                              float4* __restrict__ out) {
  const int64_t M2 = Mh / 2;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < M2;
       m += (int64_t)gridDim.x * blockDim.x) {
    float4 v = __ldg(spec + m);
    uint32_t codes = __ldg(table2 + m);
    uint16_t c0 = (uint16_t)(codes & 0xFFFF), c1 = (uint16_t)(codes >> 16);
    for (int s = 0; s < ns; ++s) {
      float4 o;
      bool k0 = in_shell(c0, s0 + s), k1 = in_shell(c1, s0 + s);
      o.x = k0 ? v.x : 0.f;
      o.y = k0 ? v.y : 0.f;
      o.z = k1 ? v.z : 0.f;
      o.w = k1 ? v.w : 0.f;
      __stcs(out + (int64_t)s * M2 + m, o);
    }
  }
}

// Indicator (kweight == 0) or |k|-weighted (kweight == 1) spectra, complex128.
__global__ void filter_indicator_kernel(int Ng, double kf, const uint16_t* __restrict__ table,
                                        int s0, int ns, int kweight,
                                        double2* __restrict__ out) {
  const int H = Ng / 2 + 1;
  const int64_t Mh = (int64_t)Ng * Ng * H;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < Mh;
       m += (int64_t)gridDim.x * blockDim.x) {
    uint16_t code = table[m];
    double val = 0.0;
    if ((code & 0xFF) != 0xFF) {
      if (kweight) {
        int c = (int)(m % H);
        int64_t r = m / H;
        int b = (int)(r % Ng);
        int a = (int)(r / Ng);
        val = mode_kk(fft_freq(a, Ng), fft_freq(b, Ng), c, kf);
      } else {
        val = 1.0;
      }
    }
    for (int s = 0; s < ns; ++s) {
      double v = in_shell(code, s0 + s) ? val : 0.0;
      out[(int64_t)s * Mh + m] = make_double2(v, 0.0);
    }
  }
}

// FP32 fields [S][K] -> their chunk-major bf16 hi / lo split (split_index), hi = bf16_rn(v),
// lo = bf16_rn(v - hi); 4 points per thread (K % 4 == 0, so a quad never straddles a
// 128-point chunk); the points K .. 128 ceil(K / 128) of the last chunk are written as zeros.
__global__ void split_kernel(const float4* __restrict__ in, __nv_bfloat16* __restrict__ split,
                             int S, int64_t K, int64_t quads_per_shell) {
  const int64_t n = (int64_t)S * quads_per_shell;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / quads_per_shell);
    const int64_t x = (i - (int64_t)s * quads_per_shell) * 4;
    const float4 v = x < K ? __ldg(in + ((int64_t)s * K + x) / 4) : make_float4(0.f, 0.f, 0.f, 0.f);
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
    *reinterpret_cast<uint2*>(split + split_index(0, s, x, S)) = hv;
    *reinterpret_cast<uint2*>(split + split_index(1, s, x, S)) = lv;
  }
}

__global__ void scale_kernel(double* v, int64_t n, double s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= s;
}

__global__ void gridinfo_finish_kernel(int64_t T, double inv_k, double* ntri, const double* s1,
                                       const double* s2, const double* s3, double* kmean) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (int64_t)gridDim.x * blockDim.x) {
    double nt = rint(ntri[t] * inv_k);
    ntri[t] = nt;
    double nan = __longlong_as_double(0x7ff8000000000000ll);
    kmean[3 * t + 0] = nt != 0.0 ? s1[t] * inv_k / nt : nan;
    kmean[3 * t + 1] = nt != 0.0 ? s2[t] * inv_k / nt : nan;
    kmean[3 * t + 2] = nt != 0.0 ? s3[t] * inv_k / nt : nan;
  }
}

__global__ void normalize_kernel(int64_t n, const double* b, const double* ntri, double* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = b[i] / ntri[i];
}

inline int grid_for(int64_t work, int threads, int max_blocks) {
  int64_t b = (work + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

}  // namespace

void launch_shell_table(const bsk_plan* p, unsigned long long* d_counts, int* d_flag,
                        cudaStream_t st) {
  double kf = 2.0 * 3.14159265358979323846 / p->L;
  int reduced = p->Ng != p->N;
  size_t shm = sizeof(unsigned long long) * (size_t)p->n;
  shell_table_kernel<<<grid_for(p->Mh, 256, p->num_sms * 8), 256, shm, st>>>(
      p->Ng, reduced, kf, p->n, p->d_edges, p->table, d_counts, d_flag);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_extract(const bsk_plan* p, const cufftComplex* fine, cufftComplex* coarse,
                    const float* axis_w, cudaStream_t st) {
  float scale = (float)(1.0 / ((double)p->N * p->N * p->N));
  extract_kernel<<<grid_for(p->Mh, 256, p->num_sms * 16), 256, 0, st>>>(
      p->N, p->Ng, scale, reinterpret_cast<const float2*>(fine), reinterpret_cast<float2*>(coarse),
      axis_w);
  BSK_CHECK_CUDA(cudaGetLastError());
}

// A grid level's coarse spectrum from its parent's: sub[a][b][c] = parent[qa mod Ngp][qb mod
// Ngp][c] (same 1/N^3 scaling, same CIC weights), zero on the level's own Nyquist planes.
__global__ void subgrid_kernel(int Ngp, int Ngs, const float2* __restrict__ parent,
                               float2* __restrict__ sub) {
  const int Hs = Ngs / 2 + 1, Hp = Ngp / 2 + 1;
  const int64_t Mh = (int64_t)Ngs * Ngs * Hs;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < Mh;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(m % Hs);
    const int64_t r = m / Hs;
    const int b = (int)(r % Ngs), a = (int)(r / Ngs);
    const int qa = fft_freq(a, Ngs), qb = fft_freq(b, Ngs);
    float2 v = make_float2(0.f, 0.f);
    if (!(qa == -Ngs / 2 || qb == -Ngs / 2 || c == Ngs / 2)) {
      const int pa = qa < 0 ? qa + Ngp : qa, pb = qb < 0 ? qb + Ngp : qb;
      v = parent[((int64_t)pa * Ngp + pb) * Hp + c];
    }
    sub[m] = v;
  }
}

void launch_subgrid(const bsk_plan* parent, const bsk_plan* level, const cufftComplex* ps,
                    cufftComplex* ls, cudaStream_t st) {
  subgrid_kernel<<<grid_for(level->Mh, 256, level->num_sms * 16), 256, 0, st>>>(
      parent->Ng, level->Ng, reinterpret_cast<const float2*>(ps), reinterpret_cast<float2*>(ls));
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_window(int N, float scale, cufftComplex* spec, const float* axis_w, int num_sms,
                   cudaStream_t st) {
  const int64_t Mh = (int64_t)N * N * (N / 2 + 1);
  window_kernel<<<grid_for(Mh, 256, num_sms * 16), 256, 0, st>>>(
      N, scale, reinterpret_cast<float2*>(spec), axis_w);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_filter(const bsk_plan* p, const cufftComplex* spec, int s0, int ns,
                   cufftComplex* out, cudaStream_t st) {
  filter_kernel<<<grid_for(p->Mh / 2, 256, p->num_sms * 16), 256, 0, st>>>(
      p->Mh, reinterpret_cast<const float4*>(spec), reinterpret_cast<const uint32_t*>(p->table),
      s0, ns, reinterpret_cast<float4*>(out));
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_filter_indicator(const bsk_plan* p, int s0, int ns, int kweight,
                             cufftDoubleComplex* out, cudaStream_t st) {
  double kf = 2.0 * 3.14159265358979323846 / p->L;
  filter_indicator_kernel<<<grid_for(p->Mh, 256, p->num_sms * 16), 256, 0, st>>>(
      p->Ng, kf, p->table, s0, ns, kweight, reinterpret_cast<double2*>(out));
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_split(const float* in, int S, int64_t K, __nv_bfloat16* split, cudaStream_t st) {
  BSK_REQUIRE(K % 4 == 0, BSK_ERR_UNSUPPORTED, "the bf16 split wants a multiple of 4 points");
  if (S <= 0 || K <= 0) return;
  const int64_t quads = (K + 127) / 128 * 32;
  split_kernel<<<grid_for((int64_t)S * quads, 256, 152 * 16), 256, 0, st>>>(
      reinterpret_cast<const float4*>(in), split, S, K, quads);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_scale(double* v, int64_t n, double s, cudaStream_t st) {
  scale_kernel<<<grid_for(n, 256, 1024), 256, 0, st>>>(v, n, s);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_gridinfo_finish(int64_t T, double inv_k, double* ntri, const double* s1,
                            const double* s2, const double* s3, double* kmean, cudaStream_t st) {
  gridinfo_finish_kernel<<<grid_for(T, 256, 1024), 256, 0, st>>>(T, inv_k, ntri, s1, s2, s3,
                                                                 kmean);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void launch_normalize(int64_t n, const double* b, const double* ntri, double* out,
                      cudaStream_t st) {
  normalize_kernel<<<grid_for(n, 256, 1024), 256, 0, st>>>(n, b, ntri, out);
  BSK_CHECK_CUDA(cudaGetLastError());
}

}  // namespace bsk
