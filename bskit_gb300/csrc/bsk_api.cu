// C ABI of the GB300 bispectrum engine: plans, cuFFT orchestration, dispatch.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>

#include "bsk_internal.cuh"

namespace bsk {

namespace {
thread_local std::string g_err;

class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev_);
    if (prev_ != dev) cudaSetDevice(dev);
    dev_ = dev;
  }
  ~DeviceGuard() {
    if (prev_ != dev_) cudaSetDevice(prev_);
  }

 private:
  int prev_ = 0, dev_ = 0;
};

template <typename F>
int guarded(F&& f) {
  cudaGetLastError();  // a failure left by an earlier call must not be reported by this one
  try {
    f();
    return BSK_OK;
  } catch (const Error& e) {
    g_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return BSK_ERR_OOM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return BSK_ERR_ARG;
  } catch (...) {  // nothing may unwind through the C ABI
    g_err = "unexpected exception";
    return BSK_ERR_STATE;
  }
}

bool nice_size(int m) {
  for (int p : {2, 3, 5, 7})
    while (m % p == 0) m /= p;
  return m == 1;
}

// Smallest even FFT-friendly Ng with Ng > 3*qmax (so no triple of shell modes
// can alias onto k = 0) and Ng <= N; N itself when none exists.
int choose_grid(int N, int qmax, int mode) {
  if (mode == BSK_GRID_NATIVE) return N;
  for (int m = 3 * qmax + 1; m < N; ++m)
    if (m % 2 == 0 && nice_size(m) && m > 2 * qmax + 1) return m;
  return N;
}

void* dmalloc(size_t bytes) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error{BSK_ERR_OOM, "cudaMalloc(" + std::to_string(bytes) + ") failed: " +
                                 cudaGetErrorString(e)};
  }
  return p;
}

void* dmalloc_async(size_t bytes, cudaStream_t st) {
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error{BSK_ERR_OOM, "cudaMallocAsync(" + std::to_string(bytes) + ") failed: " +
                                 cudaGetErrorString(e)};
  }
  return p;
}

// A stream-ordered device temporary that an error unwinding the call also releases.
// release() is the success path: it frees at that point and reports a failure.
struct AsyncTemp {
  void* ptr = nullptr;
  cudaStream_t st = nullptr;
  AsyncTemp(size_t bytes, cudaStream_t s) : ptr(dmalloc_async(bytes, s)), st(s) {}
  ~AsyncTemp() {
    if (ptr) cudaFreeAsync(ptr, st);
  }
  void release() {
    void* q = ptr;
    ptr = nullptr;
    BSK_CHECK_CUDA(cudaFreeAsync(q, st));
  }
  AsyncTemp(const AsyncTemp&) = delete;
  AsyncTemp& operator=(const AsyncTemp&) = delete;
};

// The same for a synchronous allocation, freed when the scope ends.
struct SyncTemp {
  void* ptr = nullptr;
  explicit SyncTemp(size_t bytes) : ptr(dmalloc(bytes)) {}
  ~SyncTemp() {
    if (ptr) cudaFree(ptr);
  }
  SyncTemp(const SyncTemp&) = delete;
  SyncTemp& operator=(const SyncTemp&) = delete;
};

void grow_work(bsk_plan* p, size_t ws) {
  if (ws <= p->work_bytes) return;
  if (p->work) cudaFree(p->work);
  p->work = nullptr;
  p->work = dmalloc(ws);
  p->work_bytes = ws;
}

void make_c2r(bsk_plan* p) {
  int n[3] = {p->Ng, p->Ng, p->Ng};
  BSK_CHECK_CUFFT(cufftCreate(&p->c2r));
  p->c2r_ok = true;
  BSK_CHECK_CUFFT(cufftSetAutoAllocation(p->c2r, 0));
  size_t ws = 0;
  BSK_CHECK_CUFFT(cufftMakePlanMany(p->c2r, 3, n, nullptr, 1, (int)p->Mh, nullptr, 1,
                                    (int)p->K, CUFFT_C2R, p->chunk, &ws));
  grow_work(p, ws);
}

void make_z2d(bsk_plan* p) {
  if (p->z2d_ok) return;
  int n[3] = {p->Ng, p->Ng, p->Ng};
  BSK_CHECK_CUFFT(cufftCreate(&p->z2d));
  p->z2d_ok = true;
  BSK_CHECK_CUFFT(cufftSetAutoAllocation(p->z2d, 0));
  size_t ws = 0;
  BSK_CHECK_CUFFT(cufftMakePlanMany(p->z2d, 3, n, nullptr, 1, (int)p->Mh, nullptr, 1,
                                    (int)p->K, CUFFT_Z2D, p->chunk, &ws));
  grow_work(p, ws);
}

void make_r2c(bsk_plan* p) {
  BSK_CHECK_CUFFT(cufftCreate(&p->r2c));
  p->r2c_ok = true;
  BSK_CHECK_CUFFT(cufftSetAutoAllocation(p->r2c, 0));
  size_t ws = 0;
  BSK_CHECK_CUFFT(cufftMakePlan3d(p->r2c, p->N, p->N, p->N, CUFFT_R2C, &ws));
  grow_work(p, ws);
}

void bind_work(bsk_plan* p, cufftHandle h, cudaStream_t st) {
  BSK_CHECK_CUFFT(cufftSetWorkArea(h, p->work));
  BSK_CHECK_CUFFT(cufftSetStream(h, st));
}

// Device bytes the plan holds: shell table, filter staging, per-slot spectra,
// fields and bf16 splits, and the shared cuFFT work area; with its grid-level plans.
int64_t own_footprint(const bsk_plan* p) {
  int64_t fp = (int64_t)p->Mh * 2 + (p->chunk_spec ? (int64_t)p->chunk * p->Mh * 8 : 0);
  for (const auto& s : p->slot) {
    if (s.spec) fp += p->Mh * 8;
    if (s.fields) fp += (int64_t)p->n_alloc() * p->K * 4;
    if (s.split) fp += (int64_t)split_elems(p->n_alloc(), p->K) * 2;
  }
  if (p->stream_C) fp += (int64_t)p->stream_C * p->K * (3 * 4 + (p->stream_tc ? 4 : 0));
  if (p->synth_ws) fp += (int64_t)p->synth_ws_bytes;
  return fp + (int64_t)p->work_bytes;
}

int64_t footprint(const bsk_plan* p) {
  int64_t fp = own_footprint(p);
  for (const bsk_plan* q : p->levels) fp += own_footprint(q);
  return fp;
}

// Refuse an allocation of `bytes` that would take the plan (with its grid levels: the
// budget is the root plan's) above its budget.
void check_budget(const bsk_plan* p, size_t bytes, const char* what) {
  const bsk_plan* root = p->parent ? p->parent : p;
  if (root->mem_budget == 0) return;
  const int64_t after = footprint(root) + (int64_t)bytes;
  if (after > (int64_t)root->mem_budget)
    throw Error{BSK_ERR_OOM, std::string(what) + " would take the plan to " +
                                 std::to_string(after) + " bytes, above its budget of " +
                                 std::to_string(root->mem_budget)};
}

void release_stream(bsk_plan* p) {
  for (auto& b : p->stream_f) {
    if (b.ptr) cudaFree(b.ptr);
    b = StreamBuf{};
  }
  if (p->stream_split.ptr) cudaFree(p->stream_split.ptr);
  p->stream_split = StreamBuf{};
  p->stream_C = 0;
  p->stream_tc = false;
}

void alloc_split(bsk_plan* p, FieldSlot& f) {
  if (f.split) return;
  // the chunk-major split of all n_alloc shells; zeroed once, so that the shells beyond n
  // (padding to the FFT batch, read by some tiles' boxes) and the tail of the last chunk
  // stay zero when only the synthesis writes it
  const size_t bytes = split_elems(p->n_alloc(), p->K) * sizeof(__nv_bfloat16);
  check_budget(p, bytes, "the bf16 split of the fields");
  f.split = (__nv_bfloat16*)dmalloc(bytes);
  BSK_CHECK_CUDA(cudaMemset(f.split, 0, bytes));
}

// Masked shell fields of `slot` for shells [0, n_need) (every shell by default).  With a
// grid the field synthesis supports, its pruned FFT passes write the fields (and, when
// `with_split`, their bf16 hi / lo planes in the same pass) batch by batch; otherwise filter
// kernel + batched cuFFT C2R for every shell.
void ensure_fields(bsk_plan* p, int s, cudaStream_t st, bool with_split = false,
                   int n_need = -1) {
  FieldSlot& f = p->slot[s];
  BSK_REQUIRE(f.painted, BSK_ERR_STATE, "field slot " + std::to_string(s) + " was not painted");
  const int need = n_need < 0 ? p->n : std::min(n_need, p->n);
  if (f.fields_ok && f.fields_n >= need && f.fields_from == 0) return;
  if (!f.fields) {
    check_budget(p, (size_t)p->n_alloc() * p->K * sizeof(float), "the shell fields");
    f.fields = (float*)dmalloc((size_t)p->n_alloc() * p->K * sizeof(float));
    const size_t pad = (size_t)(p->n_alloc() - p->n) * p->K;
    if (pad)
      BSK_CHECK_CUDA(cudaMemset(f.fields + (size_t)p->n * p->K, 0, pad * sizeof(float)));
  }
  if (p->use_synth) {
    if (!p->synth_ws) {
      check_budget(p, p->synth_ws_bytes, "the field-synthesis workspace");
      p->synth_ws = dmalloc(p->synth_ws_bytes);
      synth_init_workspace(p->Ng, p->synth_ws);
    }
    if (with_split) alloc_split(p, f);
    int done = 0;
    for (int s0 = 0; s0 < need; s0 += p->chunk) {
      const int ns = std::min(p->chunk, p->n - s0);
      int R = 0;
      for (int k = s0; k < s0 + ns; ++k) R = std::max(R, p->shell_r[k]);
      launch_synth(p->Ng, f.spec, p->table, s0, ns, R, p->synth_ws, f.fields,
                   with_split ? f.split : nullptr, p->n_alloc(), st);
      done = s0 + ns;
    }
    f.fields_ok = true;
    f.fields_n = done;
    f.fields_from = 0;
    if (with_split) {
      f.split_ok = true;
      f.split_n = done;
    }
    return;
  }
  bind_work(p, p->c2r, st);
  for (int s0 = 0; s0 < p->n; s0 += p->chunk) {
    int ns = std::min(p->chunk, p->n - s0);
    launch_filter(p, f.spec, s0, ns, p->chunk_spec, st);
    if (ns < p->chunk)  // the batched plan transforms `chunk` spectra: clear the unused tail
      BSK_CHECK_CUDA(cudaMemsetAsync(p->chunk_spec + (size_t)ns * p->Mh, 0,
                                     (size_t)(p->chunk - ns) * p->Mh * sizeof(cufftComplex),
                                     st));
    BSK_CHECK_CUFFT(cufftExecC2R(p->c2r, p->chunk_spec, f.fields + (size_t)s0 * p->K));
  }
  f.fields_ok = true;
  f.fields_n = p->n;
  f.fields_from = 0;
  f.split_ok = false;
}

void ensure_split(bsk_plan* p, int s, cudaStream_t st, int n_need = -1) {
  FieldSlot& f = p->slot[s];
  const int need = n_need < 0 ? p->n : std::min(n_need, p->n);
  ensure_fields(p, s, st, true, n_need);
  if (f.split_ok && f.split_n >= need) return;
  alloc_split(p, f);
  launch_split(f.fields, p->n_alloc(), p->K, f.split, st);  // FP32 valid from shell 0
  f.split_ok = true;
  f.split_n = p->n;
}

// A grid level's slot for shells [0, nn): the FP32 fields of shells >= fp_from (the pair
// factors of its bins; nn when the slot is not a pair factor) and, when `need_split`, the
// bf16 split of all of them (the column operand), in one synthesis pass per batch; batches
// that hold neither are skipped.
void ensure_level_fields(bsk_plan* q, int s, cudaStream_t st, int nn, int fp_from,
                         bool need_split) {
  FieldSlot& f = q->slot[s];
  BSK_REQUIRE(f.painted, BSK_ERR_STATE, "field slot " + std::to_string(s) + " was not painted");
  nn = std::min(nn, q->n);
  fp_from = std::min(fp_from, nn);
  const bool fp_ok = fp_from >= nn || (f.fields_ok && f.fields_from <= fp_from &&
                                       f.fields_n >= nn);
  const bool split_ok = !need_split || (f.split_ok && f.split_n >= nn);
  if (fp_ok && split_ok) return;
  if (!f.fields && fp_from < nn) {  // a column-only slot needs no FP32 fields
    check_budget(q, (size_t)q->n_alloc() * q->K * sizeof(float), "the shell fields");
    f.fields = (float*)dmalloc((size_t)q->n_alloc() * q->K * sizeof(float));
    const size_t pad = (size_t)(q->n_alloc() - q->n) * q->K;
    if (pad)
      BSK_CHECK_CUDA(cudaMemset(f.fields + (size_t)q->n * q->K, 0, pad * sizeof(float)));
  }
  if (!q->synth_ws) {
    check_budget(q, q->synth_ws_bytes, "the field-synthesis workspace");
    q->synth_ws = dmalloc(q->synth_ws_bytes);
    synth_init_workspace(q->Ng, q->synth_ws);
  }
  if (need_split) alloc_split(q, f);
  const int from = need_split ? 0 : fp_from / q->chunk * q->chunk;
  int done = from;
  for (int s0 = from; s0 < nn; s0 += q->chunk) {
    const int ns = std::min(q->chunk, q->n - s0);
    int R = 0;
    for (int k = s0; k < s0 + ns; ++k) R = std::max(R, q->shell_r[k]);
    launch_synth(q->Ng, f.spec, q->table, s0, ns, R, q->synth_ws, f.fields,
                 need_split ? f.split : nullptr, q->n_alloc(), st, 0, fp_from);
    done = s0 + ns;
  }
  // what this pass wrote replaces what the slot held
  f.fields_ok = fp_from < nn;
  f.fields_from = fp_from;
  f.fields_n = done;
  if (need_split) {
    f.split_ok = true;
    f.split_n = done;
  }
}

void free_slot(FieldSlot& f) {
  if (f.spec) cudaFree(f.spec);
  if (f.fields) cudaFree(f.fields);
  if (f.split) cudaFree(f.split);
  f = FieldSlot{};
}

void destroy_triset(bsk_triset* set) {
  if (!set) return;
  DeviceGuard g(set->plan->device);
  set->sched.release();
  for (auto& lv : set->levels) lv.sched.release();
  for (auto& kv : set->groups)
    for (auto& g : kv.second) g.sched.release();
  if (set->dups) cudaFree(set->dups);
  delete set;
}

void destroy_plan(bsk_plan* p) {
  if (!p) return;
  DeviceGuard g(p->device);
  cudaDeviceSynchronize();
  for (bsk_plan* q : p->levels) destroy_plan(q);
  p->levels.clear();
  for (auto& s : p->slot) free_slot(s);
  if (p->table) cudaFree(p->table);
  if (p->d_edges) cudaFree(p->d_edges);
  if (p->chunk_spec) cudaFree(p->chunk_spec);
  if (p->cic_w) cudaFree(p->cic_w);
  if (p->r2c_ok) cufftDestroy(p->r2c);
  if (p->r2c_sub_nfull) cufftDestroy(p->r2c_sub);
  if (p->c2r_ok) cufftDestroy(p->c2r);
  if (p->z2d_ok) cufftDestroy(p->z2d);
  if (p->work) cudaFree(p->work);
  if (p->synth_ws) cudaFree(p->synth_ws);
  release_stream(p);
  delete p;
}

// Scatter results of the first occurrence of a repeated triangle to its copies.
__global__ void copy_dups_kernel(int n, const int2* pairs, double* v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[pairs[i].x] = v[pairs[i].y];
}

void copy_dups(const bsk_triset* set, double* v, cudaStream_t st) {
  if (set->n_dups == 0) return;
  int n = set->n_dups;
  copy_dups_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, set->dups, v);
  BSK_CHECK_CUDA(cudaGetLastError());
}

void contract_dispatch(bsk_plan* p, const bsk_triset* set, const float* f1, const float* f2,
                       const float* f3, const __nv_bfloat16* split, int split_shells,
                       int64_t K, int64_t k0, int64_t k1, int precision, double* out,
                       cudaStream_t st) {
  BSK_CHECK_CUDA(cudaMemsetAsync(out, 0, (size_t)set->T * sizeof(double), st));
  switch (precision) {
    case BSK_PREC_FP64:
      launch_contract_simt_f64(set->sched, f1, f2, f3, p->n, K, k0, k1, out, p->num_sms, st);
      break;
    case BSK_PREC_FP32:
      launch_contract_simt_f32(set->sched, f1, f2, f3, p->n, K, k0, k1, out, p->num_sms, st);
      break;
    case BSK_PREC_BF16X3:
    case BSK_PREC_BF16:
      launch_contract_tc(set->sched, f1, f2, split, split_shells, p->n, K, k0, k1,
                         precision == BSK_PREC_BF16X3 ? 3 : 1, out, p->num_sms, st);
      break;
    default:
      throw Error{BSK_ERR_ARG, "unknown precision " + std::to_string(precision)};
  }
  copy_dups(set, out, st);
}

// ---------------------------------------------------------------- shell streaming
// Triangle groups of a set for chunks of C shells: key (i/C, j/C, l/C), shells
// rebased to their chunk, groups in lexicographic key order so that the first
// chunk changes least often.  Built once per (set, C).
const std::vector<StreamGroup>& stream_groups(const bsk_triset* set, int C) {
  auto it = set->groups.find(C);
  if (it != set->groups.end()) return it->second;
  std::map<std::tuple<int, int, int>, std::pair<std::vector<HostTriangle>, std::vector<int>>> by;
  for (size_t u = 0; u < set->u_tri.size(); ++u) {
    const HostTriangle& h = set->u_tri[u];
    auto& e = by[std::make_tuple(h.i / C, h.j / C, h.l / C)];
    e.first.push_back(HostTriangle{h.i % C, h.j % C, h.l % C});
    e.second.push_back(set->u_idx[u]);
  }
  std::vector<StreamGroup>& gs = set->groups[C];
  gs.resize(by.size());
  size_t g = 0;
  for (auto& kv : by) {
    gs[g].ca = std::get<0>(kv.first);
    gs[g].cb = std::get<1>(kv.first);
    gs[g].cc = std::get<2>(kv.first);
    build_schedule(kv.second.first, C, gs[g].sched, &kv.second.second);
    ++g;
  }
  return gs;
}

// FP32 fields of shells [s0, s0 + C) of `slot` into dst[C][K] (C a multiple of the
// FFT batch); shells at or beyond n are zero.
void chunk_fields(bsk_plan* p, int slot, int s0, int C, float* dst, cudaStream_t st) {
  const FieldSlot& f = p->slot[slot];
  // the synthesis needs its workspace: use it when held already or when the budget has
  // room for it, else the filter + cuFFT path (whose buffers the plan always holds)
  const bool ws_fits = p->synth_ws || p->mem_budget == 0 ||
                       footprint(p) + (int64_t)p->synth_ws_bytes <= (int64_t)p->mem_budget;
  if (p->use_synth && ws_fits) {
    if (!p->synth_ws) {
      p->synth_ws = dmalloc(p->synth_ws_bytes);
      synth_init_workspace(p->Ng, p->synth_ws);
    }
    for (int b = 0; b < C; b += p->chunk) {
      const int first = s0 + b;
      const int ns = std::max(0, std::min(p->chunk, p->n - first));
      if (ns == 0) {
        BSK_CHECK_CUDA(cudaMemsetAsync(dst + (size_t)b * p->K, 0,
                                       (size_t)(C - b) * p->K * sizeof(float), st));
        break;
      }
      int R = 0;
      for (int k = first; k < first + ns; ++k) R = std::max(R, p->shell_r[k]);
      launch_synth(p->Ng, f.spec, p->table, first, ns, R, p->synth_ws, dst, nullptr, 0, st,
                   s0);
      if (ns < p->chunk)
        BSK_CHECK_CUDA(cudaMemsetAsync(dst + (size_t)(b + ns) * p->K, 0,
                                       (size_t)(p->chunk - ns) * p->K * sizeof(float), st));
    }
    return;
  }
  bind_work(p, p->c2r, st);
  for (int b = 0; b < C; b += p->chunk) {
    const int first = s0 + b;
    const int ns = std::max(0, std::min(p->chunk, p->n - first));
    if (ns == 0) {
      BSK_CHECK_CUDA(cudaMemsetAsync(dst + (size_t)b * p->K, 0,
                                     (size_t)p->chunk * p->K * sizeof(float), st));
      continue;
    }
    launch_filter(p, f.spec, first, ns, p->chunk_spec, st);
    if (ns < p->chunk)
      BSK_CHECK_CUDA(cudaMemsetAsync(p->chunk_spec + (size_t)ns * p->Mh, 0,
                                     (size_t)(p->chunk - ns) * p->Mh * sizeof(cufftComplex),
                                     st));
    BSK_CHECK_CUFFT(cufftExecC2R(p->c2r, p->chunk_spec, dst + (size_t)b * p->K));
  }
}

// Choose the streaming chunk: the largest multiple of the FFT batch whose buffers
// (bytes_per_shell each) fit in what the budget leaves, at most all shells.
int stream_chunk(const bsk_plan* p, int64_t held, size_t bytes_per_shell, const char* what) {
  const int64_t avail = (int64_t)p->mem_budget - (footprint(p) - held);
  int C = 0;
  if (avail > 0) C = (int)std::min<int64_t>(avail / (int64_t)bytes_per_shell, p->n_alloc());
  C = C / p->chunk * p->chunk;
  if (C < p->chunk)
    throw Error{BSK_ERR_OOM, std::string(what) + ": the budget of " +
                                 std::to_string(p->mem_budget) + " bytes leaves room for no "
                                 "chunk of " + std::to_string(p->chunk) + " shells"};
  return C;
}

// Streamed B: the fields of each group's three chunks are taken from three
// C-shell buffers, recomputed only when a buffer does not hold them.
void measure_b_stream(bsk_plan* p, const bsk_triset* set, int a, int b, int c, int precision,
                      int64_t k0, int64_t k1, double* out, cudaStream_t st) {
  const bool tc = precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16;
  const size_t per_shell = (size_t)p->K * (3 * 4 + (tc ? 4 : 0));
  const int64_t held = p->stream_C ? (int64_t)p->stream_C * p->K * (12 + (p->stream_tc ? 4 : 0))
                                   : 0;
  const int C = stream_chunk(p, held, per_shell, "shell streaming");
  if (C != p->stream_C || (tc && !p->stream_tc)) {
    release_stream(p);
    for (auto& buf : p->stream_f) buf.ptr = dmalloc((size_t)C * p->K * sizeof(float));
    if (tc) p->stream_split.ptr = dmalloc(split_elems(C, p->K) * sizeof(__nv_bfloat16));
    p->stream_C = C;
    p->stream_tc = tc;
  }
  const int slots[3] = {a, b, c};
  for (int sl : slots)
    BSK_REQUIRE(p->slot[sl].painted, BSK_ERR_STATE,
                "field slot " + std::to_string(sl) + " was not painted");
  auto key_of = [&](int role, int chunk) -> int64_t {
    const int sl = slots[role];
    return ((p->slot[sl].gen * 4 + sl) << 8) | chunk;
  };
  BSK_CHECK_CUDA(cudaMemsetAsync(out, 0, (size_t)set->T * sizeof(double), st));
  const auto& groups = stream_groups(set, C);
  for (const StreamGroup& g : groups) {
    const int chunks[3] = {g.ca, g.cb, g.cc};
    int64_t want[3];
    for (int r = 0; r < 3; ++r) want[r] = key_of(r, chunks[r]);
    // roles whose FP32 fields are read: f1, f2 always; f3 unless the split of it is current
    const bool need3 = !tc || p->stream_split.key != want[2];
    const float* fp[3] = {nullptr, nullptr, nullptr};
    bool keep[3] = {false, false, false};  // buffers holding a wanted key
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q)
        if (p->stream_f[q].key == want[r] && (r < 2 || need3)) {
          fp[r] = (const float*)p->stream_f[q].ptr;
          keep[q] = true;
        }
    for (int r = 0; r < 3; ++r) {
      if (fp[r] || (r == 2 && !need3)) continue;
      int q = 0;
      while (keep[q]) ++q;  // at most three wanted keys: a free buffer exists
      chunk_fields(p, slots[r], chunks[r] * C, C, (float*)p->stream_f[q].ptr, st);
      p->stream_f[q].key = want[r];
      keep[q] = true;
      fp[r] = (const float*)p->stream_f[q].ptr;
      for (int r2 = r + 1; r2 < 3; ++r2)
        if (want[r2] == want[r]) fp[r2] = fp[r];
    }
    const __nv_bfloat16* split = nullptr;
    if (tc) {
      __nv_bfloat16* h = (__nv_bfloat16*)p->stream_split.ptr;
      if (p->stream_split.key != want[2]) {
        launch_split(fp[2], C, p->K, h, st);
        p->stream_split.key = want[2];
      }
      split = h;
    }
    switch (precision) {
      case BSK_PREC_FP64:
        launch_contract_simt_f64(g.sched, fp[0], fp[1], fp[2], C, p->K, k0, k1, out,
                                 p->num_sms, st);
        break;
      case BSK_PREC_FP32:
        launch_contract_simt_f32(g.sched, fp[0], fp[1], fp[2], C, p->K, k0, k1, out,
                                 p->num_sms, st);
        break;
      default:
        launch_contract_tc(g.sched, fp[0], fp[1], split, C, C, p->K, k0, k1,
                           precision == BSK_PREC_BF16X3 ? 3 : 1, out, p->num_sms, st);
    }
  }
  copy_dups(set, out, st);
  p->last_stream_C = C;
}

// ---------------------------------------------------------------- grid levels
// A bin (i, j, l) is exact on any grid of side Ng > r_i + r_j + r_l (the three wavevectors of
// a closed triangle cannot wrap around), with each of its shells inside the grid's Nyquist
// range (2 r < Ng); r_s is the largest |q_c| of a mode of shell s.  The plan's reduced grid
// satisfies both for every bin; bins of small shells are contracted on smaller grids, at a
// cost proportional to Ng^3 per point, with the shells they use synthesised on those grids.

// The grid-level plan of side Ng of p (made on first use, holding every shell of p that
// fits the side, at least shells [0, n)).  Its spectra come from p's slots (launch_subgrid); it has no transforms of
// its own besides the field synthesis.
bsk_plan* level_plan(bsk_plan* p, int Ng, int n) {
  for (bsk_plan* q : p->levels)
    if (q->Ng == Ng) {
      BSK_REQUIRE(q->n >= n, BSK_ERR_STATE, "internal: a grid level lacks a shell");
      return q;
    }
  // every shell that fits the side (the shells are sorted by radius): one plan per side
  // serves every triangle set of the plan
  while (n < p->n && 2 * p->shell_r[n] < Ng) ++n;
  std::unique_ptr<bsk_plan, void (*)(bsk_plan*)> q(new bsk_plan(), destroy_plan);
  q->device = p->device;
  q->num_sms = p->num_sms;
  q->N = p->N;
  q->L = p->L;
  q->n = n;
  q->parent = p;
  q->edges.assign(p->edges.begin(), p->edges.begin() + 2 * n);
  q->shell_r.assign(p->shell_r.begin(), p->shell_r.begin() + n);
  q->qmax = 0;
  for (int r : q->shell_r) q->qmax = std::max(q->qmax, r);
  BSK_REQUIRE(2 * q->qmax < Ng, BSK_ERR_STATE, "internal: a level's shell exceeds its grid");
  q->Ng = Ng;
  q->K = (int64_t)Ng * Ng * Ng;
  q->Mh = (int64_t)Ng * Ng * (Ng / 2 + 1);
  q->chunk = std::min(n, 8);
  check_budget(p, (size_t)q->Mh * sizeof(uint16_t), "a grid level's shell table");
  q->table = (uint16_t*)dmalloc((size_t)q->Mh * sizeof(uint16_t));
  q->d_edges = (double*)dmalloc((size_t)2 * n * sizeof(double));
  BSK_CHECK_CUDA(cudaMemcpy(q->d_edges, q->edges.data(), 2 * n * sizeof(double),
                            cudaMemcpyHostToDevice));
  int hf[2] = {0, 0};
  {
    SyncTemp counts_t(n * sizeof(unsigned long long));
    SyncTemp flag_t(2 * sizeof(int));
    BSK_CHECK_CUDA(cudaMemset(counts_t.ptr, 0, n * sizeof(unsigned long long)));
    BSK_CHECK_CUDA(cudaMemset(flag_t.ptr, 0, 2 * sizeof(int)));
    launch_shell_table(q.get(), (unsigned long long*)counts_t.ptr, (int*)flag_t.ptr, 0);
    BSK_CHECK_CUDA(cudaMemcpy(hf, flag_t.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost));
  }
  BSK_REQUIRE(hf[0] == 0 && hf[1] <= q->qmax, BSK_ERR_STATE,
              "internal: a grid level's shell table disagrees with its plan");
  q->use_synth = synth_supported(Ng);
  BSK_REQUIRE(q->use_synth, BSK_ERR_STATE, "internal: no field synthesis for a grid level");
  q->synth_ws_bytes = synth_workspace_bytes(Ng, q->qmax, q->chunk);
  p->levels.push_back(q.get());
  return q.release();
}

// Slot s of a level plan from the parent's slot (again after every paint of the parent).
void sync_level(bsk_plan* p, bsk_plan* q, int s, cudaStream_t st) {
  const FieldSlot& pf = p->slot[s];
  FieldSlot& qf = q->slot[s];
  BSK_REQUIRE(pf.painted, BSK_ERR_STATE, "field slot " + std::to_string(s) + " was not painted");
  if (qf.painted && qf.gen == pf.gen) return;
  if (!qf.spec) {
    check_budget(q, (size_t)q->Mh * sizeof(cufftComplex), "a grid level's spectrum");
    qf.spec = (cufftComplex*)dmalloc((size_t)q->Mh * sizeof(cufftComplex));
  }
  launch_subgrid(p, q, pf.spec, qf.spec, st);
  qf.painted = true;
  qf.gen = pf.gen;
  qf.fields_ok = false;
  qf.split_ok = false;
  qf.fields_n = qf.split_n = qf.fields_from = 0;
}

// Grid sides the levels may take (below the plan's own): the sizes whose field synthesis is
// compiled with constant strides.
const int kLevelSides[] = {48, 96, 128, 160, 192, 240, 256, 288, 320, 384, 480};
// Per point: one 128-row tile of the tensor-core contraction costs ~13 field syntheses of a
// shell (measured on the 384^3 grid: 2.44 ms per tile, 0.187 ms per shell of a batch of 8).
constexpr double kTileCost = 13.0, kShellCost = 1.0;
constexpr double kMinLevelPoints = 0.4;

// Chooses the set's grid levels (choose_level_sides over the candidate sides) and builds one
// schedule per level, a level plan for every side below the plan's own.
void build_levels(bsk_plan* p, bsk_triset* set) {
  // A bin's rounding error relative to its value falls as 1/sqrt(points summed), so a level
  // keeps at least kMinLevelPoints of the plan grid's points: its bins' relative errors stay
  // within 1.6x of the plan grid's.  (BSK_LEVEL_MIN_POINTS overrides the fraction.)
  double min_points = kMinLevelPoints;
  if (const char* e = std::getenv("BSK_LEVEL_MIN_POINTS")) min_points = std::atof(e);
  std::vector<int> sides;  // candidates, then the plan's grid
  for (int n : kLevelSides)
    if (n < p->Ng && synth_fast_size(n) &&
        std::pow((double)n / p->Ng, 3) >= min_points)
      sides.push_back(n);
  sides.push_back(p->Ng);
  const int m = (int)sides.size();
  const int nt = (int)set->u_tri.size();
  const std::vector<int> lev =
      choose_level_sides(set->u_tri, p->shell_r, sides, p->n, kTileCost, kShellCost);
  for (int j = 0; j < m; ++j) {
    std::vector<HostTriangle> tk;
    std::vector<int> idx;
    int top = -1;
    for (int t = 0; t < nt; ++t)
      if (lev[t] == j) {
        const HostTriangle& h = set->u_tri[t];
        tk.push_back(h);
        idx.push_back(set->u_idx[t]);
        top = std::max(top, std::max(h.i, std::max(h.j, h.l)));
      }
    if (tk.empty()) continue;
    GridLevel lv;
    lv.n_shells = top + 1;
    lv.src_min = top + 1;
    for (const HostTriangle& h : tk) lv.src_min = std::min(lv.src_min, std::min(h.i, h.j));
    lv.bins = (int64_t)tk.size();
    lv.plan = j == m - 1 ? p : level_plan(p, sides[j], top + 1);
    set->levels.push_back(lv);
    build_schedule(tk, lv.plan->n, set->levels.back().sched, &idx);
  }
}

// A point range [k0, k1) of the plan's grid as the matching share of a level's grid
// (128-point aligned, so that the ranges of consecutive shards tile the level's grid).
int64_t level_point(int64_t k, int64_t K, int64_t Kq) {
  if (k >= K) return Kq;
  return (int64_t)((__int128)k * Kq / K) / 128 * 128;
}

// The resident path over the set's grid levels: every level adds its bins' scaled sums
// into `out`.
void measure_levels(bsk_plan* p, const bsk_triset* set, int a, int b, int c, int precision,
                    int64_t k0, int64_t k1, double* out, cudaStream_t st) {
  const bool tc = precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16;
  BSK_CHECK_CUDA(cudaMemsetAsync(out, 0, (size_t)set->T * sizeof(double), st));
  for (const GridLevel& lv : set->levels) {
    bsk_plan* q = lv.plan;
    const int nn = lv.n_shells;
    if (q != p) {
      sync_level(p, q, a, st);
      if (b != a) sync_level(p, q, b, st);
      if (c != a && c != b) sync_level(p, q, c, st);
    }
    // tensor-core paths read FP32 fields only as pair factors (shells >= the level's smallest
    // i or j) and the split of slot c; the SIMT paths read FP32 fields of every shell
    const int sls[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
      const int sl = sls[k];
      if ((k >= 1 && sl == sls[0]) || (k == 2 && sl == sls[1])) continue;  // done already
      const bool factor = sl == a || sl == b;
      const int fp_from = !tc ? 0 : factor ? lv.src_min : nn;
      ensure_level_fields(q, sl, st, nn, fp_from, tc && sl == c);
    }
    BSK_REQUIRE(q->slot[a].fields && q->slot[b].fields &&
                    (tc ? q->slot[c].split != nullptr : q->slot[c].fields != nullptr),
                BSK_ERR_STATE, "internal: a grid level's operands were not built");
    const int64_t q0 = level_point(k0, p->K, q->K), q1 = level_point(k1, p->K, q->K);
    if (q1 <= q0) continue;
    const double scale = std::pow(p->L, 6) / (double)q->K;
    const float *fa = q->slot[a].fields, *fb = q->slot[b].fields, *fc = q->slot[c].fields;
    switch (precision) {
      case BSK_PREC_FP64:
        launch_contract_simt_f64(lv.sched, fa, fb, fc, q->n, q->K, q0, q1, out, q->num_sms, st,
                                 scale);
        break;
      case BSK_PREC_FP32:
        launch_contract_simt_f32(lv.sched, fa, fb, fc, q->n, q->K, q0, q1, out, q->num_sms, st,
                                 scale);
        break;
      default:
        launch_contract_tc(lv.sched, fa, fb, q->slot[c].split, q->n_alloc(), q->n, q->K, q0,
                           q1, precision == BSK_PREC_BF16X3 ? 3 : 1, out, q->num_sms, st,
                           scale);
        break;
    }
  }
  copy_dups(set, out, st);
}

// Device bytes the resident path still has to allocate for slots a, b, c (and the split of
// c) on every grid it uses.
int64_t resident_need(const bsk_plan* p, const bsk_triset* set, int a, int b, int c, bool tc) {
  std::vector<const bsk_plan*> grids;
  if (set->levels.empty()) grids.push_back(p);
  for (const GridLevel& lv : set->levels)
    if (std::find(grids.begin(), grids.end(), lv.plan) == grids.end()) grids.push_back(lv.plan);
  int64_t need = 0;
  for (const bsk_plan* q : grids) {
    bool seen[3] = {false, false, false};
    for (int sl : {a, b, c})
      if (!seen[sl]) {
        seen[sl] = true;
        if (!q->slot[sl].fields) need += (int64_t)q->n_alloc() * q->K * sizeof(float);
        if (q != p && !q->slot[sl].spec) need += q->Mh * (int64_t)sizeof(cufftComplex);
      }
    if (tc && !q->slot[c].split)
      need += (int64_t)split_elems(q->n_alloc(), q->K) * sizeof(__nv_bfloat16);
    // the field synthesis' workspace is allocated with the first resident fields
    if (q->use_synth && !q->synth_ws) need += (int64_t)q->synth_ws_bytes;
  }
  return need;
}

void measure_b(bsk_plan* p, const bsk_triset* set, int a, int b, int c, int precision,
               int64_t k0, int64_t k1, double* out, cudaStream_t st) {
  BSK_REQUIRE(p && set, BSK_ERR_ARG, "NULL argument");
  BSK_REQUIRE(set->plan == p, BSK_ERR_ARG, "triangle set belongs to another plan");
  BSK_REQUIRE(a >= 0 && a < 3 && b >= 0 && b < 3 && c >= 0 && c < 3, BSK_ERR_ARG,
              "slot must be 0, 1 or 2");
  BSK_REQUIRE(0 <= k0 && k0 <= k1 && k1 <= p->K, BSK_ERR_ARG, "bad point range");
  const bool tc = precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16;
  BSK_REQUIRE(tc || precision == BSK_PREC_FP32 || precision == BSK_PREC_FP64, BSK_ERR_ARG,
              "unknown precision " + std::to_string(precision));
  if (set->T == 0) return;  // nothing to write: out may be NULL
  BSK_REQUIRE(out, BSK_ERR_ARG, "NULL argument");
  if (tc)
    BSK_REQUIRE(k0 % 128 == 0 && (k1 % 128 == 0 || k1 == p->K), BSK_ERR_ARG,
                "tensor-core point ranges must start and end at multiples of 128 (or end at "
                "the whole grid)");
  if (k0 == k1) {  // an empty share of the grid (more ranks than 128-point stages): zeros
    BSK_CHECK_CUDA(cudaMemsetAsync(out, 0, (size_t)set->T * sizeof(double), st));
    return;
  }
  if (p->mem_budget) {
    // resident path: all shells of each slot (and the split of the third) stay on the device,
    // on every grid level of the set
    const int64_t need = resident_need(p, set, a, b, c, tc);
    const int64_t held =
        p->stream_C ? (int64_t)p->stream_C * p->K * (12 + (p->stream_tc ? 4 : 0)) : 0;
    if (footprint(p) - held + need > (int64_t)p->mem_budget) {
      measure_b_stream(p, set, a, b, c, precision, k0, k1, out, st);
      launch_scale(out, set->T, std::pow(p->L, 6) / (double)p->K, st);
      return;
    }
    release_stream(p);
  }
  p->last_stream_C = 0;
  if (!set->levels.empty()) {
    measure_levels(p, set, a, b, c, precision, k0, k1, out, st);
    return;
  }
  if (tc) ensure_split(p, c, st);  // first, so that a synthesis pass writes the split as well
  ensure_fields(p, a, st);
  ensure_fields(p, b, st);
  ensure_fields(p, c, st);
  const __nv_bfloat16* split = nullptr;
  if (tc) {
    ensure_split(p, c, st);
    split = p->slot[c].split;
  }
  contract_dispatch(p, set, p->slot[a].fields, p->slot[b].fields, p->slot[c].fields, split,
                    p->n_alloc(), p->K, k0, k1, precision, out, st);
  const double scale = std::pow(p->L, 6) / (double)p->K;
  launch_scale(out, set->T, scale, st);
}

// Indicator (kind 0) or |k|-weighted (kind 1) FP64 fields of shells [s0, s0 + C)
// into dst[C][K]; shells at or beyond n are zero.
void chunk_indicator(bsk_plan* p, int kind, int s0, int C, double* dst,
                     cufftDoubleComplex* spec, cudaStream_t st) {
  bind_work(p, p->z2d, st);
  for (int b = 0; b < C; b += p->chunk) {
    const int first = s0 + b;
    const int ns = std::max(0, std::min(p->chunk, p->n - first));
    if (ns == 0) {
      BSK_CHECK_CUDA(cudaMemsetAsync(dst + (size_t)b * p->K, 0,
                                     (size_t)p->chunk * p->K * sizeof(double), st));
      continue;
    }
    if (ns < p->chunk)
      BSK_CHECK_CUDA(cudaMemsetAsync(spec + (size_t)ns * p->Mh, 0,
                                     (size_t)(p->chunk - ns) * p->Mh * sizeof(cufftDoubleComplex),
                                     st));
    launch_filter_indicator(p, first, ns, kind, spec, st);
    BSK_CHECK_CUFFT(cufftExecZ2D(p->z2d, spec, dst + (size_t)b * p->K));
  }
}

// Streamed grid information: per triangle group, the indicator and |k| fields of
// its (at most three) chunks sit in six C-shell FP64 buffers, recomputed only
// when no buffer holds them.  Buffers are freed at the end.
void gridinfo_stream(bsk_plan* p, const bsk_triset* set, double* ntri, double* kmean,
                     cudaStream_t st) {
  const size_t spec_bytes = (size_t)p->chunk * p->Mh * sizeof(cufftDoubleComplex);
  const size_t fixed = spec_bytes + 3 * (size_t)set->T * sizeof(double);
  const int64_t avail = (int64_t)p->mem_budget - footprint(p) - (int64_t)fixed;
  const size_t per_shell = 6 * (size_t)p->K * sizeof(double);
  int C = avail > 0 ? (int)std::min<int64_t>(avail / (int64_t)per_shell, p->n_alloc()) : 0;
  C = C / p->chunk * p->chunk;
  BSK_REQUIRE(C >= p->chunk, BSK_ERR_OOM,
              "grid information: the budget of " + std::to_string(p->mem_budget) +
                  " bytes leaves room for no chunk of " + std::to_string(p->chunk) + " shells");
  const size_t buf_elems = (size_t)C * p->K;
  AsyncTemp pool_t(6 * buf_elems * sizeof(double), st);
  AsyncTemp spec_t(spec_bytes, st);
  AsyncTemp s1_t(3 * (size_t)set->T * sizeof(double), st);
  double* pool = (double*)pool_t.ptr;
  cufftDoubleComplex* spec = (cufftDoubleComplex*)spec_t.ptr;
  double* s1 = (double*)s1_t.ptr;
  double* s2 = s1 + set->T;
  double* s3 = s2 + set->T;
  BSK_CHECK_CUDA(cudaMemsetAsync(ntri, 0, (size_t)set->T * sizeof(double), st));
  BSK_CHECK_CUDA(cudaMemsetAsync(s1, 0, 3 * (size_t)set->T * sizeof(double), st));
  int64_t held[6] = {-1, -1, -1, -1, -1, -1};
  for (const StreamGroup& g : stream_groups(set, C)) {
    const int chunks[3] = {g.ca, g.cb, g.cc};
    const double* f[2][3];  // [kind][role]
    bool keep[6] = {false, false, false, false, false, false};
    for (int kind = 0; kind < 2; ++kind)
      for (int r = 0; r < 3; ++r) {
        f[kind][r] = nullptr;
        const int64_t key = kind * 256 + chunks[r];
        for (int q = 0; q < 6; ++q)
          if (held[q] == key) {
            f[kind][r] = pool + q * buf_elems;
            keep[q] = true;
          }
      }
    for (int kind = 0; kind < 2; ++kind)
      for (int r = 0; r < 3; ++r) {
        if (f[kind][r]) continue;
        int q = 0;
        while (keep[q]) ++q;  // at most six wanted keys: a free buffer exists
        double* dst = pool + q * buf_elems;
        chunk_indicator(p, kind, chunks[r] * C, C, dst, spec, st);
        held[q] = kind * 256 + chunks[r];
        keep[q] = true;
        for (int r2 = r; r2 < 3; ++r2)
          if (chunks[r2] == chunks[r]) f[kind][r2] = dst;
      }
    auto run = [&](const double* x, const double* y, const double* z, double* o) {
      launch_contract_simt_d64(g.sched, x, y, z, C, p->K, 0, p->K, o, p->num_sms, st);
    };
    run(f[0][0], f[0][1], f[0][2], ntri);
    run(f[1][0], f[0][1], f[0][2], s1);
    run(f[0][0], f[1][1], f[0][2], s2);
    run(f[0][0], f[0][1], f[1][2], s3);
  }
  for (double* o : {ntri, s1, s2, s3}) copy_dups(set, o, st);
  launch_gridinfo_finish(set->T, 1.0 / (double)p->K, ntri, s1, s2, s3, kmean, st);
  s1_t.release();
  spec_t.release();
  pool_t.release();
  p->last_stream_C = C;
}

}  // namespace

void set_error(const std::string& msg) { g_err = msg; }
const std::string& get_error() { return g_err; }

}  // namespace bsk

using namespace bsk;

extern "C" {

int bsk_version(void) { return 100; }

int bsk_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return BSK_ERR_ARG;
  size_t n = std::min(len - 1, g_err.size());
  std::memcpy(buf, g_err.data(), n);
  buf[n] = '\0';
  return BSK_OK;
}

int bsk_plan_create(int nmesh, double box_size, int n_shells, const double* shell_edges,
                    int grid_mode, size_t mem_budget, bsk_plan** out) {
  return guarded([&] {
    BSK_REQUIRE(out, BSK_ERR_ARG, "out is NULL");
    *out = nullptr;
    BSK_REQUIRE(nmesh >= 2 && nmesh % 2 == 0, BSK_ERR_ARG, "Nmesh must be even and >= 2");
    BSK_REQUIRE(nmesh <= 2048, BSK_ERR_UNSUPPORTED, "Nmesh above 2048");
    BSK_REQUIRE(std::isfinite(box_size) && box_size > 0, BSK_ERR_ARG, "BoxSize must be > 0");
    BSK_REQUIRE(n_shells >= 1 && n_shells <= 255, BSK_ERR_ARG, "need 1..255 shells");
    BSK_REQUIRE(shell_edges, BSK_ERR_ARG, "shell_edges is NULL");
    BSK_REQUIRE(grid_mode == BSK_GRID_REDUCED || grid_mode == BSK_GRID_NATIVE ||
                    grid_mode == BSK_GRID_REDUCED_SINGLE,
                BSK_ERR_ARG, "bad grid mode");
    // an error before the plan is handed out releases what it holds so far
    std::unique_ptr<bsk_plan, void (*)(bsk_plan*)> p(new bsk_plan(), destroy_plan);
    BSK_CHECK_CUDA(cudaGetDevice(&p->device));
    BSK_CHECK_CUDA(cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount,
                                          p->device));
    p->N = nmesh;
    p->L = box_size;
    p->n = n_shells;
    p->mem_budget = mem_budget;
    p->edges.assign(shell_edges, shell_edges + 2 * n_shells);
    double hi_max = 0.0;
    for (int s = 0; s < n_shells; ++s) {
      BSK_REQUIRE(std::isfinite(p->edges[2 * s]) && std::isfinite(p->edges[2 * s + 1]),
                  BSK_ERR_ARG, "non-finite shell edge");
      if (p->edges[2 * s + 1] >= p->edges[2 * s]) hi_max = std::max(hi_max, p->edges[2 * s + 1]);
    }
    const double kf = 2.0 * 3.14159265358979323846 / box_size;
    double qd = std::floor(hi_max / kf * (1.0 + 1e-9));
    int qmax = (int)std::min<double>(qd, nmesh / 2);
    p->qmax = qmax;
    p->Ng = choose_grid(nmesh, qmax, grid_mode);
    p->K = (int64_t)p->Ng * p->Ng * p->Ng;
    p->Mh = (int64_t)p->Ng * p->Ng * (p->Ng / 2 + 1);
    p->chunk = std::min(n_shells, 8);

    p->table = (uint16_t*)dmalloc((size_t)p->Mh * sizeof(uint16_t));
    p->d_edges = (double*)dmalloc((size_t)2 * n_shells * sizeof(double));
    BSK_CHECK_CUDA(cudaMemcpy(p->d_edges, p->edges.data(), 2 * n_shells * sizeof(double),
                              cudaMemcpyHostToDevice));
    std::vector<unsigned long long> hc(n_shells);
    int hf[2] = {0, 0};
    {
      SyncTemp counts_t(n_shells * sizeof(unsigned long long));
      SyncTemp flag_t(2 * sizeof(int));
      unsigned long long* d_counts = (unsigned long long*)counts_t.ptr;
      int* d_flag = (int*)flag_t.ptr;
      BSK_CHECK_CUDA(cudaMemset(d_counts, 0, n_shells * sizeof(unsigned long long)));
      BSK_CHECK_CUDA(cudaMemset(d_flag, 0, 2 * sizeof(int)));
      launch_shell_table(p.get(), d_counts, d_flag, 0);
      BSK_CHECK_CUDA(cudaMemcpy(hc.data(), d_counts, n_shells * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost));
      BSK_CHECK_CUDA(cudaMemcpy(hf, d_flag, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    }  // both freed here (or by an error unwinding the block)
    BSK_REQUIRE(hf[0] == 0, BSK_ERR_UNSUPPORTED,
                "a Fourier mode lies in shells that are not consecutive; give shells sorted "
                "by edge with overlaps only between neighbours");
    BSK_REQUIRE(hf[1] <= qmax || p->Ng == p->N, BSK_ERR_CUDA,
                "internal: shell mode beyond the reduced-grid bound");
    p->counts.assign(hc.begin(), hc.end());

    p->shell_r.resize(n_shells);
    for (int s = 0; s < n_shells; ++s) {
      const double hi = p->edges[2 * s + 1];
      const double q = hi >= p->edges[2 * s] ? std::floor(hi / kf * (1.0 + 1e-9)) : 0.0;
      p->shell_r[s] = (int)std::min<double>(std::max(q, 0.0), qmax);
    }
    p->use_synth = synth_supported(p->Ng);
    if (p->use_synth) p->synth_ws_bytes = synth_workspace_bytes(p->Ng, qmax, p->chunk);
    p->use_levels = grid_mode == BSK_GRID_REDUCED && p->Ng != p->N && p->use_synth;
    make_r2c(p.get());
    make_c2r(p.get());
    p->chunk_spec = (cufftComplex*)dmalloc((size_t)p->chunk * p->Mh * sizeof(cufftComplex));
    *out = p.release();
  });
}

int bsk_plan_destroy(bsk_plan* plan) {
  return guarded([&] { destroy_plan(plan); });
}

int bsk_plan_query(const bsk_plan* p, int64_t* info) {
  return guarded([&] {
    BSK_REQUIRE(p && info, BSK_ERR_ARG, "NULL argument");
    const int64_t fp = footprint(p);
    info[BSK_INFO_NMESH] = p->N;
    info[BSK_INFO_NGRID] = p->Ng;
    info[BSK_INFO_NSHELLS] = p->n;
    info[BSK_INFO_QMAX] = p->qmax;
    info[BSK_INFO_FOOTPRINT] = fp;
    info[BSK_INFO_CHUNK] = p->chunk;
    info[BSK_INFO_DEVICE] = p->device;
    info[BSK_INFO_STREAM] = p->last_stream_C;
  });
}

int bsk_shell_mode_counts(const bsk_plan* p, int64_t* counts) {
  return guarded([&] {
    BSK_REQUIRE(p && counts, BSK_ERR_ARG, "NULL argument");
    std::copy(p->counts.begin(), p->counts.end(), counts);
  });
}

int bsk_triset_create(bsk_plan* p, int64_t n_tri, const int32_t* tri, bsk_triset** out) {
  return guarded([&] {
    BSK_REQUIRE(p && out, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(n_tri >= 0 && (n_tri == 0 || tri), BSK_ERR_ARG, "bad triangle list");
    BSK_REQUIRE(n_tri < (1ll << 31), BSK_ERR_UNSUPPORTED, "too many triangles");
    *out = nullptr;
    DeviceGuard g(p->device);
    // an error before the set is handed out releases what it holds so far
    std::unique_ptr<bsk_triset, void (*)(bsk_triset*)> s(new bsk_triset(), destroy_triset);
    s->plan = p;
    s->T = n_tri;
    std::map<std::tuple<int, int, int>, int> first;
    std::vector<int2> dups;
    for (int64_t t = 0; t < n_tri; ++t) {
      HostTriangle h{tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]};
      BSK_REQUIRE(h.i >= 0 && h.j >= 0 && h.l >= 0 && h.i < p->n && h.j < p->n && h.l < p->n,
                  BSK_ERR_ARG, "triangle " + std::to_string(t) + " has a shell index outside [0, " +
                                   std::to_string(p->n) + ")");
      s->tri.push_back(h);
      s->max_shell = std::max(s->max_shell, std::max(h.i, std::max(h.j, h.l)));
      auto key = std::make_tuple(h.i, h.j, h.l);
      auto it = first.find(key);
      if (it == first.end()) {
        first.emplace(key, (int)t);
      } else {
        dups.push_back(make_int2((int)t, it->second));
      }
    }
    // schedule over unique triangles; map entries carry the first index
    {
      std::vector<char> is_first(n_tri, 0);
      for (auto& kv : first) is_first[kv.second] = 1;
      for (int64_t t = 0; t < n_tri; ++t)
        if (is_first[t]) {
          s->u_tri.push_back(s->tri[t]);
          s->u_idx.push_back((int)t);
        }
    }
    build_schedule(s->u_tri, p->n, s->sched, &s->u_idx);
    if (p->use_levels && !s->u_tri.empty()) build_levels(p, s.get());
    if (!dups.empty()) {
      s->n_dups = (int)dups.size();
      s->dups = (int2*)dmalloc(dups.size() * sizeof(int2));
      BSK_CHECK_CUDA(cudaMemcpy(s->dups, dups.data(), dups.size() * sizeof(int2),
                                cudaMemcpyHostToDevice));
    }
    *out = s.release();
  });
}

int bsk_triset_levels(const bsk_triset* set, int64_t* out, int cap) {
  int n = -1;
  const int rc = guarded([&] {
    BSK_REQUIRE(set && (cap == 0 || out), BSK_ERR_ARG, "NULL argument");
    n = (int)set->levels.size();
    for (int k = 0; k < n && k < cap; ++k) {
      const GridLevel& lv = set->levels[k];
      int64_t cols = 0, rows = 0;
      for (const TileDesc& d : lv.sched.h_tiles) {
        cols += d.nc;
        rows += d.nrows;
      }
      int64_t* o = out + 6 * k;
      o[0] = lv.plan->Ng;
      o[1] = lv.sched.n_tiles;
      o[2] = cols;
      o[3] = rows;
      o[4] = lv.bins;
      o[5] = lv.n_shells;
    }
  });
  return rc == BSK_OK ? n : rc;
}

int bsk_triset_destroy(bsk_triset* set) {
  return guarded([&] { destroy_triset(set); });
}

int64_t bsk_triset_size(const bsk_triset* set) { return set ? set->T : -1; }

int bsk_triset_schedule(const bsk_triset* set, int64_t* out) {
  return guarded([&] {
    BSK_REQUIRE(set && out, BSK_ERR_ARG, "NULL argument");
    int64_t cols = 0, rows = 0;
    for (const TileDesc& d : set->sched.h_tiles) {
      cols += d.nc;
      rows += d.nrows;
    }
    out[0] = set->sched.n_tiles;
    out[1] = cols;
    out[2] = rows;
  });
}

namespace bsk {
namespace {
// Factors 1/sqrt(1 - 2/3 sin^2(pi q / NmeshCIC)) for q = -N/2..N/2, the per-axis CIC
// window deconvolution of the mesh's source grid.
void ensure_cic_table(bsk_plan* p, int nmesh_cic) {
  if (p->cic_w && p->cic_nmesh == nmesh_cic) return;
  std::vector<float> w(p->N + 1);
  for (int i = 0; i <= p->N; ++i) {
    const int q = i - p->N / 2;
    const double s = std::sin(3.14159265358979323846 * q / nmesh_cic);
    w[i] = (float)(1.0 / std::sqrt(1.0 - 2.0 / 3.0 * s * s));
  }
  if (!p->cic_w) p->cic_w = (float*)dmalloc(w.size() * sizeof(float));
  BSK_CHECK_CUDA(cudaMemcpy(p->cic_w, w.data(), w.size() * sizeof(float),
                            cudaMemcpyHostToDevice));
  p->cic_nmesh = nmesh_cic;
}

// R2C of an N^3 block of a larger nfull^3 mesh, read in place (strided input).
void make_r2c_sub(bsk_plan* p, int nfull) {
  if (p->r2c_sub_nfull == nfull) return;
  if (p->r2c_sub_nfull) cufftDestroy(p->r2c_sub);
  p->r2c_sub_nfull = 0;
  long long n[3] = {p->N, p->N, p->N};
  long long inembed[3] = {nfull, nfull, nfull};
  long long onembed[3] = {p->N, p->N, p->N / 2 + 1};
  const long long idist = (long long)nfull * nfull * nfull;
  const long long odist = (long long)p->N * p->N * (p->N / 2 + 1);
  BSK_CHECK_CUFFT(cufftCreate(&p->r2c_sub));
  p->r2c_sub_nfull = nfull;
  BSK_CHECK_CUFFT(cufftSetAutoAllocation(p->r2c_sub, 0));
  size_t ws = 0;
  BSK_CHECK_CUFFT(cufftMakePlanMany64(p->r2c_sub, 3, n, inembed, 1, idist, onembed, 1, odist,
                                      CUFFT_R2C, 1, &ws));
  grow_work(p, ws);
}

void paint(bsk_plan* p, int slot, const float* mesh, int nmesh_cic, cudaStream_t st,
           int nfull = 0) {
  BSK_REQUIRE(p && mesh, BSK_ERR_ARG, "NULL argument");
  BSK_REQUIRE(slot >= 0 && slot < 3, BSK_ERR_ARG, "slot must be 0, 1 or 2");
  FieldSlot& f = p->slot[slot];
  const float* axis_w = nullptr;
  if (nmesh_cic > 0) {
    ensure_cic_table(p, nmesh_cic);
    axis_w = p->cic_w;
  }
  if (nfull) make_r2c_sub(p, nfull);
  cufftHandle h = nfull ? p->r2c_sub : p->r2c;
  size_t fine_elems = (size_t)p->N * p->N * (p->N / 2 + 1);
  AsyncTemp fine_t(fine_elems * sizeof(cufftComplex), st);
  cufftComplex* fine = (cufftComplex*)fine_t.ptr;
  bind_work(p, h, st);
  BSK_CHECK_CUFFT(cufftExecR2C(h, const_cast<float*>(mesh), fine));
  if (!f.spec) f.spec = (cufftComplex*)dmalloc((size_t)p->Mh * sizeof(cufftComplex));
  launch_extract(p, fine, f.spec, axis_w, st);
  fine_t.release();
  f.painted = true;
  ++f.gen;
  f.fields_ok = false;
  f.split_ok = false;
}
}  // namespace
}  // namespace bsk

int bsk_paint(bsk_plan* p, int slot, const float* mesh, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p, BSK_ERR_ARG, "NULL plan");
    DeviceGuard g(p->device);
    paint(p, slot, mesh, 0, (cudaStream_t)stream);
  });
}

int bsk_paint_cic(bsk_plan* p, int slot, const float* mesh, int nmesh_cic, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p, BSK_ERR_ARG, "NULL plan");
    BSK_REQUIRE(nmesh_cic > 0, BSK_ERR_ARG, "NmeshCIC must be positive");
    DeviceGuard g(p->device);
    paint(p, slot, mesh, nmesh_cic, (cudaStream_t)stream);
  });
}

int bsk_paint_subbox(bsk_plan* p, int slot, const float* mesh, int nmesh_full, int a, int b,
                     int c, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p && mesh, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(nmesh_full >= p->N && nmesh_full % p->N == 0, BSK_ERR_ARG,
                "the full mesh side must be a multiple of the plan's Nmesh");
    const int nsub = nmesh_full / p->N;
    BSK_REQUIRE(a >= 0 && b >= 0 && c >= 0 && a < nsub && b < nsub && c < nsub, BSK_ERR_ARG,
                "sub-box index outside [0, nmesh_full / Nmesh)");
    DeviceGuard g(p->device);
    const int64_t n = p->N, nf = nmesh_full;
    const float* origin = mesh + ((a * n) * nf + b * n) * nf + c * n;
    paint(p, slot, origin, 0, (cudaStream_t)stream, nmesh_full);
  });
}

int bsk_compensate_cic(int nmesh, int nmesh_cic, const float* mesh, float* out, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(mesh && out, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(nmesh >= 2 && nmesh % 2 == 0 && nmesh <= 4096, BSK_ERR_ARG,
                "Nmesh must be even, 2..4096");
    BSK_REQUIRE(nmesh_cic > 0, BSK_ERR_ARG, "NmeshCIC must be positive");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    BSK_CHECK_CUDA(cudaGetDevice(&dev));
    BSK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    std::vector<float> w(nmesh + 1);
    for (int i = 0; i <= nmesh; ++i) {
      const double sn = std::sin(3.14159265358979323846 * (i - nmesh / 2) / nmesh_cic);
      w[i] = (float)(1.0 / std::sqrt(1.0 - 2.0 / 3.0 * sn * sn));
    }
    const size_t mh = (size_t)nmesh * nmesh * (nmesh / 2 + 1);
    cufftHandle fwd = 0, inv = 0;
    bool fwd_ok = false, inv_ok = false;
    float* dw = nullptr;
    cufftComplex* spec = nullptr;
    try {
      BSK_CHECK_CUFFT(cufftPlan3d(&fwd, nmesh, nmesh, nmesh, CUFFT_R2C));
      fwd_ok = true;
      BSK_CHECK_CUFFT(cufftPlan3d(&inv, nmesh, nmesh, nmesh, CUFFT_C2R));
      inv_ok = true;
      BSK_CHECK_CUFFT(cufftSetStream(fwd, st));
      BSK_CHECK_CUFFT(cufftSetStream(inv, st));
      dw = (float*)dmalloc_async(w.size() * sizeof(float), st);
      spec = (cufftComplex*)dmalloc_async(mh * sizeof(cufftComplex), st);
      BSK_CHECK_CUDA(cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(float),
                                     cudaMemcpyHostToDevice, st));
      BSK_CHECK_CUFFT(cufftExecR2C(fwd, const_cast<float*>(mesh), spec));
      launch_window(nmesh, (float)(1.0 / ((double)nmesh * nmesh * nmesh)), spec, dw, sms, st);
      BSK_CHECK_CUFFT(cufftExecC2R(inv, spec, out));
      // the host table must outlive its copy; the plans are destroyed after the work
      BSK_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      if (spec) cudaFreeAsync(spec, st);
      if (dw) cudaFreeAsync(dw, st);
      if (fwd_ok) cufftDestroy(fwd);
      if (inv_ok) cufftDestroy(inv);
      throw;
    }
    BSK_CHECK_CUDA(cudaFreeAsync(spec, st));
    BSK_CHECK_CUDA(cudaFreeAsync(dw, st));
    cufftDestroy(fwd);
    cufftDestroy(inv);
  });
}

int bsk_measure_b(bsk_plan* p, const bsk_triset* set, int a, int b, int c, int precision,
                  double* out, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p, BSK_ERR_ARG, "NULL plan");
    DeviceGuard g(p->device);
    measure_b(p, set, a, b, c, precision, 0, p->K, out, (cudaStream_t)stream);
  });
}

int bsk_measure_b_range(bsk_plan* p, const bsk_triset* set, int a, int b, int c, int precision,
                        int64_t k_begin, int64_t k_end, double* out, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p, BSK_ERR_ARG, "NULL plan");
    DeviceGuard g(p->device);
    measure_b(p, set, a, b, c, precision, k_begin, k_end, out, (cudaStream_t)stream);
  });
}

int bsk_contract(bsk_plan* p, const bsk_triset* set, const float* f1, const float* f2,
                 const float* f3, int64_t K, int precision, double* out, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p && set && f1 && f2 && f3, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(((uintptr_t)f1 | (uintptr_t)f2 | (uintptr_t)f3) % 16 == 0, BSK_ERR_ARG,
                "field pointers must be 16-byte aligned");
    BSK_REQUIRE(set->plan == p, BSK_ERR_ARG, "triangle set belongs to another plan");
    BSK_REQUIRE(K > 0 && K % 8 == 0, BSK_ERR_ARG, "k_points must be a positive multiple of 8");
    BSK_REQUIRE(precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16 ||
                    precision == BSK_PREC_FP32 || precision == BSK_PREC_FP64,
                BSK_ERR_ARG, "unknown precision " + std::to_string(precision));
    DeviceGuard g(p->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (set->T == 0) return;  // nothing to write: out may be NULL
    BSK_REQUIRE(out, BSK_ERR_ARG, "NULL argument");
    std::unique_ptr<AsyncTemp> split_t;
    __nv_bfloat16* split = nullptr;
    if (precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16) {
      split_t.reset(new AsyncTemp(split_elems(p->n, K) * sizeof(__nv_bfloat16), st));
      split = (__nv_bfloat16*)split_t->ptr;
      launch_split(f3, p->n, K, split, st);
    }
    contract_dispatch(p, set, f1, f2, f3, split, p->n, K, 0, K, precision, out, st);
    if (split_t) split_t->release();
  });
}

int bsk_gridinfo(bsk_plan* p, const bsk_triset* set, double* ntri, double* kmean,
                 void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p && set, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(set->plan == p, BSK_ERR_ARG, "triangle set belongs to another plan");
    DeviceGuard g(p->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (set->T == 0) return;  // nothing to write: ntri and kmean may be NULL
    BSK_REQUIRE(ntri && kmean, BSK_ERR_ARG, "NULL argument");
    if (gridinfo_enum_supported(p)) {  // exact integer enumeration, no FFT
      p->last_stream_C = 0;
      gridinfo_enum(p, set->tri, ntri, kmean, st);
      return;
    }
    make_z2d(p);
    bind_work(p, p->z2d, st);
    const size_t fbytes = (size_t)p->n_alloc() * p->K * sizeof(double);
    const size_t spec_bytes = (size_t)p->chunk * p->Mh * sizeof(cufftDoubleComplex);
    if (p->mem_budget && footprint(p) + (int64_t)(2 * fbytes + spec_bytes + 24 * set->T) >
                             (int64_t)p->mem_budget) {
      gridinfo_stream(p, set, ntri, kmean, st);
      return;
    }
    p->last_stream_C = 0;
    AsyncTemp nf_t(fbytes, st);
    AsyncTemp kf_t(fbytes, st);
    double* nf = (double*)nf_t.ptr;
    double* kf = (double*)kf_t.ptr;
    AsyncTemp spec_t((size_t)p->chunk * p->Mh * sizeof(cufftDoubleComplex), st);
    cufftDoubleComplex* spec = (cufftDoubleComplex*)spec_t.ptr;
    for (int kw = 0; kw < 2; ++kw) {
      double* dst = kw ? kf : nf;
      for (int s0 = 0; s0 < p->n; s0 += p->chunk) {
        int ns = std::min(p->chunk, p->n - s0);
        if (ns < p->chunk)
          BSK_CHECK_CUDA(cudaMemsetAsync(
              spec + (size_t)ns * p->Mh, 0,
              (size_t)(p->chunk - ns) * p->Mh * sizeof(cufftDoubleComplex), st));
        launch_filter_indicator(p, s0, ns, kw, spec, st);
        BSK_CHECK_CUFFT(cufftExecZ2D(p->z2d, spec, dst + (size_t)s0 * p->K));
      }
    }
    spec_t.release();
    AsyncTemp s1_t((size_t)3 * set->T * sizeof(double), st);
    double* s1 = (double*)s1_t.ptr;
    double* s2 = s1 + set->T;
    double* s3 = s2 + set->T;
    auto run = [&](const double* a, const double* b, const double* c, double* o) {
      BSK_CHECK_CUDA(cudaMemsetAsync(o, 0, (size_t)set->T * sizeof(double), st));
      launch_contract_simt_d64(set->sched, a, b, c, p->n, p->K, 0, p->K, o, p->num_sms, st);
      copy_dups(set, o, st);
    };
    run(nf, nf, nf, ntri);
    run(kf, nf, nf, s1);
    run(nf, kf, nf, s2);
    run(nf, nf, kf, s3);
    launch_gridinfo_finish(set->T, 1.0 / (double)p->K, ntri, s1, s2, s3, kmean, st);
    s1_t.release();
    nf_t.release();
    kf_t.release();
  });
}

int bsk_normalize(int64_t n, const double* b, const double* ntri, double* out, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(n >= 0 && (n == 0 || (b && ntri && out)), BSK_ERR_ARG, "bad argument");
    if (n) launch_normalize(n, b, ntri, out, (cudaStream_t)stream);
  });
}

int bsk_copy_field(bsk_plan* p, int slot, int shell, float* dst, void* stream) {
  return guarded([&] {
    BSK_REQUIRE(p && dst, BSK_ERR_ARG, "NULL argument");
    BSK_REQUIRE(slot >= 0 && slot < 3 && shell >= 0 && shell < p->n, BSK_ERR_ARG,
                "bad slot or shell");
    DeviceGuard g(p->device);
    cudaStream_t st = (cudaStream_t)stream;
    ensure_fields(p, slot, st);
    BSK_CHECK_CUDA(cudaMemcpyAsync(dst, p->slot[slot].fields + (size_t)shell * p->K,
                                   (size_t)p->K * sizeof(float), cudaMemcpyDeviceToDevice, st));
  });
}

int bsk_sync_check(void* stream) {
  return guarded([&] {
    BSK_CHECK_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    if (tc_error_flag(true))
      throw Error{BSK_ERR_TIMEOUT, "tcgen05 contraction: a bounded pipeline wait expired"};
  });
}

}  // extern "C"
