// Internal declarations of the GB300 bispectrum engine (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <map>
#include <string>
#include <vector>

#include "../../include/bskit_gb300.h"

struct bsk_plan;

namespace bsk {

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
const std::string& get_error();

struct Error {
  int code;
  std::string msg;
};

#define BSK_CHECK_CUDA(expr)                                                             \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess)                                                               \
      throw ::bsk::Error{BSK_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)}; \
  } while (0)

#define BSK_CHECK_CUFFT(expr)                                                       \
  do {                                                                              \
    cufftResult _r = (expr);                                                        \
    if (_r != CUFFT_SUCCESS)                                                        \
      throw ::bsk::Error{BSK_ERR_CUFFT, std::string(#expr) + ": cufft status " +    \
                                            std::to_string((int)_r)};               \
  } while (0)

#define BSK_REQUIRE(cond, code, msg)                          \
  do {                                                        \
    if (!(cond)) throw ::bsk::Error{(code), std::string(msg)}; \
  } while (0)

// ---------------------------------------------------------------- schedule
// Rows of a tile are (i, j) shell pairs; columns are a contiguous range of
// third shells [l0, l0 + nc).  One tile = 128 rows (the tcgen05 M).
constexpr int kTileRows = 128;
constexpr int kMaxCols = 64;    // accumulator columns per tile (register budget of the drain)
constexpr int kMaxSrcRows = 64; // shells per A-source range (one 64-row TMA box)

struct TileDesc {
  int i0, j0, l0;     // first shell of the F1 rows range, F2 rows range, F3 column range
  int ni, nj, nc;     // extents (multiples of 8: nc <= 64; ni, nj <= 64; i0 == j0 when one
                      // 64-shell range covers both pair factors)
  int nrows;          // valid rows
  int row_off;        // offset of this tile's 128 row entries
  int map_off;        // offset of this tile's nc*128 map entries, layout [c][r]
  int pad;
};

struct DeviceSchedule {
  int n_tiles = 0;
  int sum_nc = 0;
  TileDesc* tiles = nullptr;   // device
  int16_t* row_i = nullptr;    // device, absolute shell index, -1 = padding row
  int16_t* row_j = nullptr;
  int32_t* map = nullptr;      // device, triangle index or -1
  int2* subs = nullptr;        // device, SIMT sub-tiles (tile, first column), 32 columns each
  int n_sub = 0;
  std::vector<TileDesc> h_tiles;
  void release();
};

struct HostTriangle {
  int i, j, l;
};

// The tile schedule of a triangle list in host memory: per tile a TileDesc, kTileRows
// pair-row shells (-1 = padding) and an nc x kTileRows map of triangle indices (-1 = not
// a bin).
struct HostSchedule {
  std::vector<TileDesc> tiles;
  std::vector<int16_t> ri, rj;
  std::vector<int32_t> map;
  int sum_nc = 0;
};

// Tile a triangle list (host only).  `n_shells` bounds the indices.  Rows with identical
// (i, j) share one pair product; the list must not repeat an (i, j, l).  Map entries are
// positions in `tri`, or map_index[position] when map_index is given.
void tile_schedule(const std::vector<HostTriangle>& tri, int n_shells,
                   const std::vector<int>* map_index, HostSchedule& out);

// tile_schedule, uploaded to the device (with the SIMT kernels' sub-tile list).
// Grid levels of a triangle set: per triangle the index in `sides` (ascending, the plan's
// own grid last) of the side it is contracted on (host only, bsk_schedule.cu).
std::vector<int> choose_level_sides(const std::vector<HostTriangle>& tri,
                                    const std::vector<int>& shell_r,
                                    const std::vector<int>& sides, int n_shells,
                                    double tile_cost, double shell_cost);
void build_schedule(const std::vector<HostTriangle>& tri, int n_shells, DeviceSchedule& out,
                    const std::vector<int>* map_index = nullptr);

// Shell streaming: the triangles whose shells fall in chunks (ca, cb, cc) of C
// shells each, scheduled with shell indices relative to their chunk.
struct StreamGroup {
  int ca = 0, cb = 0, cc = 0;
  DeviceSchedule sched;
};

// Device buffers of C shells each that hold streamed shell fields, with the
// identity of what each holds (-1 = nothing).
struct StreamBuf {
  void* ptr = nullptr;
  int64_t key = -1;
};

// ---------------------------------------------------------------- plan
// The bf16 hi / lo split of S shell fields over K points is stored chunk-major:
// [ceil(K / 128) chunks][hi, lo][S shells][128 points], so that the column tiles of one
// 128-point contraction stage (nc shells, both planes) are one contiguous block for TMA
// (256-byte pieces of rows a plane apart were ~20% slower to stream).  The tail of the last
// chunk (points K .. 128 ceil(K / 128)) is zero.
inline size_t split_elems(int S, int64_t K) { return (size_t)((K + 127) / 128) * 256 * S; }
__host__ __device__ __forceinline__ int64_t split_index(int plane, int s, int64_t x, int S) {
  return (x >> 7) * (256 * (int64_t)S) + ((int64_t)plane * S + s) * 128 + (x & 127);
}

struct FieldSlot {
  bool painted = false;
  cufftComplex* spec = nullptr;   // coarse half spectrum, scaled 1/N^3 (Ng*Ng*(Ng/2+1))
  float* fields = nullptr;        // [n][K] FP32 shell fields (nullptr until built)
  __nv_bfloat16* split = nullptr; // bf16 split of the n_alloc shells, chunk-major (above)
  bool fields_ok = false;
  bool split_ok = false;
  int fields_n = 0;               // the FP32 fields of shells [fields_from, fields_n) are valid
  int fields_from = 0;            // (0 unless a grid level only needed the later shells)
  int split_n = 0;                // the split of shells [0, split_n) is valid
  int64_t gen = 0;                // bumped by every paint (keys of streamed fields); on a grid
                                  // level's plan: the parent paint its spectrum was taken from
};

// One contraction grid of a triangle set: the bins whose three shells sum to less than the
// grid side are contracted on it (exact: q1 + q2 + q3 cannot wrap around), with the shell
// fields of the grid's plan (the set's own plan, or one of its grid-level plans).
struct GridLevel {
  bsk_plan* plan = nullptr;
  DeviceSchedule sched;   // map entries are positions in the set's output
  int n_shells = 0;       // shells [0, n_shells) the level's bins use
  int src_min = 0;        // smallest shell of the level's bins used as a pair factor (i or j)
  int64_t bins = 0;
};

}  // namespace bsk

struct bsk_plan {
  int device = 0;
  int N = 0;       // mesh side
  int Ng = 0;      // contraction grid side
  int n = 0;       // shells
  int qmax = 0;    // largest |q_c| of a mode in any shell
  double L = 0.0;
  size_t mem_budget = 0;
  int chunk = 0;   // shells per FFT batch
  std::vector<double> edges;  // 2n
  std::vector<int64_t> counts;
  int64_t K = 0;        // Ng^3
  int64_t Mh = 0;       // Ng*Ng*(Ng/2+1) half-complex modes
  uint16_t* table = nullptr;  // device [Mh] shell code
  double* d_edges = nullptr;  // device [2n]
  cufftHandle r2c = 0;        // N^3 R2C
  bool r2c_ok = false;
  cufftHandle r2c_sub = 0;    // N^3 R2C of a block of a larger mesh (strided input)
  int r2c_sub_nfull = 0;      // side of that larger mesh (0 = no plan)
  cufftHandle c2r = 0;        // Ng^3 C2R, batch = chunk
  bool c2r_ok = false;
  cufftHandle z2d = 0;        // Ng^3 Z2D, batch = chunk (grid info)
  bool z2d_ok = false;
  bsk::FieldSlot slot[3];
  cufftComplex* chunk_spec = nullptr;   // [chunk][Mh] masked spectra
  int num_sms = 0;
  float* cic_w = nullptr;               // per-axis CIC compensation factors, N+1 entries
  int cic_nmesh = 0;                    // NmeshCIC the table was built for
  void* work = nullptr;                 // cuFFT work area shared by the plan's transforms
  size_t work_bytes = 0;
  // shell streaming (used when the resident fields would exceed mem_budget)
  int stream_C = 0;                     // shells per streamed chunk (0 = buffers not held)
  bool stream_tc = false;               // buffers include the bf16 split
  bsk::StreamBuf stream_f[3];           // FP32 [C][K] each
  bsk::StreamBuf stream_split;          // bf16 hi [C][K] then lo [C][K]
  int last_stream_C = 0;                // chunk of the last streamed measurement (0 = resident)
  // field synthesis (pruned FFT passes) instead of filter + cuFFT C2R
  bool use_synth = false;
  std::vector<int> shell_r;             // largest |q_c| of a mode in each shell
  void* synth_ws = nullptr;             // twiddles + X / Y pass intermediates of one batch
  size_t synth_ws_bytes = 0;
  // grid levels: smaller contraction grids for bins of small shells (owned by the plan);
  // a level's plan has `parent` set, takes its spectra from the parent's slots and holds a
  // prefix of the parent's shells
  bool use_levels = false;
  bsk_plan* parent = nullptr;
  std::vector<bsk_plan*> levels;
  int n_alloc() const { return (n + chunk - 1) / chunk * chunk; }  // shells rounded to batches
};

struct bsk_triset {
  bsk_plan* plan = nullptr;
  int64_t T = 0;
  std::vector<bsk::HostTriangle> tri;
  int max_shell = -1;
  bsk::DeviceSchedule sched;
  int2* dups = nullptr;  // device (dst, src): repeated triangles copy the first occurrence
  int n_dups = 0;
  std::vector<bsk::HostTriangle> u_tri;  // first occurrences, in order
  std::vector<int> u_idx;                // their positions in the list
  mutable std::map<int, std::vector<bsk::StreamGroup>> groups;  // per streaming chunk size
  std::vector<bsk::GridLevel> levels;    // the resident path's grids (empty: the plan's only)
};

namespace bsk {

// ---------------------------------------------------------------- kernels
// Shell table + exact mode counts (FP64 predicate, Hermitian weights).
void launch_shell_table(const bsk_plan* p, unsigned long long* d_counts, int* d_flag,
                        cudaStream_t st);
// Copy the |q_c| < Ng/2 modes of an N^3 half spectrum into the Ng half grid,
// scaled by 1/N^3.
// axis_w: optional per-axis window factors indexed by q + N/2 (NULL = none).
void launch_extract(const bsk_plan* p, const cufftComplex* fine, cufftComplex* coarse,
                    const float* axis_w, cudaStream_t st);
// Masked spectra of shells [s0, s0+ns) into out[ns][Mh].
void launch_filter(const bsk_plan* p, const cufftComplex* spec, int s0, int ns,
                   cufftComplex* out, cudaStream_t st);
// Indicator (or |k|-weighted when kweight) spectra, complex128.
void launch_filter_indicator(const bsk_plan* p, int s0, int ns, int kweight,
                             cufftDoubleComplex* out, cudaStream_t st);
// In-place scale * w[qa] w[qb] w[qc] of an N^3 half spectrum (window deconvolution).
void launch_window(int N, float scale, cufftComplex* spec, const float* axis_w, int num_sms,
                   cudaStream_t st);
// Field synthesis: fields (and optionally the hi / lo planes) of shells [s0, s0 + ns)
// from the slot spectrum by three pruned FFT passes; R = largest |q_c| of those shells.
// Shell s is written at fields[(s - out_s0) K].
bool synth_supported(int n);
size_t synth_workspace_bytes(int n, int max_r, int batch);
// Twiddle table at the start of the workspace (synchronous; once, after allocation).
void synth_init_workspace(int n, void* work);
void launch_synth(int N, const cufftComplex* spec, const uint16_t* table, int s0, int ns, int R,
                  void* work, float* fields, __nv_bfloat16* split, int split_shells,
                  cudaStream_t st, int out_s0 = 0, int fields_from = 0);
// FP32 fields [S][K] -> their chunk-major bf16 hi / lo split (split_elems(S, K) values,
// the tail of the last chunk zeroed).
void launch_split(const float* in, int S, int64_t K, __nv_bfloat16* split, cudaStream_t st);

// SIMT contraction (Tin = float|double input fields, Tacc = float|double tile sums).
// out[t] += scale * sum over K of f1[i] f2[j] f3[l]  (out must be zeroed by the caller).
void launch_contract_simt_f32(const DeviceSchedule& s, const float* f1, const float* f2,
                              const float* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale = 1.0);
void launch_contract_simt_f64(const DeviceSchedule& s, const float* f1, const float* f2,
                              const float* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale = 1.0);
void launch_contract_simt_d64(const DeviceSchedule& s, const double* f1, const double* f2,
                              const double* f3, int n_shells, int64_t K, int64_t k_begin,
                              int64_t k_end, double* out, int num_sms, cudaStream_t st,
                              double scale = 1.0);

// tcgen05 contraction: f1/f2 FP32 (pair-product sources), f3 as bf16 hi/lo.
void launch_contract_tc(const DeviceSchedule& s, const float* f1, const float* f2,
                        const __nv_bfloat16* f3_split, int split_shells, int n_shells,
                        int64_t K, int64_t k_begin, int64_t k_end, int terms, double* out,
                        int num_sms, cudaStream_t st, double scale = 1.0);

// Bounded-wait error flag of the tcgen05 kernel (1 = a wait expired); optionally reset.
int tc_error_flag(bool reset);

// Grid information by exact lattice enumeration (counts and |k| sums in integers) for
// plans whose shell modes cannot form a triangle that wraps around the grid and that have
// at most 64 shells; ntri[T], kmean[T][3] (device).  Synchronises `st`.
bool gridinfo_enum_supported(const bsk_plan* p);
void gridinfo_enum(bsk_plan* p, const std::vector<HostTriangle>& tri, double* ntri,
                   double* kmean, cudaStream_t st);

void launch_scale(double* v, int64_t n, double s, cudaStream_t st);
// A grid level's coarse spectrum from its parent plan's coarse spectrum.
void launch_subgrid(const bsk_plan* parent, const bsk_plan* level, const cufftComplex* ps,
                    cufftComplex* ls, cudaStream_t st);
// Grid sizes the field synthesis compiles with constant strides (candidate grid levels).
bool synth_fast_size(int n);
void launch_gridinfo_finish(int64_t T, double inv_k, double* ntri, const double* s1,
                            const double* s2, const double* s3, double* kmean,
                            cudaStream_t st);
void launch_normalize(int64_t n, const double* b, const double* ntri, double* out,
                      cudaStream_t st);

}  // namespace bsk
