/*
 * bskit_gb300.h -- C ABI of the GB300 (sm_103a) FFT-bispectrum engine.
 *
 * This is the drop-in boundary below the Python `FFTBispectrum` class.  The
 * upstream package (sjforeman/bskit) is pure Python over nbodykit/pmesh/MPI
 * and has no FFI of its own, so every entry point below names the upstream
 * Python call whose work it replaces (file:line inside the bskit project).
 *
 * Conventions
 *  - Every function returns an int status (BSK_OK == 0); no exception or
 *    C++ object crosses the ABI.  bsk_last_error() gives the text of the
 *    last failure on the calling thread.
 *  - Meshes are real float32 N^3 arrays in C order (x slowest, z fastest),
 *    resident in device memory and owned by the caller.  Output vectors are
 *    caller-owned device buffers of float64.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *    Work is enqueued on that stream; the host does not synchronise except
 *    in bsk_plan_create / bsk_triset_create / bsk_shell_mode_counts /
 *    bsk_compensate_cic / bsk_sync_check / bsk_gridinfo (enumeration path) /
 *    bsk_contract_noalloc (which waits for its own schedule copies on `stream`
 *    and so cannot be captured).
 *  - A plan is bound to the CUDA device that was current at creation.
 *    Calls on one plan must be serialised by the caller; distinct plans may
 *    run on distinct streams concurrently.
 *  - Shell membership of a mode q (integer FFT frequency) is
 *        kk = sqrt((kx*kx + ky*ky) + kz*kz),  k_c = q_c * (2*pi/L)   [float64]
 *        lo <= kk <= hi                                          (closed)
 *    evaluated with correctly rounded float64 operations (no FMA).
 */
#ifndef BSKIT_GB300_H
#define BSKIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bsk_plan bsk_plan;
typedef struct bsk_triset bsk_triset;

enum bsk_status {
  BSK_OK = 0,
  BSK_ERR_ARG = 1,          /* invalid argument (same cases bskit raises ValueError for) */
  BSK_ERR_OOM = 2,          /* device allocation failed or footprint above the budget     */
  BSK_ERR_CUDA = 3,         /* CUDA runtime error                                         */
  BSK_ERR_CUFFT = 4,        /* cuFFT error                                                */
  BSK_ERR_TIMEOUT = 5,      /* a bounded device wait gave up                              */
  BSK_ERR_UNSUPPORTED = 6,  /* valid request outside what this build implements           */
  BSK_ERR_STATE = 7         /* call out of order (e.g. measure before paint)              */
};

/* Arithmetic of the triple-product contraction. */
enum bsk_precision {
  BSK_PREC_FP64 = 0,    /* FP64 SIMT on the FP32 shell fields (the FP64 yardstick)      */
  BSK_PREC_FP32 = 1,    /* plain FP32 SIMT, FP64 cross-slice sum                        */
  BSK_PREC_BF16X3 = 2,  /* tcgen05 bf16 hi*hi + hi*lo + lo*hi, FP32 accumulate, FP64 sum */
  BSK_PREC_BF16 = 3     /* tcgen05 bf16 hi*hi only                                      */
};

/* Real-space grid the contraction runs on. */
enum bsk_grid_mode {
  BSK_GRID_REDUCED = 0, /* smallest FFT-friendly Ng with Ng > 3*max|q_c| (exact: no aliasing onto the summed k=0 mode);
                           bins of small shells on smaller grids (grid levels, bsk_triset_levels) */
  BSK_GRID_NATIVE = 1,  /* Ng = N, the mesh's own grid                                   */
  BSK_GRID_REDUCED_SINGLE = 2 /* the reduced grid for every bin (no grid levels)          */
};

/* bsk_plan_query() fields */
enum bsk_info {
  BSK_INFO_NMESH = 0, BSK_INFO_NGRID = 1, BSK_INFO_NSHELLS = 2, BSK_INFO_QMAX = 3,
  BSK_INFO_FOOTPRINT = 4, BSK_INFO_CHUNK = 5, BSK_INFO_DEVICE = 6, BSK_INFO_STREAM = 7,
  BSK_INFO_COUNT = 8
};

/* Library version (major*10000 + minor*100 + patch). */
int bsk_version(void);

/* Copy the last error message of this thread into buf (NUL-terminated). */
int bsk_last_error(char* buf, size_t len);

/*
 * Create a plan for an N^3 mesh in a periodic box of side L with n shells
 * [edges[2s], edges[2s+1]].  Builds the per-mode shell table on the device,
 * the exact per-shell mode counts and the cuFFT plans.
 * mem_budget: bytes of device memory the plan may hold (0 = no limit).  When
 * the resident shell fields of a measurement (all n shells of each slot, plus
 * their bf16 split) would take the plan's footprint (BSK_INFO_FOOTPRINT) above
 * it, bsk_measure_b(_range) and bsk_gridinfo stream the fields instead: shells
 * are cut into chunks of C (a multiple of BSK_INFO_CHUNK, as large as the budget
 * allows), the triangles are grouped by the chunks of their three shells, and
 * each group runs on the fields of at most three chunks, recomputed from the
 * painted spectrum when a chunk is needed again.  BSK_INFO_STREAM reports the C
 * of the last measurement (0 = resident).  Any other allocation that would
 * exceed the budget, or a budget too small for one chunk, fails with
 * BSK_ERR_OOM before allocating and leaves the plan usable.
 * Replaces: FFTBispectrum.__init__ bin set-up, bskit/main.py:1485-1595, and
 *           the k-mask closures of main.py:1848-1852 / 264-268 / 314-320.
 */
int bsk_plan_create(int nmesh, double box_size, int n_shells, const double* shell_edges,
                    int grid_mode, size_t mem_budget, bsk_plan** out);

/* Release every device resource of the plan.  Replaces: object teardown. */
int bsk_plan_destroy(bsk_plan* plan);

/* info[BSK_INFO_COUNT] <- N, Ng, n, qmax, footprint bytes, shell chunk, device,
 * streaming chunk of the last measurement. */
int bsk_plan_query(const bsk_plan* plan, int64_t* info);

/*
 * counts[n] <- number of full-grid Fourier modes in each shell (exact int64).
 * Replaces: pk_FFT's N_modes = sum(number_field**2)/N^3, bskit/main.py:367-370.
 */
int bsk_shell_mode_counts(const bsk_plan* plan, int64_t* counts);

/*
 * Register a list of T triangle bins (host int32 [T][3] shell indices) and
 * build its contraction schedule on the plan's device.  T may be 0 (tri may
 * then be NULL): bsk_measure_b(_range), bsk_gridinfo and bsk_contract check
 * their other arguments, launch nothing and accept NULL output pointers for an
 * empty set, as bskit's measurement loops run zero times for imin == imax.
 * Replaces: FFTBispectrum.k_indices set-up, bskit/main.py:1553-1584.
 */
int bsk_triset_create(bsk_plan* plan, int64_t n_tri, const int32_t* tri, bsk_triset** out);
int bsk_triset_destroy(bsk_triset* set);
/* Number of triangles in a set. */
int64_t bsk_triset_size(const bsk_triset* set);
/*
 * Contraction schedule of a set: out[0] = tiles (128 pair rows each), out[1] = sum of
 * the tiles' column counts, out[2] = pair rows: the distinct (i, j), a pair whose
 * third shells span more than a tile's 64 columns counting once per run of at most 64.
 * The tensor-core contraction issues 2 x 128 x 3 x out[1] flops per grid point for
 * bf16x3 (useful: 2 x T).  Diagnostics; no counterpart in the reference.
 */
int bsk_triset_schedule(const bsk_triset* set, int64_t* out);
/*
 * Grid levels of a set (plans made with BSK_GRID_REDUCED): a bin (i, j, l) is contracted on
 * the smallest chosen grid side Ng with Ng > r_i + r_j + r_l and 2 r < Ng for its shells
 * (r = largest |q_c| of a shell mode), which is exact -- no closed triangle of shell modes
 * wraps around such a grid -- at a cost proportional to Ng^3; the sides are chosen to
 * minimise contraction plus field-synthesis work.  Returns the number of levels (0: one
 * grid, the plan's) or a negative error; for the first `cap` levels, out[6k .. 6k+5] =
 * Ng, tiles, sum of tile columns, pair rows, bins, shells synthesised.  Used by the
 * resident bsk_measure_b(_range) path (shell streaming keeps the plan's grid).
 * Diagnostics; no counterpart in the reference (its FFTs run on the mesh's grid).
 */
int bsk_triset_levels(const bsk_triset* set, int64_t* out, int cap);

/*
 * Forward-transform a real mesh into field slot `slot` (0, 1, 2 = the
 * reference's first / second / third source).  Invalidates that slot's
 * cached shell fields.
 * Replaces: FFTBispectrum._paint_meshes (mesh.paint(mode='complex')),
 *           bskit/main.py:1608-1621.
 */
int bsk_paint(bsk_plan* plan, int slot, const float* mesh, void* stream);

/*
 * As bsk_paint, deconvolving the CIC window of the grid the mesh was assigned
 * on: every mode is divided by prod_c sqrt(1 - 2/3 sin^2(pi q_c / nmesh_cic)).
 * Replaces: mesh.apply(CompensateCICShotnoiseNgrid, kind='circular',
 *           mode='complex'), scripts/measure/measure_bs_fast.py:45-57, 218-223.
 */
int bsk_paint_cic(bsk_plan* plan, int slot, const float* mesh, int nmesh_cic, void* stream);

/*
 * As bsk_paint for the sub-box (a, b, c) of a larger mesh: the plan's N^3 block
 * whose first point is (a N, b N, c N) in the nmesh_full^3 float32 array `mesh`
 * (nmesh_full a multiple of N).  The block is transformed where it lies (a
 * strided R2C); nothing is copied out of the full mesh.
 * Replaces: field_subbox_pm (bskit/main.py:83-147, a nearest-grid-point cut of
 *           the sub-region) + the sub-box FFTBispectrum's _paint_meshes,
 *           scripts/measure/measure_subbox_bs_fast.py:262-284.
 */
int bsk_paint_subbox(bsk_plan* plan, int slot, const float* mesh, int nmesh_full, int a, int b,
                     int c, void* stream);

/*
 * CIC window deconvolution of a whole float32 nmesh^3 mesh assigned on an
 * nmesh_cic^3 grid: out = c2r[ r2c(mesh) / N^3 / prod_c sqrt(1 - 2/3
 * sin^2(pi q_c / nmesh_cic)) ] (out may equal mesh).  Used before sub-boxes are
 * cut, as the reference compensates the full mesh first.  Creates and destroys
 * its own cuFFT plans and temporary spectrum; returns after the work is done.
 * Replaces: mesh.apply(CompensateCICShotnoiseNgrid, ...) + mesh.compute(mode=
 *           'real'), scripts/measure/measure_subbox_bs_fast.py:45-57, 236-246.
 */
int bsk_compensate_cic(int nmesh, int nmesh_cic, const float* mesh, float* out, void* stream);

/*
 * Unnormalised bispectrum of every triangle of `set`:
 *   out[t] = sum_x I^{a}_{i_t}(x) I^{b}_{j_t}(x) I^{c}_{l_t}(x) * L^6 / N^3
 * where I^{s}_i is slot s's field filtered to shell i (pmesh convention:
 * r2c / N^3, c2r unnormalised).  (a, b, c) = (0,0,0) auto, (0,0,1) <AAB>,
 * (0,1,2) <ABC>.  Shell fields are built (filter kernel + cuFFT C2R) on
 * first use after bsk_paint and cached.
 * Replaces: FFTBispectrum.measure_bispectrum_faster, bskit/main.py:1784-1938
 *           (shell loop 1846-1861, triangle sums 1871-1879) and
 *           compute_bk_FFT_value, main.py:570-672.
 */
int bsk_measure_b(bsk_plan* plan, const bsk_triset* set, int slot_a, int slot_b, int slot_c,
                  int precision, double* b_unnorm, void* stream);

/*
 * As bsk_measure_b, restricted to the contraction-grid points
 * [k_begin, k_end) of the C-ordered Ng^3 grid (an x-slab when the bounds are
 * multiples of Ng^2): partial sums that add up, over a partition of
 * [0, Ng^3), to bsk_measure_b's result.  Each GPU of a slab-sharded job calls
 * this for its slab and the partial vectors are summed (all-reduce).  The
 * tensor-core precisions need k_begin and k_end at multiples of 128 (k_end may
 * also be Ng^3), their pipeline stage.
 * Replaces: the per-rank local sums of bskit's MPI slabs, main.py:1875-1879.
 */
int bsk_measure_b_range(bsk_plan* plan, const bsk_triset* set, int slot_a, int slot_b,
                        int slot_c, int precision, int64_t k_begin, int64_t k_end,
                        double* b_unnorm, void* stream);

/*
 * Grid information of every triangle: ntri[t] = exact triangle count,
 * kmean[3t+a] = mean |k_a| over the bin's triangles (NaN when ntri == 0).
 * When no triangle of shell modes can wrap around the grid (grid side above
 * three times the largest |q_c| of a shell mode: every reduced plan) and the
 * plan has at most 64 shells, the sums are evaluated exactly by enumerating
 * the lattice triangles q1 + q2 + q3 = 0 (integer counts, fixed-point |q|
 * sums); otherwise from FP64 indicator / |k| fields and an FP64 contraction
 * (counts are the rounded FP64 sums).  The enumeration synchronises `stream`.
 * Replaces: FFTBispectrum.measure_gridinfo_faster, bskit/main.py:1941-2132,
 *           compute_Nbin / compute_k_means_on_grid, main.py:431-567.
 */
int bsk_gridinfo(bsk_plan* plan, const bsk_triset* set, double* ntri, double* kmean, void* stream);

/*
 * b_out[t] = b_unnorm[t] / ntri[t]   (FP64, device pointers).
 * Replaces: scripts/process/process_fast_bs_measurement.py:76.
 */
int bsk_normalize(int64_t n, const double* b_unnorm, const double* ntri, double* b_out, void* stream);

/*
 * Contract caller-provided real-space fields (device, float32 [n][K], each
 * 16-byte aligned) for a triangle set:
 *   out[t] = sum_k f1[i_t][k] f2[j_t][k] f3[l_t][k]  (no scale).
 * Used by the precision study and the kernel tests; bsk_measure_b calls the
 * same kernels on the plan's own fields.
 * Replaces: the per-triangle np.sum(I_a*I_b*I_c), bskit/main.py:1875.
 */
int bsk_contract(bsk_plan* plan, const bsk_triset* set, const float* f1, const float* f2,
                 const float* f3, int64_t k_points, int precision, double* out, void* stream);

/*
 * dst (device, K = Ng^3 floats) <- slot's FP32 field of one shell on the
 * contraction grid (built on demand).  Inspection aid for tests.
 * Replaces: reading delta_fields[i] after main.py:1861.
 */
int bsk_copy_field(bsk_plan* plan, int slot, int shell, float* dst, void* stream);

/*
 * Synchronise `stream` and report device-side failures that surface only
 * asynchronously: BSK_ERR_TIMEOUT when a bounded pipeline wait of the
 * tensor-core contraction expired (the kernel then stops early and its
 * results are invalid), BSK_ERR_CUDA for a CUDA error.
 * Replaces: (none -- bskit's MPI collectives block instead).
 */
int bsk_sync_check(void* stream);

/*
 * Allocation-free variant of bsk_contract for the tensor-core precisions
 * (BSK_PREC_BF16X3, BSK_PREC_BF16): out[t] = sum_k f1[i_t][k] f2[j_t][k] f3[l_t][k]
 * for n_tri host triangles (int32 [T][3] shell indices, no repeats) over
 * device fields [n_shells][k_points] (16-byte aligned).  No counterpart in the
 * reference: it serves callers that cannot call cudaMalloc -- a process whose
 * framework reserved the device memory up front, or a pipeline that forbids
 * cudaMalloc/cudaFree (which synchronise and can fail) on its hot path.
 * All scratch (the contraction schedule and the bf16 split of f3) lives in one
 * 64 MiB static device array of the library, held by every GPU that loads the
 * library until exit; a request needing more (about n_shells * k_points * 4
 * bytes plus the schedule) is rejected with BSK_ERR_ARG.  The array may only be
 * committed when the library's device code first loads on a device: make one
 * warm-up call per device before reserving the rest of its memory (no room for
 * the array is reported as BSK_ERR_OOM).  The first call on a device also looks
 * up the array's address.  Every call synchronises `stream` (it copies the
 * schedule from host memory and waits for the copies); a call on a stream that
 * is being captured is rejected with BSK_ERR_STATE.  A CUDA error pending on the
 * calling thread from earlier work is consumed once the arguments are checked.
 * Calls share the array: each rewrites what it reads, but calls whose work
 * overlaps on the GPU race.  No plan or triangle set is needed.
 */
int bsk_contract_noalloc(int n_shells, int64_t n_tri, const int32_t* tri, const float* f1,
                         const float* f2, const float* f3, int64_t k_points, int precision,
                         double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* BSKIT_GB300_H */
