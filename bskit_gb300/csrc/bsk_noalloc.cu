// Allocation-free tensor-core contraction: bsk_contract_noalloc.
//
// Some callers cannot call cudaMalloc at the moment they need a bispectrum:
// applications whose framework reserved (nearly) all device memory in its own
// pool at start-up, and real-time or embedded pipelines that forbid
// cudaMalloc/cudaFree on the hot path because they synchronise the device and
// can fail under fragmentation.  For them this file offers one entry point
// that computes the same bf16x3 / bf16 contraction as bsk_contract but takes
// all of its scratch -- the contraction schedule and the bf16 hi/lo split of
// the column fields -- from one file-scope device array of fixed size
// (kStaticScratchBytes, 64 MiB).  The caller passes the fields, the triangle
// list and the output buffer; nothing is allocated.
//
// Properties callers rely on:
//  * the array is part of this library's device image: every GPU that loads
//    the library holds it until the process exits.  With CUDA's lazy module
//    loading the array is committed when the library's device code is first
//    loaded on a device, which may be this entry point's first call: make one
//    warm-up call on each device before reserving the rest of its memory;
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current);
//  * every call synchronises `stream`: the schedule is copied from pageable
//    host memory, and the call waits for those copies before it returns.  A
//    call made while `stream` is being captured into a CUDA graph is rejected
//    with BSK_ERR_STATE before it enqueues anything;
//  * any CUDA error still pending on the calling thread from earlier work is
//    consumed (cleared) once the arguments have passed their checks;
//  * every call shares the array and it keeps the last call's contents; each
//    call rewrites everything it later reads (and zeroes the output), so no
//    result depends on an earlier call -- but two calls whose work overlaps on
//    the GPU (different streams, no ordering) race on the array;
//  * requests that do not fit in the array are rejected with BSK_ERR_ARG, and
//    so are field pointers that are not 16-byte aligned (the kernels read
//    them with 16-byte vector loads and TMA).
#include <algorithm>
#include <mutex>
#include <set>
#include <tuple>

#include "bsk_internal.cuh"

namespace bsk {
namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;  // first calls from several host threads resolve the address once

void* scratch_address(int dev) {
  BSK_REQUIRE(dev >= 0 && dev < kMaxDevices, BSK_ERR_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      // the array is committed when the module loads: no room for it is an out-of-memory
      throw Error{e == cudaErrorMemoryAllocation ? BSK_ERR_OOM : BSK_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(static scratch): ") +
                      cudaGetErrorString(e)};
    }
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// The triangle list as the shared tiler takes it.  A repeated (i, j, l) would put two
// triangles in one schedule entry, so it is rejected (the plan path maps repeats onto
// their first occurrence instead).
std::vector<HostTriangle> checked_triangles(int64_t T, const int32_t* tri, int n) {
  std::vector<HostTriangle> out;
  out.reserve((size_t)T);
  std::set<std::tuple<int, int, int>> seen;
  for (int64_t t = 0; t < T; ++t) {
    const int i = tri[3 * t], j = tri[3 * t + 1], l = tri[3 * t + 2];
    BSK_REQUIRE(i >= 0 && j >= 0 && l >= 0 && i < n && j < n && l < n, BSK_ERR_ARG,
                "triangle " + std::to_string(t) + " has a shell index outside [0, n_shells)");
    BSK_REQUIRE(seen.emplace(i, j, l).second, BSK_ERR_ARG, "repeated triangle in the list");
    out.push_back(HostTriangle{i, j, l});
  }
  return out;
}

}  // namespace
}  // namespace bsk

using namespace bsk;

extern "C" int bsk_contract_noalloc(int n_shells, int64_t n_tri, const int32_t* tri,
                                    const float* f1, const float* f2, const float* f3,
                                    int64_t k_points, int precision, double* out, void* stream) {
  try {
    BSK_REQUIRE(n_shells >= 1 && n_shells <= 255, BSK_ERR_ARG, "need 1..255 shells");
    BSK_REQUIRE(n_tri >= 0 && (n_tri == 0 || (tri && out)), BSK_ERR_ARG, "bad triangle list");
    BSK_REQUIRE(f1 && f2 && f3, BSK_ERR_ARG, "NULL field pointer");
    BSK_REQUIRE(((uintptr_t)f1 | (uintptr_t)f2 | (uintptr_t)f3) % 16 == 0, BSK_ERR_ARG,
                "field pointers must be 16-byte aligned");
    BSK_REQUIRE(k_points > 0 && k_points % 8 == 0, BSK_ERR_ARG,
                "k_points must be a positive multiple of 8");
    BSK_REQUIRE(precision == BSK_PREC_BF16X3 || precision == BSK_PREC_BF16, BSK_ERR_ARG,
                "the allocation-free contraction runs the tensor-core precisions (bf16x3, bf16)");
    BSK_REQUIRE(((uintptr_t)out) % 8 == 0, BSK_ERR_ARG, "output pointer must be 8-byte aligned");
    if (n_tri == 0) return BSK_OK;
    cudaStream_t st = (cudaStream_t)stream;
    // the call synchronises its stream (pageable copies + wait below), which a capture forbids
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    BSK_CHECK_CUDA(cudaStreamIsCapturing(st, &cap));
    BSK_REQUIRE(cap == cudaStreamCaptureStatusNone, BSK_ERR_STATE,
                "bsk_contract_noalloc synchronises its stream and cannot be captured into a "
                "CUDA graph; call it outside stream capture");
    cudaGetLastError();  // a stale error of earlier work must not be reported as this call's
    int dev = 0;
    BSK_CHECK_CUDA(cudaGetDevice(&dev));
    int num_sms = 0;
    BSK_CHECK_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));

    HostSchedule tb;
    tile_schedule(checked_triangles(n_tri, tri, n_shells), n_shells, nullptr, tb);
    const size_t b_tiles = align256(tb.tiles.size() * sizeof(TileDesc));
    const size_t b_rows = align256(tb.ri.size() * sizeof(int16_t));
    const size_t b_map = align256(tb.map.size() * sizeof(int32_t));
    const size_t b_split = align256(split_elems(n_shells, k_points) * sizeof(__nv_bfloat16));
    const size_t need = b_tiles + 2 * b_rows + b_map + b_split;
    BSK_REQUIRE(need <= kStaticScratchBytes, BSK_ERR_ARG,
                "request needs " + std::to_string(need) + " bytes of scratch; the static area "
                "holds " + std::to_string(kStaticScratchBytes) + " (n_shells * k_points * 4 "
                "bytes, k_points rounded up to a multiple of 128, plus the schedule)");

    unsigned char* base = (unsigned char*)scratch_address(dev);
    DeviceSchedule s;
    s.n_tiles = (int)tb.tiles.size();
    s.tiles = reinterpret_cast<TileDesc*>(base);
    s.row_i = reinterpret_cast<int16_t*>(base + b_tiles);
    s.row_j = reinterpret_cast<int16_t*>(base + b_tiles + b_rows);
    s.map = reinterpret_cast<int32_t*>(base + b_tiles + 2 * b_rows);
    s.h_tiles = tb.tiles;
    __nv_bfloat16* split =
        reinterpret_cast<__nv_bfloat16*>(base + b_tiles + 2 * b_rows + b_map);
    BSK_CHECK_CUDA(cudaMemcpyAsync(s.tiles, tb.tiles.data(), tb.tiles.size() * sizeof(TileDesc),
                                   cudaMemcpyHostToDevice, st));
    BSK_CHECK_CUDA(cudaMemcpyAsync(s.row_i, tb.ri.data(), tb.ri.size() * sizeof(int16_t),
                                   cudaMemcpyHostToDevice, st));
    BSK_CHECK_CUDA(cudaMemcpyAsync(s.row_j, tb.rj.data(), tb.rj.size() * sizeof(int16_t),
                                   cudaMemcpyHostToDevice, st));
    BSK_CHECK_CUDA(cudaMemcpyAsync(s.map, tb.map.data(), tb.map.size() * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, st));
    // host vectors are released at return: the copies above must have read them
    BSK_CHECK_CUDA(cudaStreamSynchronize(st));
    launch_split(f3, n_shells, k_points, split, st);  // also zeroes the last chunk's tail
    BSK_CHECK_CUDA(cudaMemsetAsync(out, 0, (size_t)n_tri * sizeof(double), st));
    launch_contract_tc(s, f1, f2, split, n_shells, n_shells, k_points, 0, k_points,
                       precision == BSK_PREC_BF16X3 ? 3 : 1, out, num_sms, st);
    s.tiles = nullptr;  // the schedule lives in the static area: nothing to release
    s.row_i = s.row_j = nullptr;
    s.map = nullptr;
    return BSK_OK;
  } catch (const Error& e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {  // the host-side tiling tables
    set_error("host allocation failed");
    return BSK_ERR_OOM;
  } catch (const std::exception& e) {
    set_error(e.what());
    return BSK_ERR_ARG;
  } catch (...) {  // nothing may unwind through the C ABI
    set_error("unexpected exception");
    return BSK_ERR_STATE;
  }
}
