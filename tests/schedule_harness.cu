// Host-only driver of the contraction schedule (bskit_gb300/csrc/bsk_schedule.cu) for the
// CPU tests: linked with --wrap for cudaMalloc / cudaMemcpy / cudaFree, so that the
// schedule's device arrays are host memory and no GPU is needed.  Reads "n T" and T
// triangles "i j l" from the file argv[1]; prints the tiles, the pair rows and the map.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bsk_internal.cuh"

extern "C" cudaError_t __wrap_cudaMalloc(void** p, size_t n) {
  *p = malloc(n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t __wrap_cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  memcpy(d, s, n);
  return cudaSuccess;
}
extern "C" cudaError_t __wrap_cudaFree(void* p) {
  free(p);
  return cudaSuccess;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* f = fopen(argv[1], "r");
  if (!f) return 2;
  int n = 0, T = 0;
  if (fscanf(f, "%d %d", &n, &T) != 2) return 3;
  std::vector<bsk::HostTriangle> tri(T);
  for (int t = 0; t < T; ++t)
    if (fscanf(f, "%d %d %d", &tri[t].i, &tri[t].j, &tri[t].l) != 3) return 3;
  fclose(f);
  bsk::DeviceSchedule s;
  try {
    bsk::build_schedule(tri, n, s);
  } catch (const bsk::Error& e) {
    printf("error %d %s\n", e.code, e.msg.c_str());
    return 0;
  }
  printf("tiles %d sum_nc %d\n", s.n_tiles, s.sum_nc);
  size_t rows = 0, maps = 0;
  for (int u = 0; u < s.n_tiles; ++u) {
    const bsk::TileDesc& d = s.h_tiles[u];
    printf("tile %d %d %d %d %d %d %d %d %d\n", d.i0, d.j0, d.l0, d.ni, d.nj, d.nc, d.nrows,
           d.row_off, d.map_off);
    rows = d.row_off + bsk::kTileRows;
    maps = d.map_off + (size_t)d.nc * bsk::kTileRows;
  }
  for (size_t r = 0; r < rows; ++r) printf("r %d %d\n", s.row_i[r], s.row_j[r]);
  for (size_t m = 0; m < maps; ++m) printf("m %d\n", s.map[m]);
  return 0;
}
