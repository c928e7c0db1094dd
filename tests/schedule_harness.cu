// Host-only driver of the contraction schedule (bskit_gb300/csrc/bsk_schedule.cu) for the
// CPU tests: linked with --wrap for cudaMalloc / cudaMemcpy / cudaFree, so that the
// schedule's device arrays are host memory and no GPU is needed.  Reads "n T" and T
// triangles "i j l" from the file argv[1]; prints the tiles, the pair rows and the map.
#include <algorithm>
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

// "levels" mode: reads "n T M", the n shell radii, the M candidate sides and T triangles;
// prints the side chosen for each triangle ("lev t k") and, for every pair of candidate
// sides (previous chosen side i, or -1 for none; side j), the modelled cost of the level of
// side j holding the bins with side_i <= v < side_j ("cost i j value"), computed here from
// the tiler on its own, so that the test can check the choice against every subset.
static int levels_mode(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return 2;
  int n = 0, T = 0, M = 0;
  if (fscanf(f, "%d %d %d", &n, &T, &M) != 3) return 3;
  std::vector<int> r(n), sides(M);
  for (int& x : r)
    if (fscanf(f, "%d", &x) != 1) return 3;
  for (int& x : sides)
    if (fscanf(f, "%d", &x) != 1) return 3;
  std::vector<bsk::HostTriangle> tri(T);
  for (int t = 0; t < T; ++t)
    if (fscanf(f, "%d %d %d", &tri[t].i, &tri[t].j, &tri[t].l) != 3) return 3;
  fclose(f);
  const double tile_cost = 13.0, shell_cost = 1.0;
  std::vector<int> lev;
  try {
    lev = bsk::choose_level_sides(tri, r, sides, n, tile_cost, shell_cost);
  } catch (const bsk::Error& e) {
    printf("error %d %s\n", e.code, e.msg.c_str());
    return 0;
  }
  for (int t = 0; t < T; ++t) printf("lev %d %d\n", t, lev[t]);
  for (int j = 0; j < M; ++j)
    for (int i = -1; i < j; ++i) {
      const int lo = i < 0 ? 0 : sides[i];
      std::vector<bsk::HostTriangle> tk;
      int top = -1;
      for (const bsk::HostTriangle& h : tri) {
        const int v = std::max(r[h.i] + r[h.j] + r[h.l], 2 * std::max(r[h.i], std::max(r[h.j], r[h.l])));
        if (v >= lo && v < sides[j]) {
          tk.push_back(h);
          top = std::max(top, std::max(h.i, std::max(h.j, h.l)));
        }
      }
      double c = 0.0;
      if (!tk.empty()) {
        bsk::HostSchedule hs;
        bsk::tile_schedule(tk, n, nullptr, hs);
        c = (double)sides[j] * sides[j] * sides[j] * (tile_cost * hs.tiles.size() + shell_cost * (top + 1));
      }
      printf("cost %d %d %.17g\n", i, j, c);
    }
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 3 && strcmp(argv[1], "levels") == 0) return levels_mode(argv[2]);
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
