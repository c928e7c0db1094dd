// Host-side tile schedule for the triple-product contraction.
//
// B[t] = sum_x F1[i_t](x) F2[j_t](x) F3[l_t](x) is evaluated as a GEMM
//   C[(i,j), l] = sum_x (F1[i] * F2[j])(x) * F3[l](x)
// restricted to the (pair, l) entries that are triangle bins.  Every distinct
// (i, j) pair is one GEMM row; rows are sorted by the range of third shells
// they need and packed 128 to a tile, each tile covering a contiguous column
// range [l0, l0 + nc), nc a multiple of 8.  Inside a tile the rows are ordered
// by (i, j): the tensor-core kernel's A-operand warps each handle 32 consecutive
// rows, and rows that share a shell read the same shared-memory words, which a
// warp's load serves once (a broadcast).  Ordered by (i, j), a warp's 32 rows
// span few distinct i and j, so its loads of the two pair factors take about
// 40% fewer shared-memory wavefronts than with the packing order.  The map
// [c][r] -> t scatters tile entries back to triangle bins (-1 for entries that
// are not bins).
#include <algorithm>
#include <cmath>
#include <map>

#include "bsk_internal.cuh"

namespace bsk {

void DeviceSchedule::release() {
  if (tiles) cudaFree(tiles);
  if (row_i) cudaFree(row_i);
  if (row_j) cudaFree(row_j);
  if (map) cudaFree(map);
  if (subs) cudaFree(subs);
  subs = nullptr;
  n_sub = 0;
  tiles = nullptr;
  row_i = row_j = nullptr;
  map = nullptr;
  n_tiles = 0;
  sum_nc = 0;
  h_tiles.clear();
}

namespace {
struct Row {
  int i, j;
  int lmin, lmax;
  std::vector<std::pair<int, int>> cols;  // (l, t)
};

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }
}  // namespace

void tile_schedule(const std::vector<HostTriangle>& tri, int n_shells,
                   const std::vector<int>* map_index, HostSchedule& out) {
  std::map<std::pair<int, int>, int> index;
  std::vector<Row> rows;
  for (size_t t = 0; t < tri.size(); ++t) {
    const HostTriangle& h = tri[t];
    BSK_REQUIRE(h.i >= 0 && h.j >= 0 && h.l >= 0 && h.i < n_shells && h.j < n_shells &&
                    h.l < n_shells,
                BSK_ERR_ARG, "triangle shell index out of range");
    auto key = std::make_pair(h.i, h.j);
    auto it = index.find(key);
    int r;
    if (it == index.end()) {
      r = (int)rows.size();
      index.emplace(key, r);
      rows.push_back(Row{h.i, h.j, h.l, h.l, {}});
    } else {
      r = it->second;
    }
    Row& R = rows[r];
    R.lmin = std::min(R.lmin, h.l);
    R.lmax = std::max(R.lmax, h.l);
    R.cols.emplace_back(h.l, map_index ? (*map_index)[t] : (int)t);
  }
  // A tile holds at most kMaxCols column shells, so a pair whose third shells span more
  // (possible with more than kMaxCols shells) becomes several rows, each over a run of at
  // most kMaxCols consecutive shells.  With kMaxCols shells or fewer nothing is cut.
  {
    std::vector<Row> cut;
    cut.reserve(rows.size());
    for (Row& R : rows) {
      if (R.lmax - R.lmin + 1 <= kMaxCols) {
        cut.push_back(std::move(R));
        continue;
      }
      std::sort(R.cols.begin(), R.cols.end());
      Row seg{R.i, R.j, R.cols[0].first, R.cols[0].first, {}};
      for (const auto& c : R.cols) {
        if (c.first - seg.lmin + 1 > kMaxCols) {
          cut.push_back(std::move(seg));
          seg = Row{R.i, R.j, c.first, c.first, {}};
        }
        seg.lmax = c.first;
        seg.cols.push_back(c);
      }
      cut.push_back(std::move(seg));
    }
    rows.swap(cut);
  }
  std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) {
    if (a.lmax != b.lmax) return a.lmax < b.lmax;
    if (a.lmin != b.lmin) return a.lmin < b.lmin;
    if (a.j != b.j) return a.j < b.j;
    return a.i < b.i;
  });

  // Greedy packing under the tile constraints.
  std::vector<std::vector<int>> groups;
  {
    std::vector<int> cur;
    int lmin = 0, lmax = 0, imin = 0, imax = 0, jmin = 0, jmax = 0;
    for (int r = 0; r < (int)rows.size(); ++r) {
      const Row& R = rows[r];
      if (!cur.empty()) {
        int nl = std::min(lmin, R.lmin), xl = std::max(lmax, R.lmax);
        int ni = std::min(imin, R.i), xi = std::max(imax, R.i);
        int nj = std::min(jmin, R.j), xj = std::max(jmax, R.j);
        bool fits = (int)cur.size() < kTileRows && round_up(xl - nl + 1, 8) <= kMaxCols &&
                    round_up(xi - ni + 1, 8) <= kMaxSrcRows &&
                    round_up(xj - nj + 1, 8) <= kMaxSrcRows;
        if (fits) {
          cur.push_back(r);
          lmin = nl; lmax = xl; imin = ni; imax = xi; jmin = nj; jmax = xj;
          continue;
        }
        groups.push_back(cur);
        cur.clear();
      }
      cur.push_back(r);
      lmin = R.lmin; lmax = R.lmax; imin = imax = R.i; jmin = jmax = R.j;
    }
    if (!cur.empty()) groups.push_back(cur);
  }

  std::vector<TileDesc>& tiles = out.tiles;
  std::vector<int16_t>& ri = out.ri;
  std::vector<int16_t>& rj = out.rj;
  std::vector<int32_t>& map = out.map;
  tiles.clear();
  ri.clear();
  rj.clear();
  map.clear();
  int sum_nc = 0;
  for (auto& g : groups) {
    std::sort(g.begin(), g.end(), [&rows](int a, int b) {
      if (rows[a].i != rows[b].i) return rows[a].i < rows[b].i;
      if (rows[a].j != rows[b].j) return rows[a].j < rows[b].j;
      return rows[a].lmin < rows[b].lmin;  // the two runs of a pair cut at 64 columns
    });
    TileDesc d{};
    int lmin = 1 << 30, lmax = -1, imin = 1 << 30, imax = -1, jmin = 1 << 30, jmax = -1;
    for (int r : g) {
      lmin = std::min(lmin, rows[r].lmin); lmax = std::max(lmax, rows[r].lmax);
      imin = std::min(imin, rows[r].i); imax = std::max(imax, rows[r].i);
      jmin = std::min(jmin, rows[r].j); jmax = std::max(jmax, rows[r].j);
    }
    d.l0 = lmin;
    const int lo_ij = std::min(imin, jmin), hi_ij = std::max(imax, jmax);
    if (hi_ij - lo_ij < kMaxSrcRows) {  // one source range serves both pair factors
      d.i0 = d.j0 = lo_ij;
      d.ni = d.nj = round_up(hi_ij - lo_ij + 1, 8);
    } else {
      d.i0 = imin; d.j0 = jmin;
      d.ni = round_up(imax - imin + 1, 8);
      d.nj = round_up(jmax - jmin + 1, 8);
    }
    d.nc = std::max(8, round_up(lmax - lmin + 1, 8));
    BSK_REQUIRE(d.nc <= kMaxCols && d.ni <= kMaxSrcRows && d.nj <= kMaxSrcRows, BSK_ERR_STATE,
                "internal: a tile exceeds its column or source span");
    d.nrows = (int)g.size();
    d.row_off = (int)ri.size();
    d.map_off = (int)map.size();
    sum_nc += d.nc;
    ri.resize(ri.size() + kTileRows, (int16_t)-1);
    rj.resize(rj.size() + kTileRows, (int16_t)-1);
    map.resize(map.size() + (size_t)d.nc * kTileRows, -1);
    for (int k = 0; k < (int)g.size(); ++k) {
      const Row& R = rows[g[k]];
      ri[d.row_off + k] = (int16_t)R.i;
      rj[d.row_off + k] = (int16_t)R.j;
      for (auto& c : R.cols) map[d.map_off + (size_t)(c.first - lmin) * kTileRows + k] = c.second;
    }
    tiles.push_back(d);
  }
  out.sum_nc = sum_nc;
}

// Grid levels of a triangle set (host only).  Bin t can use any side S > v_t =
// max(r_i + r_j + r_l, 2 max(r_i, r_j, r_l)) (no closed triangle of its modes wraps around,
// its shells fit the Nyquist range) and goes to the smallest chosen side, so a level's bins
// are those with v_t in [previous chosen side, its side): its modelled cost -- side^3 x
// (tile_cost x tiles of its schedule + shell_cost x the shell prefix it synthesises) --
// depends on those two sides only, and the cheapest chain of sides ending at the last one
// (the plan's own grid, which holds every bin) is a shortest path over the candidates.
// Returns, per triangle, the index in `sides` of its side.
std::vector<int> choose_level_sides(const std::vector<HostTriangle>& tri,
                                    const std::vector<int>& shell_r,
                                    const std::vector<int>& sides, int n_shells,
                                    double tile_cost, double shell_cost) {
  const int m = (int)sides.size();
  const int nt = (int)tri.size();
  BSK_REQUIRE(m >= 1, BSK_ERR_STATE, "internal: no grid side");
  std::vector<int> v(nt);
  for (int t = 0; t < nt; ++t) {
    const HostTriangle& h = tri[t];
    const int ri = shell_r[h.i], rj = shell_r[h.j], rl = shell_r[h.l];
    v[t] = std::max(ri + rj + rl, 2 * std::max(ri, std::max(rj, rl)));
    BSK_REQUIRE(v[t] < sides[m - 1], BSK_ERR_STATE, "internal: a bin exceeds the plan's grid");
  }
  // modelled cost of the level of side `side` holding the bins with lo <= v < side
  auto cost = [&](int lo, int side) {
    std::vector<HostTriangle> tk;
    int top = -1;
    for (int t = 0; t < nt; ++t)
      if (v[t] >= lo && v[t] < side) {
        tk.push_back(tri[t]);
        top = std::max(top, std::max(tri[t].i, std::max(tri[t].j, tri[t].l)));
      }
    if (tk.empty()) return 0.0;
    HostSchedule hs;
    tile_schedule(tk, n_shells, nullptr, hs);
    return std::pow((double)side, 3) * (tile_cost * hs.tiles.size() + shell_cost * (top + 1));
  };
  // best[j]: cheapest chain covering the bins with v < sides[j], ending at sides[j]
  std::vector<double> best(m, 0.0);
  std::vector<int> prev(m, -1);
  for (int j = 0; j < m; ++j) {
    best[j] = cost(0, sides[j]);
    for (int i = 0; i < j; ++i) {
      const double c = best[i] + cost(sides[i], sides[j]);
      if (c < best[j]) {
        best[j] = c;
        prev[j] = i;
      }
    }
  }
  std::vector<int> chain;
  for (int j = m - 1; j >= 0; j = prev[j]) chain.push_back(j);
  std::vector<int> lev(nt, m - 1);
  for (int t = 0; t < nt; ++t)
    for (int k = (int)chain.size() - 1; k >= 0; --k)  // chain is largest side first
      if (v[t] < sides[chain[k]]) {
        lev[t] = chain[k];
        break;
      }
  return lev;
}

void build_schedule(const std::vector<HostTriangle>& tri, int n_shells, DeviceSchedule& out,
                    const std::vector<int>* map_index) {
  out.release();
  HostSchedule hs;
  tile_schedule(tri, n_shells, map_index, hs);
  const std::vector<TileDesc>& tiles = hs.tiles;
  const std::vector<int16_t>& ri = hs.ri;
  const std::vector<int16_t>& rj = hs.rj;
  const std::vector<int32_t>& map = hs.map;
  out.n_tiles = (int)tiles.size();
  out.sum_nc = hs.sum_nc;
  out.h_tiles = tiles;
  if (tiles.empty()) return;
  BSK_CHECK_CUDA(cudaMalloc(&out.tiles, tiles.size() * sizeof(TileDesc)));
  BSK_CHECK_CUDA(cudaMalloc(&out.row_i, ri.size() * sizeof(int16_t)));
  BSK_CHECK_CUDA(cudaMalloc(&out.row_j, rj.size() * sizeof(int16_t)));
  BSK_CHECK_CUDA(cudaMalloc(&out.map, map.size() * sizeof(int32_t)));
  BSK_CHECK_CUDA(cudaMemcpy(out.tiles, tiles.data(), tiles.size() * sizeof(TileDesc),
                            cudaMemcpyHostToDevice));
  BSK_CHECK_CUDA(cudaMemcpy(out.row_i, ri.data(), ri.size() * sizeof(int16_t),
                            cudaMemcpyHostToDevice));
  BSK_CHECK_CUDA(cudaMemcpy(out.row_j, rj.data(), rj.size() * sizeof(int16_t),
                            cudaMemcpyHostToDevice));
  BSK_CHECK_CUDA(cudaMemcpy(out.map, map.data(), map.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
  std::vector<int2> subs;
  for (int u = 0; u < (int)tiles.size(); ++u)
    for (int c = 0; c < tiles[u].nc; c += 32) subs.push_back(make_int2(u, c));
  out.n_sub = (int)subs.size();
  BSK_CHECK_CUDA(cudaMalloc(&out.subs, subs.size() * sizeof(int2)));
  BSK_CHECK_CUDA(cudaMemcpy(out.subs, subs.data(), subs.size() * sizeof(int2),
                            cudaMemcpyHostToDevice));
}

}  // namespace bsk
