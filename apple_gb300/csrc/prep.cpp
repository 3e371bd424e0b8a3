// Host-side mesh preparation: vertex and element orders, tiles and slots.
//
// The reference launches one thread per (tet, quadrature point) over the
// mesher's cell order and scatters with global atomics
// (warp/fem/_base.py:117-119, 288-289).  Here the mesh is cut, once, into
// tiles of up to kTileVerts distinct vertices so that a CTA can stage its
// vertices in shared memory and reduce the element-to-vertex scatter there;
// each (tile, vertex) pair then owns one slot in a vertex-major CSR that
// the vertex pass sums in a fixed order.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "agb_internal.h"

namespace agb {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

const char* last_error() { return g_last_error.c_str(); }

void clear_error() { g_last_error.clear(); }

// 21 bits per axis interleaved into a 63-bit key.
static inline uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

static std::vector<uint64_t> morton_keys(int n, const double* xyz) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], xyz[3 * i + c]);
      hi[c] = std::max(hi[c], xyz[3 * i + c]);
    }
  double ext = 0.0;
  for (int c = 0; c < 3; ++c) ext = std::max(ext, hi[c] - lo[c]);
  const double scale = ext > 0.0 ? (double)((1u << 21) - 1) / ext : 0.0;
  std::vector<uint64_t> key(n);
  for (int i = 0; i < n; ++i) {
    uint64_t q[3];
    for (int c = 0; c < 3; ++c) {
      double t = (xyz[3 * i + c] - lo[c]) * scale;
      t = std::min(std::max(t, 0.0), (double)((1u << 21) - 1));
      q[c] = (uint64_t)t;
    }
    key[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
  }
  return key;
}

std::vector<int32_t> morton_order(int n, const double* xyz) {
  std::vector<uint64_t> key = morton_keys(n, xyz);
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return key[a] != key[b] ? key[a] < key[b] : a < b;
  });
  return order;
}

int region_compute(int n_cells, const int32_t* cells, const double* points,
                   const double* fraction, double* D9, double* dV) {
  int n_bad = 0;
  for (int e = 0; e < n_cells; ++e) {
    const double* X0 = points + 3 * cells[4 * e + 0];
    double Dm[3][3];  // columns X_a - X_0, a = 1..3 (dXdr with dhdr of element/_tetra.py:37-45)
    for (int a = 1; a < 4; ++a) {
      const double* Xa = points + 3 * cells[4 * e + a];
      for (int i = 0; i < 3; ++i) Dm[i][a - 1] = Xa[i] - X0[i];
    }
    const double c00 = Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1];
    const double c01 = Dm[1][2] * Dm[2][0] - Dm[1][0] * Dm[2][2];
    const double c02 = Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0];
    const double det = Dm[0][0] * c00 + Dm[0][1] * c01 + Dm[0][2] * c02;
    const double inv = 1.0 / det;
    double Mi[3][3];
    Mi[0][0] = c00 * inv;
    Mi[1][0] = c01 * inv;
    Mi[2][0] = c02 * inv;
    Mi[0][1] = (Dm[0][2] * Dm[2][1] - Dm[0][1] * Dm[2][2]) * inv;
    Mi[1][1] = (Dm[0][0] * Dm[2][2] - Dm[0][2] * Dm[2][0]) * inv;
    Mi[2][1] = (Dm[0][1] * Dm[2][0] - Dm[0][0] * Dm[2][1]) * inv;
    Mi[0][2] = (Dm[0][1] * Dm[1][2] - Dm[0][2] * Dm[1][1]) * inv;
    Mi[1][2] = (Dm[0][2] * Dm[1][0] - Dm[0][0] * Dm[1][2]) * inv;
    Mi[2][2] = (Dm[0][0] * Dm[1][1] - Dm[0][1] * Dm[1][0]) * inv;
    // dhdX row a (a >= 1) = row a-1 of drdX = Dm^-1
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D9[9 * e + 3 * i + j] = Mi[i][j];
    double v = det / 6.0;  // quadrature weight 1/6 (quadrature/_tetra.py:14-15)
    if (fraction) v *= fraction[e];
    dV[e] = v;
    if (!(det > 0.0)) ++n_bad;  // region/_region.py:98-99 warns on dV <= 0
  }
  return n_bad;
}

int build_tiles(int n_cells, const int32_t* cells, const double* centroid, const double* D9,
                const double* mudv, const double* lamdv, int tile_elems, TilePlan* plan) {
  if (tile_elems <= 0) tile_elems = 1024;
  std::vector<int32_t> order = morton_order(n_cells, centroid);

  int n_points = 0;
  for (int e = 0; e < 4 * n_cells; ++e) n_points = std::max(n_points, cells[e] + 1);
  std::vector<int32_t> stamp(n_points, -1);

  plan->n_cells = n_cells;
  plan->tile_estart.assign(1, 0);
  plan->tile_vstart.assign(1, 0);
  plan->tile_gstart.assign(1, 0);
  plan->group_estart.clear();
  plan->tv_vid.clear();
  plan->elem_user.clear();
  plan->elem_user.reserve(n_cells);
  plan->ids.assign(n_cells, 0);
  plan->D.assign(9 * (size_t)n_cells, 0.0);
  plan->mudv.assign(n_cells, 0.0);
  plan->lamdv.assign(n_cells, 0.0);

  // greedy tiles along the Morton order
  std::vector<int32_t> tile_elems_list;
  std::vector<int32_t> tile_verts;
  int tile_id = 0;
  auto flush = [&]() {
    if (tile_elems_list.empty()) return;
    std::sort(tile_verts.begin(), tile_verts.end());
    const int nv = (int)tile_verts.size();
    // local ids by sorted vertex order
    auto local = [&](int32_t v) {
      return (int)(std::lower_bound(tile_verts.begin(), tile_verts.end(), v) - tile_verts.begin());
    };
    // element order inside the tile: warp groups of <= 32 elements in which
    // no vertex occurs more than 4 times (first fit along a strided walk of
    // the Morton order), then, per group, a corner order for every element
    // such that the elements' corners k = 0..3 are 32 distinct vertices for
    // each k (a proper 4-edge-colouring of the bipartite element-vertex
    // incidence graph, which exists since every degree is <= 4).  A warp then
    // adds the corner-k contributions of its 32 lanes into its own shared
    // memory copy with plain loads and stores: no atomics, no lost updates.
    const int ne = (int)tile_elems_list.size();
    const int stride = (ne + 31) / 32;
    std::vector<int32_t> walk;
    walk.reserve(ne);
    for (int c = 0; c < stride; ++c)
      for (int l = 0; l < 32; ++l)
        if (l * stride + c < ne) walk.push_back(tile_elems_list[l * stride + c]);
    std::vector<std::vector<int32_t>> groups;
    std::vector<std::array<uint8_t, kTileVerts>> mult;
    for (const int32_t eu : walk) {
      int lc[4];
      for (int a = 0; a < 4; ++a) lc[a] = local(cells[4 * eu + a]);
      size_t g = 0;
      for (; g < groups.size(); ++g) {
        if (groups[g].size() >= 32) continue;
        bool ok = true;
        for (int a = 0; a < 4 && ok; ++a) ok = mult[g][lc[a]] < 4;
        if (ok) break;
      }
      if (g == groups.size()) {
        groups.emplace_back();
        mult.emplace_back();
        mult.back().fill(0);
      }
      groups[g].push_back(eu);
      for (int a = 0; a < 4; ++a) ++mult[g][lc[a]];
    }
    for (const auto& grp : groups) {
      const int n = (int)grp.size();
      // colour[k][a] = position of element k's original corner a
      std::vector<std::array<int8_t, 4>> pos(n);
      std::vector<std::array<int, 4>> at_e(n);            // element k, colour c -> vertex or -1
      std::array<std::array<int, 4>, kTileVerts> at_v;     // vertex, colour -> element or -1
      for (auto& r : at_e) r.fill(-1);
      for (auto& r : at_v) r.fill(-1);
      std::vector<std::array<int, 4>> lc(n);
      for (int k = 0; k < n; ++k)
        for (int a = 0; a < 4; ++a) lc[k][a] = local(cells[4 * grp[k] + a]);
      for (int k = 0; k < n; ++k) {
        for (int a = 0; a < 4; ++a) {
          const int v = lc[k][a];
          int al = 0, be = 0;
          while (at_e[k][al] >= 0) ++al;  // free at the element
          while (at_v[v][be] >= 0) ++be;  // free at the vertex
          if (at_v[v][al] >= 0) {
            // flip the al/be alternating path that starts at v along colour al
            std::vector<std::pair<int, int>> path;  // (element, vertex) edges on the path
            int cv = v, c = al, other = be;
            while (true) {
              const int ek = at_v[cv][c];
              if (ek < 0) break;
              path.push_back({ek, cv});
              const int nv2 = at_e[ek][other];
              if (nv2 < 0) break;
              path.push_back({ek, nv2});
              cv = nv2;
            }
            // recolour: edges alternate al, be along the path
            for (size_t q = 0; q < path.size(); ++q) {
              const int ek = path[q].first, vv = path[q].second;
              const int cold = (q % 2 == 0) ? al : be;
              at_e[ek][cold] = -1;
              at_v[vv][cold] = -1;
            }
            for (size_t q = 0; q < path.size(); ++q) {
              const int ek = path[q].first, vv = path[q].second;
              const int cnew = (q % 2 == 0) ? be : al;
              at_e[ek][cnew] = vv;
              at_v[vv][cnew] = ek;
            }
          }
          at_e[k][al] = v;
          at_v[v][al] = k;
        }
      }
      plan->group_estart.push_back((int32_t)plan->elem_user.size());
      for (int k = 0; k < n; ++k) {
        const int32_t eu = grp[k];
        // original dhdX rows: row 0 = -(rows 1..3)
        double R[4][3];
        for (int j = 0; j < 3; ++j) {
          R[1][j] = D9[9 * (size_t)eu + j];
          R[2][j] = D9[9 * (size_t)eu + 3 + j];
          R[3][j] = D9[9 * (size_t)eu + 6 + j];
          R[0][j] = -(R[1][j] + R[2][j] + R[3][j]);
        }
        int orig_of_pos[4];
        for (int c = 0; c < 4; ++c) {
          const int v = at_e[k][c];
          int a = 0;
          while (lc[k][a] != v) ++a;
          orig_of_pos[c] = a;
        }
        const int ei = (int)plan->elem_user.size();
        plan->elem_user.push_back(eu);
        uint32_t packed = 0;
        for (int c = 0; c < 4; ++c) packed |= (uint32_t)lc[k][orig_of_pos[c]] << (8 * c);
        plan->ids[ei] = packed;
        for (int r = 0; r < 3; ++r)
          for (int j = 0; j < 3; ++j)
            plan->D[(size_t)(3 * r + j) * n_cells + ei] = R[orig_of_pos[r + 1]][j];
        plan->mudv[ei] = mudv[eu];
        plan->lamdv[ei] = lamdv ? lamdv[eu] : 0.0;
      }
    }
    plan->tile_gstart.push_back((int32_t)plan->group_estart.size());
    for (int i = 0; i < nv; ++i) plan->tv_vid.push_back(tile_verts[i]);
    plan->tile_estart.push_back((int32_t)plan->elem_user.size());
    plan->tile_vstart.push_back((int32_t)plan->tv_vid.size());
    tile_elems_list.clear();
    tile_verts.clear();
    ++tile_id;
  };
  for (int k = 0; k < n_cells; ++k) {
    const int32_t e = order[k];
    int fresh = 0;
    for (int a = 0; a < 4; ++a) {
      const int32_t v = cells[4 * e + a];
      bool dup = stamp[v] == tile_id;
      for (int b = 0; b < a; ++b) dup = dup || cells[4 * e + b] == v;
      fresh += dup ? 0 : 1;
    }
    if ((int)tile_elems_list.size() + 1 > tile_elems ||
        (int)tile_verts.size() + fresh > kTileVerts)
      flush();
    for (int a = 0; a < 4; ++a) {
      const int32_t v = cells[4 * e + a];
      if (stamp[v] != tile_id) {
        stamp[v] = tile_id;
        tile_verts.push_back(v);
      }
    }
    tile_elems_list.push_back(e);
  }
  flush();
  plan->group_estart.push_back((int32_t)plan->elem_user.size());
  plan->n_tiles = (int)plan->tile_estart.size() - 1;
  plan->n_tv = (int)plan->tv_vid.size();
  return AGB_OK;
}

void build_slots(int n_points, const std::vector<const TilePlan*>& plans,
                 std::vector<SlotMap>* per_plan, std::vector<int32_t>* off) {
  std::vector<int32_t> count(n_points + 1, 0);
  for (const TilePlan* p : plans)
    for (int32_t v : p->tv_vid) ++count[v + 1];
  off->assign(n_points + 1, 0);
  for (int v = 0; v < n_points; ++v) (*off)[v + 1] = (*off)[v] + count[v + 1];
  std::vector<int32_t> cursor(off->begin(), off->end() - 1);
  per_plan->assign(plans.size(), SlotMap{});
  for (size_t k = 0; k < plans.size(); ++k) {
    const TilePlan* p = plans[k];
    SlotMap& sm = (*per_plan)[k];
    sm.slot_of_tv.resize(p->n_tv);
    for (int i = 0; i < p->n_tv; ++i) sm.slot_of_tv[i] = cursor[p->tv_vid[i]]++;
    sm.off = *off;
  }
}

}  // namespace agb
