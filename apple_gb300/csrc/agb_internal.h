// Internal declarations shared by the host runtime (prep.cpp, capi.cu) and
// the kernels (fem_kernels.cu, solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/apple_gb300.h"

namespace agb {

void set_error(const char* fmt, ...);
// forget the last message (calls that add a message only when none was set)
void clear_error();

#define AGB_CHECK_CUDA(call)                                                                  \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      ::agb::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__,    \
                       __LINE__);                                                             \
      return AGB_E_CUDA;                                                                      \
    }                                                                                         \
  } while (0)

#define AGB_REQUIRE(cond, code, ...) \
  do {                               \
    if (!(cond)) {                   \
      ::agb::set_error(__VA_ARGS__); \
      return (code);                 \
    }                                \
  } while (0)

// Maximum distinct vertices of one tile: local corner ids are 8-bit.
constexpr int kTileVerts = 256;
// Threads of one element-pass CTA.
constexpr int kElemThreads = 256;
// Threads of one vertex-pass CTA.
constexpr int kVertThreads = 256;

// Host-side result of tiling one potential's mesh (prep.cpp).
struct TilePlan {
  int n_cells = 0;
  int n_tiles = 0;
  int n_tv = 0;                      // tile-vertex entries (sum over tiles)
  std::vector<int32_t> tile_estart;  // n_tiles + 1, element ranges
  std::vector<int32_t> tile_vstart;  // n_tiles + 1, tile-vertex ranges
  std::vector<int32_t> tile_gstart;  // n_tiles + 1, warp-group ranges
  std::vector<int32_t> group_estart; // n_groups + 1, element ranges of conflict-free warp groups
  std::vector<int32_t> tv_vid;       // n_tv, internal vertex id
  std::vector<int32_t> elem_user;    // internal element -> caller's cell index
  std::vector<uint32_t> ids;         // packed 4 x 8-bit local corner ids
  std::vector<double> D;             // 9 x n_cells, rows 1..3 of dhdX (component-major)
  std::vector<double> mudv;          // mu * dV
  std::vector<double> lamdv;         // lambda * dV
};

// Vertex-major CSR over slots: slots of internal vertex v are
// [off[v], off[v+1]); slot_of_tv maps a tile-vertex entry to its slot.
struct SlotMap {
  std::vector<int32_t> off;
  std::vector<int32_t> slot_of_tv;
};

// Morton order of points (host); returns user_of_internal.
std::vector<int32_t> morton_order(int n, const double* xyz);

// Region precompute in FP64 (jax/fem/region/_region.py:84-108).  Writes
// rows 1..3 of dhdX (Dm^-1) and dV = det(Dm)/6 * fraction.  Returns the
// number of cells with dV <= 0.
int region_compute(int n_cells, const int32_t* cells, const double* points,
                   const double* fraction, double* D9 /*n x 9*/, double* dV);

// Build the tile plan.  cells_int are internal vertex ids.
int build_tiles(int n_cells, const int32_t* cells_int, const double* centroid_xyz,
                const double* D9, const double* mudv, const double* lamdv, int tile_elems,
                TilePlan* plan);

// One slot map over several plans (a model); plans[k]->n_tv entries each.
void build_slots(int n_points, const std::vector<const TilePlan*>& plans,
                 std::vector<SlotMap>* per_plan, std::vector<int32_t>* off);

}  // namespace agb

// ---------------------------------------------------------------------------
// opaque handle types of the C ABI
// ---------------------------------------------------------------------------

struct agb_space {
  int32_t n_points = 0;
  std::vector<int32_t> user_of_internal;
  std::vector<int32_t> internal_of_user;
  std::vector<double> points_internal;  // rest positions in internal order (may be empty)
  int32_t* d_user_of_internal = nullptr;
};

namespace agb {
// Device view of one potential's element data, passed to kernels by value.
struct FemView {
  int material;
  int n_tiles;
  int n_cells;
  const int32_t* tile_estart;
  const int32_t* tile_vstart;
  const int32_t* tile_gstart;
  const int32_t* group_estart;
  const int32_t* tv_vid;
  // FP32: rec = float4[3][n_cells]; FP64: rec = double[11][n_cells] + ids
  const void* rec;
  const uint32_t* ids;
  // stable Neo-Hookean muscle: the activation offset S = A - I per element
  // (A = I + sym(a), a the cell's 6-vector); FP32: float4[2][n_cells] =
  // (S00 S11 S22 S01), (S02 S12 0 0); FP64: double[6][n_cells].  The records
  // of a muscle potential hold D A instead of D.
  const void* act;
};
}  // namespace agb

struct agb_fem {
  agb_space* space = nullptr;
  int material = 0;
  int precision = 0;
  agb::TilePlan plan;
  agb::SlotMap own_slots;         // slots when used on its own
  std::vector<int32_t> own_off;
  // device
  int32_t* d_tile_estart = nullptr;
  int32_t* d_tile_vstart = nullptr;
  int32_t* d_tile_gstart = nullptr;
  int32_t* d_group_estart = nullptr;
  int32_t* d_tv_vid = nullptr;
  int32_t* d_own_slot = nullptr;  // tile-vertex -> slot (standalone)
  int32_t* d_own_off = nullptr;   // n_points + 1
  void* d_rec = nullptr;
  uint32_t* d_ids = nullptr;
  std::vector<double> vol_internal;  // dV * fraction per internal element
  std::vector<double> act_internal;  // muscle: activation (6 per internal element)
  void* d_act = nullptr;             // muscle: S stream (FemView::act)
  int32_t* d_elem_user = nullptr;    // internal -> caller's cell index (on first use)
  void* d_vol = nullptr;             // R per internal element (on first use)
  // scratch for the standalone evaluation API
  void* d_u = nullptr;      // V4<R> n_points
  void* d_p = nullptr;      // V4<R> n_points
  void* d_slots = nullptr;  // V4<R> [3][n_tv]
  double* d_partials = nullptr;
  unsigned* d_counter = nullptr;
  agb::FemView view() const;
};

struct agb_model {
  agb_space* space = nullptr;
  int precision = 0;
  std::vector<agb_fem*> fems;
  std::vector<agb::SlotMap> slots;  // per potential
  std::vector<int32_t> off;         // model CSR
  int32_t n_slots = 0;
  int32_t n_force = 0;
  std::vector<uint8_t> mask_internal;  // n_points, 3 bits
  std::vector<double> fixed_internal;  // n_points x 3
  std::vector<double> force_internal;  // n_points x 3 (summed per vertex)
  // device
  int32_t* d_off = nullptr;
  std::vector<int32_t*> d_slot_of_tv;  // per potential
  void* d_fixed = nullptr;             // V4<R> n_points: fixed values, w = mask bits
  void* d_force = nullptr;             // V4<R> n_points or null
  void* d_u = nullptr;
  void* d_p = nullptr;
  void* d_slots = nullptr;             // V4<R> [3][n_slots]
  double* d_partials = nullptr;
  unsigned* d_counter = nullptr;
};
