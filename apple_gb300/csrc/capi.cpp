// C ABI of apple_gb300: handle lifetimes, uploads and launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "agb_internal.h"
#include "kernels.h"
#include "solver.h"

namespace agb {
const char* last_error();
}

using namespace agb;

namespace {

template <class T>
int dalloc(T** p, size_t n) {
  *p = nullptr;
  AGB_CHECK_CUDA(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
  return AGB_OK;
}

int dalloc_bytes(void** p, size_t bytes) {
  *p = nullptr;
  AGB_CHECK_CUDA(cudaMalloc(p, std::max<size_t>(bytes, 16)));
  return AGB_OK;
}

int upload(void* d, const void* h, size_t bytes) {
  if (bytes == 0) return AGB_OK;
  AGB_CHECK_CUDA(cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice));
  return AGB_OK;
}

template <class T>
int dupload(T** d, const std::vector<T>& h) {
  int rc = dalloc(d, h.size());
  if (rc) return rc;
  return upload(*d, h.data(), h.size() * sizeof(T));
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

#define RC(call)           \
  do {                     \
    int rc_ = (call);      \
    if (rc_) return rc_;   \
  } while (0)

// element records of a plan in the kernels' layout
// D A per element (component-major like TilePlan::D) for activations
// act[6 e + k] = (a00 a11 a22 a01 a02 a12); A = I + sym(a)
std::vector<double> muscle_D(const TilePlan& plan, const std::vector<double>& act) {
  const size_t n = (size_t)plan.n_cells;
  std::vector<double> out(9 * n);
  for (size_t e = 0; e < n; ++e) {
    const double* a = &act[6 * e];
    const double A[3][3] = {{1.0 + a[0], a[3], a[4]}, {a[3], 1.0 + a[1], a[5]}, {a[4], a[5], 1.0 + a[2]}};
    for (int r = 0; r < 3; ++r)
      for (int j = 0; j < 3; ++j) {
        double v = 0.0;
        for (int m = 0; m < 3; ++m) v += plan.D[(3 * r + m) * n + e] * A[m][j];
        out[(3 * r + j) * n + e] = v;
      }
  }
  return out;
}

// the activation offset stream (FemView::act) of a muscle potential
int upload_act(const std::vector<double>& act, size_t n, int precision, void** d_act) {
  if (precision == AGB_F32) {
    std::vector<float> v(8 * n, 0.0f);
    for (size_t e = 0; e < n; ++e) {
      const double* a = &act[6 * e];
      float* s0 = &v[4 * e];
      float* s1 = &v[4 * (n + e)];
      s0[0] = (float)a[0];
      s0[1] = (float)a[1];
      s0[2] = (float)a[2];
      s0[3] = (float)a[3];
      s1[0] = (float)a[4];
      s1[1] = (float)a[5];
    }
    if (!*d_act) RC(dalloc_bytes(d_act, v.size() * sizeof(float)));
    return upload(*d_act, v.data(), v.size() * sizeof(float));
  }
  std::vector<double> v(6 * n);
  for (size_t e = 0; e < n; ++e)
    for (int k = 0; k < 6; ++k) v[k * n + e] = act[6 * e + k];
  if (!*d_act) RC(dalloc_bytes(d_act, v.size() * sizeof(double)));
  return upload(*d_act, v.data(), v.size() * sizeof(double));
}

int upload_records(const TilePlan& plan, int precision, void** d_rec, uint32_t** d_ids,
                   const std::vector<double>* D_override = nullptr) {
  const size_t n = (size_t)plan.n_cells;
  const std::vector<double>& D = D_override ? *D_override : plan.D;
  if (precision == AGB_F32) {
    std::vector<float> rec(12 * n);
    for (size_t e = 0; e < n; ++e) {
      float* A = &rec[4 * e];
      float* B = &rec[4 * (n + e)];
      float* C = &rec[4 * (2 * n + e)];
      for (int k = 0; k < 4; ++k) A[k] = (float)D[k * n + e];
      for (int k = 0; k < 4; ++k) B[k] = (float)D[(4 + k) * n + e];
      C[0] = (float)D[8 * n + e];
      C[1] = (float)plan.mudv[e];
      C[2] = (float)plan.lamdv[e];
      std::memcpy(&C[3], &plan.ids[e], 4);
    }
    if (!*d_rec) RC(dalloc_bytes(d_rec, rec.size() * sizeof(float)));
    return upload(*d_rec, rec.data(), rec.size() * sizeof(float));
  }
  std::vector<double> rec(11 * n);
  for (size_t k = 0; k < 9; ++k)
    std::memcpy(&rec[k * n], &D[k * n], n * sizeof(double));
  std::memcpy(&rec[9 * n], plan.mudv.data(), n * sizeof(double));
  std::memcpy(&rec[10 * n], plan.lamdv.data(), n * sizeof(double));
  if (!*d_rec) RC(dalloc_bytes(d_rec, rec.size() * sizeof(double)));
  RC(upload(*d_rec, rec.data(), rec.size() * sizeof(double)));
  if (*d_ids) return upload(*d_ids, plan.ids.data(), plan.ids.size() * sizeof(uint32_t));
  return dupload(d_ids, plan.ids);
}

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

int check_launch(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return AGB_E_CUDA;
  }
  return AGB_OK;
}

template <class R>
std::vector<R> pack_v4(const std::vector<double>& xyz, const std::vector<uint8_t>* mask) {
  const size_t n = xyz.size() / 3;
  std::vector<R> out(4 * n);
  for (size_t i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) out[4 * i + c] = (R)xyz[3 * i + c];
    out[4 * i + 3] = mask ? (R)(*mask)[i] : R(0);
  }
  return out;
}

// internal -> caller cell index and dV * fraction on the device (first use)
int ensure_vjp_tables(agb_fem* f) {
  if (f->d_elem_user) return AGB_OK;
  RC(dupload(&f->d_elem_user, f->plan.elem_user));
  if (f->precision == AGB_F64) {
    RC(dalloc_bytes(&f->d_vol, 8 * f->vol_internal.size()));
    return upload(f->d_vol, f->vol_internal.data(), 8 * f->vol_internal.size());
  }
  std::vector<float> v(f->vol_internal.begin(), f->vol_internal.end());
  RC(dalloc_bytes(&f->d_vol, 4 * v.size()));
  return upload(f->d_vol, v.data(), 4 * v.size());
}

// 64-bit FNV-1a over byte ranges: the checkpoint fingerprint of a solver
struct Fnv64 {
  uint64_t h = 0xcbf29ce484222325ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      h ^= c[i];
      h *= 0x100000001b3ull;
    }
  }
  template <class T>
  void vec(const std::vector<T>& v) {
    const uint64_t n = v.size();
    bytes(&n, sizeof(n));
    bytes(v.data(), v.size() * sizeof(T));
  }
  template <class T>
  void val(const T& v) {
    bytes(&v, sizeof(T));
  }
};

// What a checkpoint depends on besides its sizes: the mesh of every potential
// (tiles, corner ids, element geometry, mu dV, lambda dV), the fixed mask and
// values, the external force per vertex and the solver parameters.  Muscle
// activations are left out: they are a control input that
// agb_fem_set_activation changes in place between solves.
uint64_t solver_fingerprint(const agb_model* m, const agb_pncg_params& prm, int precision, int material) {
  Fnv64 f;
  f.val(precision);
  f.val(material);
  f.val(m->space->n_points);
  f.vec(m->mask_internal);
  f.vec(m->fixed_internal);
  f.vec(m->force_internal);
  for (const agb_fem* fe : m->fems) {
    f.val(fe->material);
    f.vec(fe->plan.tile_estart);
    f.vec(fe->plan.tile_vstart);
    f.vec(fe->plan.tv_vid);
    f.vec(fe->plan.ids);
    f.vec(fe->plan.D);
    f.vec(fe->plan.mudv);
    f.vec(fe->plan.lamdv);
  }
  f.val(prm.max_steps);
  f.val(prm.rtol);
  f.val(prm.atol);
  f.val(prm.armijo_c);
  f.val(prm.overstep);
  f.val(prm.beta_max);
  f.val(prm.max_backtracking);
  f.val(prm.refresh_ratio);
  return f.h;
}

}  // namespace

FemView agb_fem::view() const {
  FemView v{};
  v.material = material;
  v.n_tiles = plan.n_tiles;
  v.n_cells = plan.n_cells;
  v.tile_estart = d_tile_estart;
  v.tile_vstart = d_tile_vstart;
  v.tile_gstart = d_tile_gstart;
  v.group_estart = d_group_estart;
  v.tv_vid = d_tv_vid;
  v.rec = d_rec;
  v.ids = d_ids;
  v.act = d_act;
  return v;
}

extern "C" {

const char* agb_last_error(void) { return agb::last_error(); }
const char* agb_version(void) { return "apple_gb300 0.1.0 (sm_103a)"; }

// ---------------------------------------------------------------------------
// space
// ---------------------------------------------------------------------------
int agb_space_create(int32_t n_points, const double* points, agb_space** out) {
  AGB_REQUIRE(out && n_points >= 0, AGB_E_INVALID, "agb_space_create: bad arguments");
  *out = nullptr;
  agb_space* s = new (std::nothrow) agb_space();
  AGB_REQUIRE(s, AGB_E_INVALID, "agb_space_create: out of host memory");
  s->n_points = n_points;
  if (points) {
    s->user_of_internal = morton_order(n_points, points);
    s->points_internal.resize(3 * (size_t)n_points);
    for (int i = 0; i < n_points; ++i)
      for (int c = 0; c < 3; ++c) s->points_internal[3 * i + c] = points[3 * s->user_of_internal[i] + c];
  } else {
    s->user_of_internal.resize(n_points);
    for (int i = 0; i < n_points; ++i) s->user_of_internal[i] = i;
  }
  s->internal_of_user.resize(n_points);
  for (int i = 0; i < n_points; ++i) s->internal_of_user[s->user_of_internal[i]] = i;
  int rc = dupload(&s->d_user_of_internal, s->user_of_internal);
  if (rc) {
    delete s;
    return rc;
  }
  *out = s;
  return AGB_OK;
}

int agb_space_destroy(agb_space* s) {
  if (!s) return AGB_OK;
  dfree(s->d_user_of_internal);
  delete s;
  return AGB_OK;
}

int agb_space_order(const agb_space* s, int32_t* internal_of_user) {
  AGB_REQUIRE(s && internal_of_user, AGB_E_INVALID, "agb_space_order: null argument");
  std::memcpy(internal_of_user, s->internal_of_user.data(), sizeof(int32_t) * s->n_points);
  return AGB_OK;
}

int agb_region_compute(int32_t n_cells, const int32_t* cells, int32_t n_points,
                       const double* points, const double* fraction, double* dhdX, double* dV,
                       int32_t* n_nonpositive) {
  AGB_REQUIRE(n_cells >= 0 && (n_cells == 0 || (cells && points && dhdX && dV)), AGB_E_INVALID,
              "agb_region_compute: null argument");
  for (int64_t k = 0; k < 4 * (int64_t)n_cells; ++k)
    AGB_REQUIRE(cells[k] >= 0 && cells[k] < n_points, AGB_E_MESH,
                "agb_region_compute: point id %d outside [0, %d)", cells[k], n_points);
  std::vector<double> D9(9 * (size_t)n_cells);
  const int bad = region_compute(n_cells, cells, points, fraction, D9.data(), dV);
  for (int e = 0; e < n_cells; ++e) {
    double* row = dhdX + 12 * (size_t)e;
    for (int j = 0; j < 3; ++j) {
      row[3 + j] = D9[9 * (size_t)e + j];
      row[6 + j] = D9[9 * (size_t)e + 3 + j];
      row[9 + j] = D9[9 * (size_t)e + 6 + j];
      row[j] = -(row[3 + j] + row[6 + j] + row[9 + j]);
    }
  }
  if (n_nonpositive) *n_nonpositive = bad;
  return AGB_OK;
}

// ---------------------------------------------------------------------------
// FEM potential
// ---------------------------------------------------------------------------
int agb_fem_destroy(agb_fem* f) {
  if (!f) return AGB_OK;
  for (void* p : {(void*)f->d_tile_estart, (void*)f->d_tile_vstart, (void*)f->d_tile_gstart,
                  (void*)f->d_group_estart, (void*)f->d_tv_vid,
                  (void*)f->d_own_slot, (void*)f->d_own_off, f->d_rec, (void*)f->d_ids, f->d_u,
                  f->d_p, f->d_slots, (void*)f->d_partials, (void*)f->d_counter,
                  (void*)f->d_elem_user, f->d_vol, f->d_act})
    dfree(p);
  delete f;
  return AGB_OK;
}

int agb_fem_create(agb_space* space, int material, int precision, int32_t n_cells,
                   const int32_t* cells, const double* points, const double* dhdX,
                   const double* dV, const double* fraction, const double* mu,
                   const double* lambda, int32_t tile_elems, agb_fem** out) {
  clear_error();
  AGB_REQUIRE(out, AGB_E_INVALID, "agb_fem_create: out is null");
  *out = nullptr;
  AGB_REQUIRE(space, AGB_E_INVALID, "agb_fem_create: space is null");
  AGB_REQUIRE(material == AGB_ARAP || material == AGB_STABLE_NEO_HOOKEAN ||
                  material == AGB_STABLE_NEO_HOOKEAN_MUSCLE, AGB_E_INVALID,
              "agb_fem_create: unknown material %d", material);
  AGB_REQUIRE(precision == AGB_F32 || precision == AGB_F64, AGB_E_INVALID,
              "agb_fem_create: unknown precision %d", precision);
  AGB_REQUIRE(n_cells >= 0 && (n_cells == 0 || cells), AGB_E_INVALID, "agb_fem_create: cells");
  AGB_REQUIRE(mu || n_cells == 0, AGB_E_INVALID, "agb_fem_create: mu is null");
  AGB_REQUIRE(material == AGB_ARAP || lambda || n_cells == 0, AGB_E_INVALID,
              "agb_fem_create: lambda is null for stable Neo-Hookean");
  const int np = space->n_points;
  for (int64_t k = 0; k < 4 * (int64_t)n_cells; ++k)
    AGB_REQUIRE(cells[k] >= 0 && cells[k] < np, AGB_E_MESH,
                "agb_fem_create: cell %lld corner %lld has point id %d outside [0, %d)",
                (long long)(k / 4), (long long)(k % 4), cells[k], np);
  const double* pts_user = points;
  std::vector<double> pts_from_space;
  if (!pts_user && !space->points_internal.empty()) {
    pts_from_space.resize(3 * (size_t)np);
    for (int i = 0; i < np; ++i)
      for (int c = 0; c < 3; ++c)
        pts_from_space[3 * space->user_of_internal[i] + c] = space->points_internal[3 * i + c];
    pts_user = pts_from_space.data();
  }
  AGB_REQUIRE((dhdX && dV) || pts_user, AGB_E_INVALID,
              "agb_fem_create: need dhdX and dV, or rest positions");

  std::vector<double> D9(9 * (size_t)n_cells), vol(n_cells);
  if (pts_user && (!dhdX || !dV)) {
    std::vector<double> d9c(9 * (size_t)n_cells), vc(n_cells);
    region_compute(n_cells, cells, pts_user, nullptr, d9c.data(), vc.data());
    if (!dhdX) D9 = d9c;
    if (!dV) vol = vc;
  }
  if (dhdX)
    for (int e = 0; e < n_cells; ++e)
      for (int k = 0; k < 9; ++k) D9[9 * (size_t)e + k] = dhdX[12 * (size_t)e + 3 + k];
  if (dV)
    for (int e = 0; e < n_cells; ++e) vol[e] = dV[e];
  if (fraction)
    for (int e = 0; e < n_cells; ++e) vol[e] *= fraction[e];
  std::vector<double> mudv(n_cells), lamdv(n_cells, 0.0);
  for (int e = 0; e < n_cells; ++e) {
    mudv[e] = mu[e] * vol[e];
    if (lambda && material != AGB_ARAP) lamdv[e] = lambda[e] * vol[e];
  }
  std::vector<int32_t> cells_int(4 * (size_t)n_cells);
  for (size_t k = 0; k < cells_int.size(); ++k) cells_int[k] = space->internal_of_user[cells[k]];
  std::vector<double> centroid(3 * (size_t)n_cells);
  for (int e = 0; e < n_cells; ++e)
    for (int c = 0; c < 3; ++c) {
      double s = 0.0;
      for (int a = 0; a < 4; ++a)
        s += pts_user ? pts_user[3 * (size_t)cells[4 * e + a] + c]
                      : (c == 0 ? (double)cells_int[4 * e + a] : 0.0);
      centroid[3 * (size_t)e + c] = 0.25 * s;
    }

  agb_fem* f = new (std::nothrow) agb_fem();
  AGB_REQUIRE(f, AGB_E_INVALID, "agb_fem_create: out of host memory");
  f->space = space;
  f->material = material;
  f->precision = precision;
  int rc = build_tiles(n_cells, cells_int.data(), centroid.data(), D9.data(), mudv.data(),
                       lamdv.data(), tile_elems, &f->plan);
  std::vector<SlotMap> sm;
  if (!rc) {
    build_slots(np, {&f->plan}, &sm, &f->own_off);
    f->own_slots = sm[0];
    f->vol_internal.resize(n_cells);
    for (int e = 0; e < n_cells; ++e) f->vol_internal[e] = vol[f->plan.elem_user[e]];
  }
  const TilePlan& P = f->plan;
  const size_t v4 = v4_bytes(precision);
  const size_t n_part = (size_t)std::max(P.n_tiles, unpack_blocks(np)) * 2;
  if (!rc) rc = dupload(&f->d_tile_estart, P.tile_estart);
  if (!rc) rc = dupload(&f->d_tile_vstart, P.tile_vstart);
  if (!rc) rc = dupload(&f->d_tile_gstart, P.tile_gstart);
  if (!rc) rc = dupload(&f->d_group_estart, P.group_estart);
  if (!rc) rc = dupload(&f->d_tv_vid, P.tv_vid);
  if (!rc) rc = dupload(&f->d_own_slot, f->own_slots.slot_of_tv);
  if (!rc) rc = dupload(&f->d_own_off, f->own_off);
  if (!rc) rc = upload_records(P, precision, &f->d_rec, &f->d_ids);
  if (!rc && material == AGB_STABLE_NEO_HOOKEAN_MUSCLE) {
    f->act_internal.assign(6 * (size_t)n_cells, 0.0);
    rc = upload_act(f->act_internal, (size_t)n_cells, precision, &f->d_act);
  }
  if (!rc) rc = dalloc_bytes(&f->d_u, v4 * np);
  if (!rc) rc = dalloc_bytes(&f->d_p, v4 * np);
  if (!rc) rc = dalloc_bytes(&f->d_slots, v4 * 3 * (size_t)P.n_tv);
  if (!rc) rc = dalloc(&f->d_partials, n_part);
  if (!rc) rc = dalloc(&f->d_counter, 1);
  if (!rc && cudaMemset(f->d_counter, 0, sizeof(unsigned)) != cudaSuccess) rc = AGB_E_CUDA;
  if (rc) {
    if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_fem_create: CUDA allocation failed");
    agb_fem_destroy(f);
    return rc;
  }
  *out = f;
  return AGB_OK;
}

int agb_fem_info(const agb_fem* f, int32_t* n_tiles, int32_t* n_tv) {
  AGB_REQUIRE(f, AGB_E_INVALID, "agb_fem_info: null handle");
  if (n_tiles) *n_tiles = f->plan.n_tiles;
  if (n_tv) *n_tv = f->plan.n_tv;
  return AGB_OK;
}

int agb_plan_tiles(int32_t n_points, int32_t n_cells, const int32_t* cells, const double* points,
                   int32_t tile_elems, int32_t* n_tiles, int32_t* n_groups, int32_t* tile_of_cell,
                   int32_t* group_of_cell, int32_t* slot_cells) {
  AGB_REQUIRE(n_points > 0 && n_cells >= 0 && (n_cells == 0 || cells) && points && tile_elems >= 0 && n_tiles &&
                  n_groups,
              AGB_E_INVALID, "agb_plan_tiles: bad arguments");
  for (int64_t k = 0; k < 4 * (int64_t)n_cells; ++k)
    AGB_REQUIRE(cells[k] >= 0 && cells[k] < n_points, AGB_E_MESH,
                "agb_plan_tiles: cell %lld corner %lld has point id %d outside [0, %d)", (long long)(k / 4),
                (long long)(k % 4), cells[k], n_points);
  // the same vertex order and element order as agb_space_create + agb_fem_create
  const std::vector<int32_t> uoi = morton_order(n_points, points);
  std::vector<int32_t> iou(n_points);
  for (int i = 0; i < n_points; ++i) iou[uoi[i]] = i;
  std::vector<int32_t> cells_int(4 * (size_t)n_cells);
  for (size_t k = 0; k < cells_int.size(); ++k) cells_int[k] = iou[cells[k]];
  std::vector<double> centroid(3 * (size_t)n_cells), D9(9 * (size_t)n_cells, 0.0), zero(n_cells, 0.0);
  for (int e = 0; e < n_cells; ++e)
    for (int c = 0; c < 3; ++c) {
      double s = 0.0;
      for (int a = 0; a < 4; ++a) s += points[3 * (size_t)cells[4 * e + a] + c];
      centroid[3 * (size_t)e + c] = 0.25 * s;
    }
  TilePlan P;
  RC(build_tiles(n_cells, cells_int.data(), centroid.data(), D9.data(), zero.data(), zero.data(), tile_elems, &P));
  *n_tiles = P.n_tiles;
  *n_groups = (int32_t)P.group_estart.size() - 1;
  for (int t = 0; t < P.n_tiles; ++t) {
    const int vs = P.tile_vstart[t];
    for (int g = P.tile_gstart[t]; g < P.tile_gstart[t + 1]; ++g)
      for (int e = P.group_estart[g]; e < P.group_estart[g + 1]; ++e) {
        const int eu = P.elem_user[e];
        if (tile_of_cell) tile_of_cell[eu] = t;
        if (group_of_cell) group_of_cell[eu] = g;
        if (slot_cells)
          for (int a = 0; a < 4; ++a)
            slot_cells[4 * (size_t)eu + a] = uoi[P.tv_vid[vs + (int)((P.ids[e] >> (8 * a)) & 0xffu)]];
      }
  }
  return AGB_OK;
}

int agb_fem_cells(const agb_fem* f, int32_t* cells_out, uint32_t* tile_color_hash) {
  AGB_REQUIRE(f && cells_out, AGB_E_INVALID, "agb_fem_cells: null argument");
  const TilePlan& P = f->plan;
  const std::vector<int32_t>& uoi = f->space->user_of_internal;
  uint32_t h = 2166136261u;  // FNV-1a over (tile, group, element, corner order)
  auto mix = [&h](uint32_t v) {
    for (int k = 0; k < 4; ++k) {
      h ^= (v >> (8 * k)) & 0xffu;
      h *= 16777619u;
    }
  };
  for (int t = 0; t < P.n_tiles; ++t) {
    const int vs = P.tile_vstart[t];
    for (int g = P.tile_gstart[t]; g < P.tile_gstart[t + 1]; ++g) {
      mix((uint32_t)g);
      for (int e = P.group_estart[g]; e < P.group_estart[g + 1]; ++e) {
        const int eu = P.elem_user[e];
        mix((uint32_t)eu);
        for (int a = 0; a < 4; ++a) {
          const int l = (int)((P.ids[e] >> (8 * a)) & 0xffu);
          const int32_t v = uoi[P.tv_vid[vs + l]];
          cells_out[4 * (size_t)eu + a] = v;
          mix((uint32_t)v);
        }
      }
    }
  }
  if (tile_color_hash) *tile_color_hash = h;
  return AGB_OK;
}

int agb_fem_eval(agb_fem* f, unsigned flags, const void* u, const void* p, double* energy,
                 void* grad, void* diag, void* prod, double* quad, void* stream) {
  AGB_REQUIRE(f && u, AGB_E_INVALID, "agb_fem_eval: null handle or u");
  AGB_REQUIRE(!(flags & ~31u), AGB_E_INVALID, "agb_fem_eval: unknown flags %u", flags);
  AGB_REQUIRE(!(flags & AGB_FUN) || energy, AGB_E_INVALID, "agb_fem_eval: energy output is null");
  AGB_REQUIRE(!(flags & AGB_GRAD) || grad, AGB_E_INVALID, "agb_fem_eval: grad output is null");
  AGB_REQUIRE(!(flags & AGB_HESS_DIAG) || diag, AGB_E_INVALID, "agb_fem_eval: hess_diag output is null");
  AGB_REQUIRE(!(flags & AGB_HESS_PROD) || prod, AGB_E_INVALID, "agb_fem_eval: hess_prod output is null");
  AGB_REQUIRE(!(flags & AGB_HESS_QUAD) || quad, AGB_E_INVALID, "agb_fem_eval: hess_quad output is null");
  const bool need_p = flags & (AGB_HESS_PROD | AGB_HESS_QUAD);
  AGB_REQUIRE(!need_p || p, AGB_E_INVALID, "agb_fem_eval: p is null");
  if (!flags) return AGB_OK;
  cudaStream_t s = as_stream(stream);
  const int np = f->space->n_points;
  RC(check_launch(launch_pack(f->precision, np, f->space->d_user_of_internal, u, f->d_u,
                              need_p ? p : nullptr, f->d_p, s),
                  "pack"));
  RC(check_launch(launch_fem_eval(f->precision, f->view(), flags, f->d_u, f->d_p, f->d_own_slot,
                                  f->d_slots, f->plan.n_tv, f->d_partials, f->d_counter, energy,
                                  quad, s),
                  "fem_eval"));
  const unsigned vec = flags & (AGB_GRAD | AGB_HESS_DIAG | AGB_HESS_PROD);
  if (vec)
    RC(check_launch(launch_unpack(f->precision, np, f->space->d_user_of_internal, f->d_own_off,
                                  f->d_slots, f->plan.n_tv, vec, grad, diag, prod, nullptr,
                                  f->d_u, f->d_partials, f->d_counter, nullptr, s),
                    "unpack"));
  return AGB_OK;
}

int agb_fem_fun(agb_fem* f, const void* u, double* out, void* s) {
  return agb_fem_eval(f, AGB_FUN, u, nullptr, out, nullptr, nullptr, nullptr, nullptr, s);
}
int agb_fem_grad(agb_fem* f, const void* u, void* out, void* s) {
  return agb_fem_eval(f, AGB_GRAD, u, nullptr, nullptr, out, nullptr, nullptr, nullptr, s);
}
int agb_fem_hess_diag(agb_fem* f, const void* u, void* out, void* s) {
  return agb_fem_eval(f, AGB_HESS_DIAG, u, nullptr, nullptr, nullptr, out, nullptr, nullptr, s);
}
int agb_fem_hess_prod(agb_fem* f, const void* u, const void* p, void* out, void* s) {
  return agb_fem_eval(f, AGB_HESS_PROD, u, p, nullptr, nullptr, nullptr, out, nullptr, s);
}
int agb_fem_hess_quad(agb_fem* f, const void* u, const void* p, double* out, void* s) {
  return agb_fem_eval(f, AGB_HESS_QUAD, u, p, nullptr, nullptr, nullptr, nullptr, out, s);
}

// ---------------------------------------------------------------------------
// model
// ---------------------------------------------------------------------------
int agb_model_destroy(agb_model* m) {
  if (!m) return AGB_OK;
  for (int32_t* p : m->d_slot_of_tv) dfree(p);
  for (void* p : {(void*)m->d_off, m->d_fixed, m->d_force, m->d_u, m->d_p, m->d_slots,
                  (void*)m->d_partials, (void*)m->d_counter})
    dfree(p);
  delete m;
  return AGB_OK;
}

int agb_model_create(agb_space* space, int precision, int32_t n_pot, agb_fem* const* pots,
                     const uint8_t* fixed_mask, const double* fixed_values, int32_t n_force,
                     const int32_t* force_index, const double* force, agb_model** out) {
  clear_error();
  AGB_REQUIRE(out, AGB_E_INVALID, "agb_model_create: out is null");
  *out = nullptr;
  AGB_REQUIRE(space && n_pot >= 0 && (n_pot == 0 || pots), AGB_E_INVALID,
              "agb_model_create: need a space and a potential array");
  AGB_REQUIRE(precision == AGB_F32 || precision == AGB_F64, AGB_E_INVALID,
              "agb_model_create: unknown precision %d", precision);
  const int prec = precision;
  for (int k = 0; k < n_pot; ++k) {
    AGB_REQUIRE(pots[k], AGB_E_INVALID, "agb_model_create: potential %d is null", k);
    AGB_REQUIRE(pots[k]->space == space, AGB_E_INVALID,
                "agb_model_create: potential %d is on another space", k);
    AGB_REQUIRE(pots[k]->precision == prec, AGB_E_INVALID,
                "agb_model_create: potentials mix precisions");
  }
  AGB_REQUIRE(n_force >= 0 && (n_force == 0 || (force_index && force)), AGB_E_INVALID,
              "agb_model_create: force arrays");
  const int np = space->n_points;
  for (int k = 0; k < n_force; ++k)
    AGB_REQUIRE(force_index[k] >= 0 && force_index[k] < np, AGB_E_MESH,
                "agb_model_create: force index %d out of range", force_index[k]);

  agb_model* m = new (std::nothrow) agb_model();
  AGB_REQUIRE(m, AGB_E_INVALID, "agb_model_create: out of host memory");
  m->space = space;
  m->precision = prec;
  m->fems.assign(pots, pots + n_pot);
  std::vector<const TilePlan*> plans;
  for (agb_fem* f : m->fems) plans.push_back(&f->plan);
  build_slots(np, plans, &m->slots, &m->off);
  m->n_slots = m->off[np];
  m->mask_internal.assign(np, 0);
  m->fixed_internal.assign(3 * (size_t)np, 0.0);
  m->force_internal.assign(3 * (size_t)np, 0.0);
  for (int u = 0; u < np; ++u) {
    const int i = space->internal_of_user[u];
    uint8_t bits = 0;
    for (int c = 0; c < 3; ++c) {
      if (fixed_mask && fixed_mask[3 * (size_t)u + c]) bits |= (uint8_t)(1u << c);
      if (fixed_values && (bits >> c & 1u)) m->fixed_internal[3 * (size_t)i + c] = fixed_values[3 * (size_t)u + c];
    }
    m->mask_internal[i] = bits;
  }
  for (int k = 0; k < n_force; ++k) {
    const int i = space->internal_of_user[force_index[k]];
    for (int c = 0; c < 3; ++c) m->force_internal[3 * (size_t)i + c] += force[3 * (size_t)k + c];
  }
  m->n_force = n_force;
  const size_t v4 = v4_bytes(prec);
  int rc = dupload(&m->d_off, m->off);
  m->d_slot_of_tv.assign(n_pot, nullptr);
  for (int k = 0; k < n_pot && !rc; ++k) rc = dupload(&m->d_slot_of_tv[k], m->slots[k].slot_of_tv);
  if (!rc) rc = dalloc_bytes(&m->d_fixed, v4 * np);
  if (!rc) {
    if (prec == AGB_F64) {
      auto h = pack_v4<double>(m->fixed_internal, &m->mask_internal);
      rc = upload(m->d_fixed, h.data(), v4 * np);
    } else {
      auto h = pack_v4<float>(m->fixed_internal, &m->mask_internal);
      rc = upload(m->d_fixed, h.data(), v4 * np);
    }
  }
  if (!rc && n_force > 0) {
    rc = dalloc_bytes(&m->d_force, v4 * np);
    if (!rc) {
      if (prec == AGB_F64) {
        auto h = pack_v4<double>(m->force_internal, nullptr);
        rc = upload(m->d_force, h.data(), v4 * np);
      } else {
        auto h = pack_v4<float>(m->force_internal, nullptr);
        rc = upload(m->d_force, h.data(), v4 * np);
      }
    }
  }
  int max_tiles = 0;
  for (agb_fem* f : m->fems) max_tiles = std::max(max_tiles, f->plan.n_tiles);
  const size_t n_part = (size_t)std::max(max_tiles, unpack_blocks(np)) * 2;
  if (!rc) rc = dalloc_bytes(&m->d_u, v4 * np);
  if (!rc) rc = dalloc_bytes(&m->d_p, v4 * np);
  if (!rc) rc = dalloc_bytes(&m->d_slots, v4 * 3 * (size_t)m->n_slots);
  if (!rc) rc = dalloc(&m->d_partials, n_part);
  if (!rc) rc = dalloc(&m->d_counter, 1);
  if (!rc && cudaMemset(m->d_counter, 0, sizeof(unsigned)) != cudaSuccess) rc = AGB_E_CUDA;
  if (rc) {
    if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_model_create: CUDA allocation failed");
    agb_model_destroy(m);
    return rc;
  }
  *out = m;
  return AGB_OK;
}

int agb_dof_to_free(int32_t precision, int64_t n_free, const int64_t* free_index, const void* full,
                    void* free_out, void* stream) {
  clear_error();
  AGB_REQUIRE(precision == AGB_F32 || precision == AGB_F64, AGB_E_INVALID, "agb_dof_to_free: bad precision");
  AGB_REQUIRE(n_free >= 0, AGB_E_INVALID, "agb_dof_to_free: negative size");
  AGB_REQUIRE(n_free == 0 || (free_index && full && free_out), AGB_E_INVALID, "agb_dof_to_free: null argument");
  return check_launch(launch_dof_to_free(precision, n_free, free_index, full, free_out, as_stream(stream)),
                      "dof_to_free");
}

int agb_dof_to_full(int32_t precision, int64_t n_full, const int32_t* slot, const void* free_in,
                    const void* fill, void* full_out, void* stream) {
  clear_error();
  AGB_REQUIRE(precision == AGB_F32 || precision == AGB_F64, AGB_E_INVALID, "agb_dof_to_full: bad precision");
  AGB_REQUIRE(n_full >= 0, AGB_E_INVALID, "agb_dof_to_full: negative size");
  AGB_REQUIRE(n_full == 0 || (slot && full_out), AGB_E_INVALID, "agb_dof_to_full: null argument");
  return check_launch(launch_dof_to_full(precision, n_full, slot, free_in, fill, full_out, as_stream(stream)),
                      "dof_to_full");
}

int agb_model_eval(agb_model* m, unsigned flags, const void* u, const void* p, double* energy,
                   void* grad, void* diag, void* prod, double* quad, void* stream) {
  AGB_REQUIRE(m && u, AGB_E_INVALID, "agb_model_eval: null handle or u");
  AGB_REQUIRE(!(flags & ~31u), AGB_E_INVALID, "agb_model_eval: unknown flags %u", flags);
  const bool need_p = flags & (AGB_HESS_PROD | AGB_HESS_QUAD);
  AGB_REQUIRE(!need_p || p, AGB_E_INVALID, "agb_model_eval: p is null");
  AGB_REQUIRE(!(flags & AGB_FUN) || energy, AGB_E_INVALID, "agb_model_eval: energy is null");
  AGB_REQUIRE(!(flags & AGB_GRAD) || grad, AGB_E_INVALID, "agb_model_eval: grad is null");
  AGB_REQUIRE(!(flags & AGB_HESS_DIAG) || diag, AGB_E_INVALID, "agb_model_eval: hess_diag is null");
  AGB_REQUIRE(!(flags & AGB_HESS_PROD) || prod, AGB_E_INVALID, "agb_model_eval: hess_prod is null");
  AGB_REQUIRE(!(flags & AGB_HESS_QUAD) || quad, AGB_E_INVALID, "agb_model_eval: hess_quad is null");
  cudaStream_t s = as_stream(stream);
  const int np = m->space->n_points;
  const size_t vec_bytes = 3 * (size_t)np * real_bytes(m->precision);
  // WarpModel: zero, then every potential accumulates (warp/model/_model.py:13-36)
  if (flags & AGB_FUN) AGB_CHECK_CUDA(cudaMemsetAsync(energy, 0, sizeof(double), s));
  if (flags & AGB_HESS_QUAD) AGB_CHECK_CUDA(cudaMemsetAsync(quad, 0, sizeof(double), s));
  if (flags & AGB_GRAD) AGB_CHECK_CUDA(cudaMemsetAsync(grad, 0, vec_bytes, s));
  if (flags & AGB_HESS_DIAG) AGB_CHECK_CUDA(cudaMemsetAsync(diag, 0, vec_bytes, s));
  if (flags & AGB_HESS_PROD) AGB_CHECK_CUDA(cudaMemsetAsync(prod, 0, vec_bytes, s));
  if (!flags) return AGB_OK;
  RC(check_launch(launch_pack(m->precision, np, m->space->d_user_of_internal, u, m->d_u,
                              need_p ? p : nullptr, m->d_p, s),
                  "pack"));
  for (size_t k = 0; k < m->fems.size(); ++k)
    RC(check_launch(launch_fem_eval(m->precision, m->fems[k]->view(), flags, m->d_u, m->d_p,
                                    m->d_slot_of_tv[k], m->d_slots, m->n_slots, m->d_partials,
                                    m->d_counter, energy, quad, s),
                    "fem_eval"));
  const unsigned vec = flags & (AGB_GRAD | AGB_HESS_DIAG | AGB_HESS_PROD | AGB_FUN);
  const bool ext = m->d_force != nullptr;
  if ((vec & ~AGB_FUN) || (ext && (flags & AGB_FUN)))
    RC(check_launch(launch_unpack(m->precision, np, m->space->d_user_of_internal, m->d_off,
                                  m->d_slots, m->n_slots, vec, grad, diag, prod, m->d_force,
                                  m->d_u, m->d_partials, m->d_counter, energy, s),
                    "unpack"));
  return AGB_OK;
}

// ---------------------------------------------------------------------------
// PNCG solver
// ---------------------------------------------------------------------------
void agb_pncg_default_params(agb_pncg_params* p) {
  if (!p) return;
  p->max_steps = 1500;
  p->rtol = 1e-6;
  p->atol = 0.0;
  p->max_backtracking = 8;
  p->armijo_c = 1e-4;
  p->overstep = 1.0;
  p->beta_max = 10.0;
  p->refresh_ratio = -1.0;
}

int agb_solver_destroy(agb_solver* sv) {
  if (!sv) return AGB_OK;
  if (sv->loop_exec) cudaGraphExecDestroy(sv->loop_exec);
  if (sv->cg_exec) cudaGraphExecDestroy(sv->cg_exec);
  for (void* p : {sv->d_cg, sv->d_cg_part, (void*)sv->d_cg_cnt, (void*)sv->d_cg_state}) dfree(p);
  if (sv->h_cg_state) cudaFreeHost(sv->h_cg_state);
  if (sv->step_exec) cudaGraphExecDestroy(sv->step_exec);
  if (sv->capture_stream) cudaStreamDestroy(sv->capture_stream);
  for (void* p : {(void*)sv->d_tile_estart, (void*)sv->d_tile_vstart, (void*)sv->d_tile_gstart,
                  (void*)sv->d_group_estart, (void*)sv->d_tv_vid,
                  (void*)sv->d_slot_of_tv, sv->d_rec, (void*)sv->d_ids, sv->d_xa, sv->d_gd, sv->d_p0,
                  sv->d_p1, sv->d_xref, sv->d_gref, sv->d_svd, sv->d_slots, sv->d_part, (void*)sv->d_cnt,
                  (void*)sv->d_state, sv->d_u_tmp, sv->d_act})
    dfree(p);
  if (sv->h_state) cudaFreeHost(sv->h_state);
  delete sv;
  return AGB_OK;
}

// ARAP: both per-element SVD caches, 3 V4 per cell each
static size_t svd_cache_bytes(const agb_solver* sv) {
  return 2 * 3 * v4_bytes(sv->precision) * (size_t)sv->fv.n_cells;
}

int agb_solver_create(agb_model* m, const agb_pncg_params* params, agb_solver** out) {
  clear_error();
  AGB_REQUIRE(out && m, AGB_E_INVALID, "agb_solver_create: null argument");
  *out = nullptr;
  AGB_REQUIRE(!m->fems.empty(), AGB_E_INVALID, "agb_solver_create: the model has no FEM potential");
  // one material per solver; stable Neo-Hookean and muscle potentials mix as
  // muscles (a stable Neo-Hookean cell is a muscle cell with zero activation)
  bool any_arap = false, any_snh = false, any_muscle = false;
  int64_t n_cells = 0;
  for (agb_fem* f : m->fems) {
    n_cells += f->plan.n_cells;
    any_arap |= f->material == AGB_ARAP;
    any_snh |= f->material == AGB_STABLE_NEO_HOOKEAN;
    any_muscle |= f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
  }
  AGB_REQUIRE(!(any_arap && (any_snh || any_muscle)), AGB_E_INVALID,
              "agb_solver_create: ARAP and stable Neo-Hookean potentials cannot share a solver");
  AGB_REQUIRE(n_cells > 0, AGB_E_INVALID, "agb_solver_create: the model's FEM potentials have no cells");
  const int mat = any_arap ? AGB_ARAP : (any_muscle ? AGB_STABLE_NEO_HOOKEAN_MUSCLE : AGB_STABLE_NEO_HOOKEAN);
  agb_pncg_params prm;
  agb_pncg_default_params(&prm);
  if (params) prm = *params;
  AGB_REQUIRE(prm.max_steps >= 0 && prm.max_backtracking >= 0 && prm.max_backtracking <= 60 &&
                  prm.refresh_ratio < 1.0,
              AGB_E_INVALID, "agb_solver_create: bad parameters");
  if (prm.refresh_ratio < 0.0) prm.refresh_ratio = (prm.rtol < 1e-5 && prm.atol == 0.0) ? 1e-1 : 0.0;
  agb_solver* sv = new (std::nothrow) agb_solver();
  AGB_REQUIRE(sv, AGB_E_INVALID, "agb_solver_create: out of host memory");
  sv->model = m;
  sv->params = prm;
  sv->precision = m->precision;
  sv->fingerprint = solver_fingerprint(m, prm, m->precision, mat);
  const int np = m->space->n_points;
  int rc = AGB_OK;
  // element data: one potential is used in place; several are concatenated
  std::vector<int32_t> slot_of_tv;
  if (m->fems.size() == 1) {
    sv->fv = m->fems[0]->view();
    slot_of_tv = m->slots[0].slot_of_tv;
  } else {
    TilePlan& P = sv->plan;
    P.tile_estart.assign(1, 0);
    P.tile_vstart.assign(1, 0);
    P.tile_gstart.assign(1, 0);
    P.group_estart.clear();
    for (size_t k = 0; k < m->fems.size(); ++k) {
      const TilePlan& Q = m->fems[k]->plan;
      const int eoff = P.n_cells, voff = P.n_tv, goff = (int)P.group_estart.size();
      for (int t = 0; t < Q.n_tiles; ++t) {
        P.tile_estart.push_back(eoff + Q.tile_estart[t + 1]);
        P.tile_vstart.push_back(voff + Q.tile_vstart[t + 1]);
        P.tile_gstart.push_back(goff + Q.tile_gstart[t + 1]);
      }
      for (size_t g = 0; g + 1 < Q.group_estart.size(); ++g) P.group_estart.push_back(eoff + Q.group_estart[g]);
      P.tv_vid.insert(P.tv_vid.end(), Q.tv_vid.begin(), Q.tv_vid.end());
      P.ids.insert(P.ids.end(), Q.ids.begin(), Q.ids.end());
      P.mudv.insert(P.mudv.end(), Q.mudv.begin(), Q.mudv.end());
      P.lamdv.insert(P.lamdv.end(), Q.lamdv.begin(), Q.lamdv.end());
      slot_of_tv.insert(slot_of_tv.end(), m->slots[k].slot_of_tv.begin(), m->slots[k].slot_of_tv.end());
      P.n_cells += Q.n_cells;
      P.n_tv += Q.n_tv;
      P.n_tiles += Q.n_tiles;
    }
    P.group_estart.push_back(P.n_cells);
    P.D.assign(9 * (size_t)P.n_cells, 0.0);
    // muscle solvers: records hold D A (D for stable Neo-Hookean potentials)
    // and the activation stream is concatenated (zeros for them)
    std::vector<double> act_all;
    if (mat == AGB_STABLE_NEO_HOOKEAN_MUSCLE) act_all.assign(6 * (size_t)P.n_cells, 0.0);
    int eoff = 0;
    for (agb_fem* f : m->fems) {
      const TilePlan& Q = f->plan;
      const bool muscle = f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
      const std::vector<double> DA = muscle ? muscle_D(Q, f->act_internal) : std::vector<double>();
      const std::vector<double>& Dq = muscle ? DA : Q.D;
      for (int k = 0; k < 9; ++k)
        std::memcpy(&P.D[(size_t)k * P.n_cells + eoff], &Dq[(size_t)k * Q.n_cells], sizeof(double) * Q.n_cells);
      if (muscle) std::memcpy(&act_all[6 * (size_t)eoff], f->act_internal.data(), sizeof(double) * 6 * Q.n_cells);
      eoff += Q.n_cells;
    }
    if (!rc && !act_all.empty()) rc = upload_act(act_all, (size_t)P.n_cells, sv->precision, &sv->d_act);
    if (!rc) rc = dupload(&sv->d_tile_estart, P.tile_estart);
    if (!rc) rc = dupload(&sv->d_tile_vstart, P.tile_vstart);
    if (!rc) rc = dupload(&sv->d_tile_gstart, P.tile_gstart);
    if (!rc) rc = dupload(&sv->d_group_estart, P.group_estart);
    if (!rc) rc = dupload(&sv->d_tv_vid, P.tv_vid);
    if (!rc) rc = upload_records(P, sv->precision, &sv->d_rec, &sv->d_ids);
    sv->fv.material = mat;
    sv->fv.n_tiles = P.n_tiles;
    sv->fv.n_cells = P.n_cells;
    sv->fv.tile_estart = sv->d_tile_estart;
    sv->fv.tile_vstart = sv->d_tile_vstart;
    sv->fv.tile_gstart = sv->d_tile_gstart;
    sv->fv.group_estart = sv->d_group_estart;
    sv->fv.tv_vid = sv->d_tv_vid;
    sv->fv.rec = sv->d_rec;
    sv->fv.ids = sv->d_ids;
    sv->fv.act = sv->d_act;
  }
  if (!rc) rc = dupload(&sv->d_slot_of_tv, slot_of_tv);
  const size_t v4 = v4_bytes(sv->precision);
  const int vblocks = solver_vertex_blocks(np);
  const size_t nt = (size_t)sv->fv.n_tiles;
  const size_t gt = (nt + 31) / 32, gv = ((size_t)vblocks + 31) / 32;
  // partials: direction (nt x 6 + gt x 6), gradient (nt), vertex (vb x 12 + gv x 12), trial (nt x 3 + gt x 3)
  const size_t off_ga = nt * 6, off_b = off_ga + gt * 6, off_v = off_b + nt, off_gv = off_v + (size_t)vblocks * 12,
               off_t = off_gv + gv * 12, off_gt = off_t + nt * 3, n_part = off_gt + gt * 3;
  const size_t n_cnt = (gt + 1) + (gv + 1) + (gt + 1);
  if (!rc) rc = dalloc_bytes(&sv->d_xa, 2 * v4 * np);
  if (!rc) rc = dalloc_bytes(&sv->d_gd, 2 * v4 * np);
  if (!rc) rc = dalloc_bytes(&sv->d_p0, v4 * np);
  if (!rc) rc = dalloc_bytes(&sv->d_p1, v4 * np);
  const bool delta = sv->precision == AGB_F32 && mat != AGB_ARAP && prm.refresh_ratio > 0.0;
  if (!rc && delta) rc = dalloc_bytes(&sv->d_xref, v4 * np);
  if (!rc && delta) rc = dalloc_bytes(&sv->d_gref, v4 * np);
  if (!rc && mat == AGB_ARAP) rc = dalloc_bytes(&sv->d_svd, svd_cache_bytes(sv));
  if (!rc) rc = dalloc_bytes(&sv->d_slots, v4 * 2 * (size_t)m->n_slots);
  if (!rc) rc = dalloc_bytes(&sv->d_part, 8 * n_part);
  if (!rc) rc = dalloc(&sv->d_cnt, n_cnt);
  if (!rc && cudaMemset(sv->d_cnt, 0, n_cnt * sizeof(unsigned)) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc && solver_prepare_kernels(sv->precision) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc) rc = dalloc(&sv->d_state, 1);
  if (!rc) rc = dalloc_bytes(&sv->d_u_tmp, 3 * real_bytes(sv->precision) * np);
  if (!rc && cudaMallocHost((void**)&sv->h_state, sizeof(SolverState)) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc && cudaStreamCreateWithFlags(&sv->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = AGB_E_CUDA;
  if (!rc) {
    SolverState st{};
    st.rtol = prm.rtol;
    st.atol = prm.atol;
    st.armijo_c = prm.armijo_c;
    st.overstep = prm.overstep;
    st.beta_max = prm.beta_max;
    st.max_steps = prm.max_steps;
    st.max_bt = prm.max_backtracking;
    st.done = 1;
    st.result = AGB_RUNNING;
    st.decided = 1;
    st.ref_ratio = delta ? prm.refresh_ratio : 0.0;
    rc = upload(sv->d_state, &st, sizeof(st));
  }
  if (rc) {
    if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_solver_create: CUDA allocation failed");
    agb_solver_destroy(sv);
    return rc;
  }
  SolveArgs& a = sv->args;
  a.fv = sv->fv;
  a.n_points = np;
  a.precision = sv->precision;
  a.xa = sv->d_xa;
  a.gd = sv->d_gd;
  a.p0 = sv->d_p0;
  a.p1 = sv->d_p1;
  a.xref = sv->d_xref;
  a.gref = sv->d_gref;
  a.svd = sv->d_svd;
  a.delta = delta ? 1 : 0;
  a.force = m->d_force;
  a.slot_of_tv = sv->d_slot_of_tv;
  a.off = m->d_off;
  a.slots = sv->d_slots;
  a.n_slots = m->n_slots;
  a.st = sv->d_state;
  char* part = (char*)sv->d_part;
  a.part_a = part;
  a.gpart_a = part + 8 * off_ga;
  a.part_b = part + 8 * off_b;
  a.part_v = part + 8 * off_v;
  a.gpart_v = part + 8 * off_gv;
  a.part_t = part + 8 * off_t;
  a.gpart_t = part + 8 * off_gt;
  a.cnt_a = sv->d_cnt;
  a.cnt_v = sv->d_cnt + (gt + 1);
  a.cnt_t = sv->d_cnt + (gt + 1) + (gv + 1);
  a.vblocks = vblocks;
  a.max_bt = prm.max_backtracking;
  a.cond = 0;
  a.cond_outer = 0;
  a.refresh_exits = 0;
  a.guard = 0;
  *out = sv;
  return AGB_OK;
}

int agb_solver_reset(agb_solver* sv, const void* u, void* stream) {
  AGB_REQUIRE(sv && u, AGB_E_INVALID, "agb_solver_reset: null argument");
  cudaStream_t s = as_stream(stream);
  RC(check_launch(launch_solver_init(sv->args, u, sv->model->d_fixed,
                                     sv->model->space->d_user_of_internal, s),
                  "solver_init"));
  if (sv->args.delta) {  // x_ref = x_0 and g(x_0) in FP64 before the first gradient pass
    RC(check_launch(launch_solver_force_refresh(sv->args, s), "solver_refresh"));
    RC(check_launch(launch_solver_refresh(sv->args, s), "solver_refresh"));
  }
  RC(check_launch(launch_solver_first(sv->args, s), "solver_first"));
  sv->has_state = true;
  return AGB_OK;
}

// Capture into `graph` after `deps` (which may be empty): the three passes
// of one iteration (refresh = false) or the two refresh passes as plain
// launches (refresh = true).
// Iterations per body of agb_solver_iterate's WHILE loop: the second of two
// is guarded (its passes return at once when the first ended the run), its
// direction pass a programmatic dependent of the first's vertex pass, and
// the loop's condition is evaluated once per two iterations.
#ifndef AGB_LOOP_UNROLL
#define AGB_LOOP_UNROLL 2
#endif

static cudaError_t capture_into(agb_solver* sv, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t n_deps,
                                const SolveArgs& a, bool refresh) {
  cudaStream_t cs = sv->capture_stream;
  cudaError_t e = cudaStreamBeginCaptureToGraph(cs, graph, deps, nullptr, n_deps, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = refresh ? launch_solver_refresh(a, cs, false) : launch_solver_iteration(a, a.cond != 0, cs);
  for (int k = 1; !refresh && le == cudaSuccess && k < AGB_LOOP_UNROLL; ++k) {
    SolveArgs ag = a;
    ag.guard = 1;
    le = launch_solver_iteration(ag, ag.cond != 0, cs);
  }
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(cs, &captured);
  return e == cudaSuccess ? le : e;
}

static cudaError_t add_conditional(cudaGraph_t g, const cudaGraphNode_t* deps, size_t n_deps,
                                   cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                                   cudaGraphNode_t* node, cudaGraph_t* body) {
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = 1;
  cudaError_t e = cudaGraphAddNode(node, g, deps, nullptr, n_deps, &np);
  if (e == cudaSuccess) *body = np.conditional.phGraph_out[0];
  return e;
}

// agb_solver_iterate's graph.  Without the reference-state correction:
//   WHILE(c) { direction, gradient, vertex }   (the vertex pass sets c).
// With it, the refresh passes run only when one is due:
//   WHILE(outer) { WHILE(c) { direction, gradient, vertex }; refresh element, refresh vertex }
// The vertex pass ends the inner loop when the solve ends, reaches the
// iteration limit or asks for a refresh; the refresh vertex pass (which does
// the refresh only if it was asked for) continues the outer loop and re-arms
// the inner one unless the solve ended or reached the limit.
static int build_loop_graph(agb_solver* sv) {
  cudaGraph_t g = nullptr;
  AGB_CHECK_CUDA(cudaGraphCreate(&g, 0));
  const SolveArgs& a = sv->args;
  cudaGraphConditionalHandle h_out = 0, h_in = 0;
  cudaGraphNode_t w_out = nullptr, w_in = nullptr;
  cudaGraph_t body_out = nullptr, body_in = nullptr;
  cudaError_t e = cudaSuccess;
  if (a.delta) {
    e = cudaGraphConditionalHandleCreate(&h_out, g, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = add_conditional(g, nullptr, 0, h_out, cudaGraphCondTypeWhile, &w_out, &body_out);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h_in, body_out, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = add_conditional(body_out, nullptr, 0, h_in, cudaGraphCondTypeWhile, &w_in, &body_in);
    if (e == cudaSuccess) {
      SolveArgs ai = a;
      ai.cond = (unsigned long long)h_in;
      ai.refresh_exits = 1;
      e = capture_into(sv, body_in, nullptr, 0, ai, false);
    }
    if (e == cudaSuccess) {
      SolveArgs ar = a;
      ar.cond = (unsigned long long)h_in;
      ar.cond_outer = (unsigned long long)h_out;
      e = capture_into(sv, body_out, &w_in, 1, ar, true);
    }
  } else {
    e = cudaGraphConditionalHandleCreate(&h_in, g, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = add_conditional(g, nullptr, 0, h_in, cudaGraphCondTypeWhile, &w_in, &body_in);
    if (e == cudaSuccess) {
      SolveArgs ai = a;
      ai.cond = (unsigned long long)h_in;
      e = capture_into(sv, body_in, nullptr, 0, ai, false);
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&sv->loop_exec, g, 0);
  cudaGraphDestroy(g);
  return check_launch(e, "solver loop graph");
}

// agb_solver_step's graph: one iteration; with the reference-state
// correction the two refresh passes follow as programmatic dependents and
// return at once unless a refresh is due (an IF node around them costs more
// than their idle launches: 130.8 against 124 us per iteration measured on
// the 1.5M-tet grid).
static int build_step_graph(agb_solver* sv) {
  cudaGraph_t g = nullptr;
  AGB_CHECK_CUDA(cudaGraphCreate(&g, 0));
  cudaStream_t cs = sv->capture_stream;
  const SolveArgs& a = sv->args;
  cudaError_t e = cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  size_t n_nodes = 0;
  if (e == cudaSuccess) {
    cudaError_t le = launch_solver_iteration(a, false, cs);
    if (le == cudaSuccess && a.delta) le = launch_solver_refresh(a, cs, true);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(cs, &captured);
    if (e == cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphGetNodes(g, nullptr, &n_nodes);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&sv->step_exec, g, 0);
  cudaGraphDestroy(g);
  sv->step_kernels = (int)n_nodes;
  return check_launch(e, "solver step graph");
}

int agb_solver_step_kernels(agb_solver* sv, int32_t* n_kernels) {
  AGB_REQUIRE(sv && n_kernels, AGB_E_INVALID, "agb_solver_step_kernels: null argument");
  if (!sv->step_exec) RC(build_step_graph(sv));
  *n_kernels = sv->step_kernels;
  return AGB_OK;
}

int agb_solver_iterate(agb_solver* sv, int32_t n_steps, void* stream) {
  AGB_REQUIRE(sv && n_steps >= 0, AGB_E_INVALID, "agb_solver_iterate: bad argument");
  if (n_steps == 0) return AGB_OK;
  if (!sv->loop_exec) RC(build_loop_graph(sv));
  cudaStream_t s = as_stream(stream);
  RC(check_launch(launch_solver_set_limit(sv->args, n_steps, s), "set_limit"));
  AGB_CHECK_CUDA(cudaGraphLaunch(sv->loop_exec, s));
  return AGB_OK;
}

int agb_solver_step(agb_solver* sv, void* stream) {
  AGB_REQUIRE(sv, AGB_E_INVALID, "agb_solver_step: null handle");
  if (!sv->step_exec) RC(build_step_graph(sv));
  AGB_CHECK_CUDA(cudaGraphLaunch(sv->step_exec, as_stream(stream)));
  return AGB_OK;
}

// the vertex pass stores the preconditioner's fill as its reciprocal
static double hess_diag_mean(const SolverState& st) { return st.inv_mean > 0.0 ? 1.0 / st.inv_mean : 1.0; }

int agb_solver_read(agb_solver* sv, void* u_out, agb_pncg_stats* stats, void* stream) {
  AGB_REQUIRE(sv, AGB_E_INVALID, "agb_solver_read: null handle");
  cudaStream_t s = as_stream(stream);
  if (u_out)
    RC(check_launch(launch_solver_unpack_x(sv->args, nullptr, sv->model->space->d_user_of_internal,
                                           u_out, s),
                    "unpack_x"));
  RC(check_launch(launch_solver_energy(sv->args, s), "solver_energy"));
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->h_state, sv->d_state, sizeof(SolverState),
                                 cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  const SolverState& st = *sv->h_state;
  if (stats) {
    stats->result = st.done ? st.result : AGB_RUNNING;
    stats->n_steps = st.iter;
    stats->grad_norm = st.gnorm;
    stats->grad_norm_first = st.gnorm0;
    stats->energy = st.energy;
    stats->alpha = st.ls_ok ? st.t : 0.0;
    stats->beta = st.beta;
    stats->line_search_steps = st.ls_steps;
    stats->line_search_ok = st.ls_ok;
    stats->hess_diag_mean = hess_diag_mean(st);
  }
  AGB_REQUIRE(st.error == 0, AGB_E_DEVICE, "solver: device guard %d tripped", st.error);
  return AGB_OK;
}

int agb_solver_read_direction(agb_solver* sv, void* p_host, void* stream) {
  AGB_REQUIRE(sv && p_host, AGB_E_INVALID, "agb_solver_read_direction: null argument");
  AGB_REQUIRE(sv->has_state, AGB_E_INVALID, "agb_solver_read_direction: call agb_solver_reset first");
  cudaStream_t s = as_stream(stream);
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->h_state, sv->d_state, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  // the vertex pass flips pbuf after each iteration, so p[pbuf] (the next
  // iteration's p_prev) holds the direction of the iteration just finished
  const void* src = sv->h_state->pbuf ? sv->d_p1 : sv->d_p0;
  const int np = sv->args.n_points;
  const size_t rb = real_bytes(sv->precision);
  std::vector<unsigned char> p4(4 * rb * (size_t)np);
  AGB_CHECK_CUDA(cudaMemcpyAsync(p4.data(), src, p4.size(), cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  const std::vector<int32_t>& uoi = sv->model->space->user_of_internal;
  unsigned char* out = static_cast<unsigned char*>(p_host);
  for (int i = 0; i < np; ++i)  // V4 (x, y, z, pad) at internal i -> 3 reals at caller uoi[i]
    std::memcpy(out + 3 * rb * (size_t)uoi[i], p4.data() + 4 * rb * (size_t)i, 3 * rb);
  return AGB_OK;
}

int agb_solver_read_gradient(agb_solver* sv, void* g_host, void* d_host, void* stream) {
  AGB_REQUIRE(sv, AGB_E_INVALID, "agb_solver_read_gradient: null handle");
  AGB_REQUIRE(sv->has_state, AGB_E_INVALID, "agb_solver_read_gradient: call agb_solver_reset first");
  cudaStream_t s = as_stream(stream);
  const int np = sv->args.n_points;
  const size_t rb = real_bytes(sv->precision);
  std::vector<unsigned char> gd(8 * rb * (size_t)np);  // per vertex: (g, 0), (d, 0)
  AGB_CHECK_CUDA(cudaMemcpyAsync(gd.data(), sv->d_gd, gd.size(), cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  const std::vector<int32_t>& uoi = sv->model->space->user_of_internal;
  unsigned char* go = static_cast<unsigned char*>(g_host);
  unsigned char* dout = static_cast<unsigned char*>(d_host);
  for (int i = 0; i < np; ++i) {
    const size_t o = 3 * rb * (size_t)uoi[i];
    if (go) std::memcpy(go + o, gd.data() + 8 * rb * (size_t)i, 3 * rb);
    if (dout) std::memcpy(dout + o, gd.data() + 8 * rb * (size_t)i + 4 * rb, 3 * rb);
  }
  return AGB_OK;
}

int agb_solver_read_reductions(agb_solver* sv, double* out5, void* stream) {
  AGB_REQUIRE(sv && out5, AGB_E_INVALID, "agb_solver_read_reductions: null argument");
  cudaStream_t s = as_stream(stream);
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->h_state, sv->d_state, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  const SolverState& st = *sv->h_state;
  out5[0] = st.hq;
  out5[1] = st.gd;
  out5[2] = st.gnorm;
  out5[3] = st.inv_mean;
  out5[4] = st.beta;
  return AGB_OK;
}

// checkpoint layout: header, then xa (2 V4 per vertex), gd (2 V4), p0, p1,
// [xref, gref when the FP32 correction is on], [the two SVD caches (ARAP)],
// SolverState
struct CheckpointHeader {
  uint64_t magic;
  int32_t version, precision, n_points, delta, state_bytes, pad;
  uint64_t fingerprint;  // solver_fingerprint of the saving solver
};
constexpr uint64_t kCheckpointMagic = 0x4147424350544b31ull;  // "AGBCPTK1"
constexpr int32_t kCheckpointVersion = 3;

static size_t checkpoint_vec_bytes(const agb_solver* sv) {
  const size_t v4 = v4_bytes(sv->precision) * (size_t)sv->args.n_points;
  return 2 * v4 + 2 * v4 + v4 + v4 + (sv->args.delta ? 2 * v4 : 0) + (sv->d_svd ? svd_cache_bytes(sv) : 0);
}

int agb_solver_checkpoint_size(agb_solver* sv, size_t* bytes) {
  AGB_REQUIRE(sv && bytes, AGB_E_INVALID, "agb_solver_checkpoint_size: null argument");
  *bytes = sizeof(CheckpointHeader) + checkpoint_vec_bytes(sv) + sizeof(SolverState);
  return AGB_OK;
}

static std::vector<std::pair<void*, size_t>> checkpoint_arrays(agb_solver* sv) {
  const size_t v4 = v4_bytes(sv->precision) * (size_t)sv->args.n_points;
  std::vector<std::pair<void*, size_t>> a = {{sv->d_xa, 2 * v4}, {sv->d_gd, 2 * v4}, {sv->d_p0, v4}, {sv->d_p1, v4}};
  if (sv->args.delta) {
    a.push_back({sv->d_xref, v4});
    a.push_back({sv->d_gref, v4});
  }
  if (sv->d_svd) a.push_back({sv->d_svd, svd_cache_bytes(sv)});
  a.push_back({(void*)sv->d_state, sizeof(SolverState)});
  return a;
}

int agb_solver_save(agb_solver* sv, void* host, void* stream) {
  AGB_REQUIRE(sv && host, AGB_E_INVALID, "agb_solver_save: null argument");
  cudaStream_t s = as_stream(stream);
  CheckpointHeader h{kCheckpointMagic, kCheckpointVersion, sv->precision, sv->args.n_points, sv->args.delta,
                     (int32_t)sizeof(SolverState), 0, sv->fingerprint};
  std::memcpy(host, &h, sizeof(h));
  char* dst = static_cast<char*>(host) + sizeof(h);
  for (const auto& [ptr, n] : checkpoint_arrays(sv)) {
    AGB_CHECK_CUDA(cudaMemcpyAsync(dst, ptr, n, cudaMemcpyDeviceToHost, s));
    dst += n;
  }
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  return AGB_OK;
}

int agb_solver_load(agb_solver* sv, const void* host, size_t bytes, void* stream) {
  clear_error();
  AGB_REQUIRE(sv && host, AGB_E_INVALID, "agb_solver_load: null argument");
  const size_t expect = sizeof(CheckpointHeader) + checkpoint_vec_bytes(sv) + sizeof(SolverState);
  AGB_REQUIRE(bytes >= sizeof(CheckpointHeader), AGB_E_INVALID,
              "agb_solver_load: %zu bytes is shorter than a checkpoint header", bytes);
  CheckpointHeader h;
  std::memcpy(&h, host, sizeof(h));
  AGB_REQUIRE(h.magic == kCheckpointMagic && h.version == kCheckpointVersion, AGB_E_INVALID,
              "agb_solver_load: not a checkpoint of this version");
  AGB_REQUIRE(bytes == expect, AGB_E_INVALID,
              "agb_solver_load: buffer of %zu bytes, this solver's checkpoints have %zu", bytes, expect);
  AGB_REQUIRE(h.precision == sv->precision && h.n_points == sv->args.n_points && h.delta == sv->args.delta &&
                  h.state_bytes == (int32_t)sizeof(SolverState),
              AGB_E_INVALID,
              "agb_solver_load: checkpoint of another solver (precision %d, %d points, correction %d)",
              h.precision, h.n_points, h.delta);
  AGB_REQUIRE(h.fingerprint == sv->fingerprint, AGB_E_INVALID,
              "agb_solver_load: checkpoint of another model or parameter set (fingerprint %016llx, "
              "this solver %016llx)",
              (unsigned long long)h.fingerprint, (unsigned long long)sv->fingerprint);
  cudaStream_t s = as_stream(stream);
  const char* src = static_cast<const char*>(host) + sizeof(h);
  for (const auto& [ptr, n] : checkpoint_arrays(sv)) {
    AGB_CHECK_CUDA(cudaMemcpyAsync(ptr, src, n, cudaMemcpyHostToDevice, s));
    src += n;
  }
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  sv->has_state = true;
  return AGB_OK;
}

int agb_solver_time_passes(agb_solver* sv, int32_t reps, void* flush, size_t flush_bytes,
                           float* ms, void* stream) {
  clear_error();
  AGB_REQUIRE(sv && ms && reps > 0, AGB_E_INVALID, "agb_solver_time_passes: bad argument");
  cudaStream_t s = as_stream(stream);
  cudaEvent_t e0, e1;
  AGB_CHECK_CUDA(cudaEventCreate(&e0));
  AGB_CHECK_CUDA(cudaEventCreate(&e1));
  int rc = AGB_OK;
  for (int which = 0; which < 3 && !rc; ++which) {
    float total = 0.0f;
    for (int r = 0; r < reps && !rc; ++r) {
      if (flush && flush_bytes && cudaMemsetAsync(flush, r & 0xff, flush_bytes, s) != cudaSuccess) rc = AGB_E_CUDA;
      if (!rc && cudaEventRecord(e0, s) != cudaSuccess) rc = AGB_E_CUDA;
      if (!rc) rc = check_launch(launch_solver_pass(sv->args, which, s), "time_passes");
      if (!rc && cudaEventRecord(e1, s) != cudaSuccess) rc = AGB_E_CUDA;
      float t = 0.0f;
      if (!rc && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
        rc = AGB_E_CUDA;
      total += t;
    }
    ms[which] = total / (float)reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_solver_time_passes: CUDA call failed");
  return rc;
}

int agb_pncg_minimize_host(agb_solver* sv, void* u_host, agb_pncg_stats* stats, void* stream) {
  AGB_REQUIRE(sv && u_host, AGB_E_INVALID, "agb_pncg_minimize_host: null argument");
  cudaStream_t s = as_stream(stream);
  const size_t bytes = 3 * real_bytes(sv->precision) * (size_t)sv->model->space->n_points;
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->d_u_tmp, u_host, bytes, cudaMemcpyHostToDevice, s));
  RC(agb_solver_reset(sv, sv->d_u_tmp, stream));
  RC(agb_solver_iterate(sv, sv->params.max_steps, stream));
  RC(agb_solver_read(sv, sv->d_u_tmp, stats, stream));
  AGB_CHECK_CUDA(cudaMemcpyAsync(u_host, sv->d_u_tmp, bytes, cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  return AGB_OK;
}


// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
void agb_cg_default_params(agb_cg_params* p) {
  if (!p) return;
  p->max_iter = 10000;
  p->rtol = 1e-6;
  p->atol = 0.0;
}

static int cg_setup(agb_solver* sv) {
  if (sv->d_cg) return AGB_OK;
  clear_error();
  const int np = sv->args.n_points;
  const size_t v4 = v4_bytes(sv->precision);
  const int vblocks = sv->args.vblocks;
  const size_t gv = ((size_t)vblocks + 31) / 32;
  int rc = dalloc_bytes(&sv->d_cg, 6 * v4 * (size_t)np);
  if (!rc) rc = dalloc_bytes(&sv->d_cg_part, 8 * 2 * ((size_t)vblocks + gv));
  if (!rc) rc = dalloc(&sv->d_cg_cnt, gv + 1);
  if (!rc && cudaMemset(sv->d_cg_cnt, 0, (gv + 1) * sizeof(unsigned)) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc) rc = dalloc(&sv->d_cg_state, 1);
  if (!rc && cudaMallocHost((void**)&sv->h_cg_state, sizeof(CgState)) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc && cg_prepare_kernels(sv->precision) != cudaSuccess) rc = AGB_E_CUDA;
  if (rc) {
    if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_solver_adjoint: CUDA allocation failed");
    return rc;
  }
  CgArgs& c = sv->cg;
  c.a = sv->args;
  char* base = (char*)sv->d_cg;
  const size_t vb = v4 * (size_t)np;
  c.lam = base;
  c.res = base + vb;
  c.q = base + 2 * vb;
  c.minv = base + 3 * vb;
  c.p0 = base + 4 * vb;
  c.p1 = base + 5 * vb;
  c.part = sv->d_cg_part;
  c.cnt = sv->d_cg_cnt;
  c.cs = sv->d_cg_state;
  c.vblocks = vblocks;
  c.cond = 0;
  return AGB_OK;
}

static int build_cg_graph(agb_solver* sv) {
  cudaGraph_t g = nullptr;
  AGB_CHECK_CUDA(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return check_launch(e, "cudaGraphConditionalHandleCreate");
  }
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return check_launch(e, "cudaGraphAddNode(conditional)");
  }
  cudaGraph_t body = np.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(sv->capture_stream, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    CgArgs c = sv->cg;
    c.cond = (unsigned long long)h;
    cudaError_t le = launch_cg_iteration(c, sv->capture_stream);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(sv->capture_stream, &captured);
    if (e == cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&sv->cg_exec, g, 0);
  cudaGraphDestroy(g);
  return check_launch(e, "adjoint CG graph");
}

int agb_solver_adjoint(agb_solver* sv, const void* rhs, void* lam, const agb_cg_params* params,
                       agb_cg_stats* stats, void* stream) {
  AGB_REQUIRE(sv && rhs && lam, AGB_E_INVALID, "agb_solver_adjoint: null argument");
  agb_cg_params prm;
  agb_cg_default_params(&prm);
  if (params) prm = *params;
  AGB_REQUIRE(prm.max_iter >= 0 && prm.rtol >= 0.0 && prm.atol >= 0.0, AGB_E_INVALID,
              "agb_solver_adjoint: bad parameters");
  RC(cg_setup(sv));
  if (!sv->cg_exec) RC(build_cg_graph(sv));
  cudaStream_t s = as_stream(stream);
  CgState init{};
  init.rtol = prm.rtol;
  init.atol = prm.atol;
  init.max_iter = prm.max_iter;
  init.done = 1;
  init.result = AGB_RUNNING;
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->d_cg_state, &init, sizeof(CgState), cudaMemcpyHostToDevice, s));
  const int32_t* uoi = sv->model->space->d_user_of_internal;
  RC(check_launch(launch_cg_init(sv->cg, rhs, uoi, s), "cg_init"));
  if (prm.max_iter > 0) {
    RC(check_launch(launch_cg_set_limit(sv->cg, prm.max_iter, s), "cg_set_limit"));
    AGB_CHECK_CUDA(cudaGraphLaunch(sv->cg_exec, s));
  }
  RC(check_launch(launch_cg_unpack(sv->cg, uoi, lam, s), "cg_unpack"));
  AGB_CHECK_CUDA(cudaMemcpyAsync(sv->h_cg_state, sv->d_cg_state, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  const CgState& cs = *sv->h_cg_state;
  if (stats) {
    stats->result = cs.done ? cs.result : AGB_MAX_STEPS_REACHED;
    stats->n_iter = cs.iter;
    stats->residual = std::sqrt(std::max(cs.rr, 0.0));
    stats->residual_first = std::sqrt(std::max(cs.rr0, 0.0));
  }
  return AGB_OK;
}

int agb_fem_grad_param_vjp(agb_fem* f, const void* u, const void* w, void* out_mu, void* out_lambda,
                           void* stream) {
  AGB_REQUIRE(f && u && w && out_mu, AGB_E_INVALID, "agb_fem_grad_param_vjp: null argument");
  cudaStream_t s = as_stream(stream);
  RC(ensure_vjp_tables(f));
  const int np = f->space->n_points;
  RC(check_launch(launch_pack(f->precision, np, f->space->d_user_of_internal, u, f->d_u, w, f->d_p, s),
                  "pack"));
  RC(check_launch(launch_param_vjp(f->view(), f->precision, f->d_u, f->d_p, f->d_vol, f->d_elem_user,
                                   out_mu, f->material != AGB_ARAP ? out_lambda : nullptr, s),
                  "param_vjp"));
  return AGB_OK;
}

// ---------------------------------------------------------------------------
// batched PNCG
// ---------------------------------------------------------------------------
int agb_batch_destroy(agb_batch* b) {
  if (!b) return AGB_OK;
  if (b->loop_exec) cudaGraphExecDestroy(b->loop_exec);
  if (b->step_exec) cudaGraphExecDestroy(b->step_exec);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  for (void* p : {(void*)b->d_tile_estart, (void*)b->d_tile_vstart, (void*)b->d_tile_gstart,
                  (void*)b->d_group_estart, (void*)b->d_tv_vid, b->d_rec, (void*)b->d_ids,
                  (void*)b->d_slot_of_tv, (void*)b->d_off, (void*)b->d_uoi, b->d_fixed, b->d_force,
                  (void*)b->d_tile_mesh, (void*)b->d_mesh_tile0, (void*)b->d_chunk_v0, (void*)b->d_chunk_mesh,
                  (void*)b->d_mesh_chunk0, b->d_xa, b->d_gd, b->d_p0, b->d_p1, b->d_xref, b->d_gref, b->d_slots,
                  b->d_svd, b->d_part, b->d_act,
                  (void*)b->d_state, (void*)b->d_bstate})
    dfree(p);
  if (b->h_state) cudaFreeHost(b->h_state);
  delete b;
  return AGB_OK;
}

int agb_batch_create(int32_t n_models, agb_model* const* models, const agb_pncg_params* params,
                     int32_t chunk_verts, agb_batch** out) {
  clear_error();
  AGB_REQUIRE(out && n_models > 0 && models, AGB_E_INVALID, "agb_batch_create: bad arguments");
  *out = nullptr;
  const int prec = models[0]->precision;
  for (int k = 0; k < n_models; ++k) {
    agb_model* m = models[k];
    AGB_REQUIRE(m && !m->fems.empty(), AGB_E_INVALID, "agb_batch_create: model %d has no FEM potential", k);
    AGB_REQUIRE(m->precision == prec, AGB_E_INVALID, "agb_batch_create: models must share a precision");
    int64_t n_cells = 0;
    for (agb_fem* f : m->fems) n_cells += f->plan.n_cells;
    AGB_REQUIRE(n_cells > 0, AGB_E_INVALID, "agb_batch_create: model %d: its FEM potentials have no cells", k);
  }
  // one material per batch, as per solver: ARAP, or stable Neo-Hookean and
  // muscle potentials, where with any muscle every cell runs as a muscle cell
  // (zero activation for the stable Neo-Hookean ones)
  bool any_muscle = false, any_arap = false, any_snh = false;
  for (int k = 0; k < n_models; ++k)
    for (agb_fem* f : models[k]->fems) {
      any_muscle |= f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
      any_arap |= f->material == AGB_ARAP;
      any_snh |= f->material == AGB_STABLE_NEO_HOOKEAN;
    }
  AGB_REQUIRE(!(any_arap && (any_snh || any_muscle)), AGB_E_INVALID,
              "agb_batch_create: ARAP and stable Neo-Hookean potentials cannot share a batch");
  const int bmat = any_arap ? AGB_ARAP : (any_muscle ? AGB_STABLE_NEO_HOOKEAN_MUSCLE : AGB_STABLE_NEO_HOOKEAN);
  agb_pncg_params prm;
  agb_pncg_default_params(&prm);
  if (params) prm = *params;
  AGB_REQUIRE(prm.max_steps >= 0 && prm.max_backtracking >= 0 && prm.max_backtracking <= 60, AGB_E_INVALID,
              "agb_batch_create: bad parameters");
  if (chunk_verts <= 0) chunk_verts = 512;
  AGB_REQUIRE(prm.refresh_ratio < 1.0, AGB_E_INVALID, "agb_batch_create: bad parameters");
  if (prm.refresh_ratio < 0.0) prm.refresh_ratio = (prm.rtol < 1e-5 && prm.atol == 0.0) ? 1e-1 : 0.0;
  const bool delta = prec == AGB_F32 && bmat != AGB_ARAP && prm.refresh_ratio > 0.0;
  agb_batch* b = new (std::nothrow) agb_batch();
  AGB_REQUIRE(b, AGB_E_INVALID, "agb_batch_create: out of host memory");
  b->models.assign(models, models + n_models);
  b->params = prm;
  b->precision = prec;
  b->chunk_verts = chunk_verts;
  // concatenation: vertices, tiles, slots, CSR, DOF data
  TilePlan& P = b->plan;
  P.tile_estart.assign(1, 0);
  P.tile_vstart.assign(1, 0);
  P.tile_gstart.assign(1, 0);
  P.group_estart.clear();
  std::vector<int32_t> slot_of_tv, off(1, 0), uoi, tile_mesh, mesh_tile0(1, 0), chunk_v0(1, 0), chunk_mesh,
      mesh_chunk0(1, 0);
  std::vector<double> fixed, force;
  std::vector<uint8_t> mask;
  bool any_force = false;
  b->vert_off.assign(1, 0);
  for (int k = 0; k < n_models; ++k) {
    agb_model* m = models[k];
    const int voff = b->vert_off.back(), np = m->space->n_points;
    const int soff = off.back();
    for (size_t q = 0; q < m->fems.size(); ++q) {
      const TilePlan& Q = m->fems[q]->plan;
      const int eoff = P.n_cells, tvoff = P.n_tv, goff = (int)P.group_estart.size();
      for (int t = 0; t < Q.n_tiles; ++t) {
        P.tile_estart.push_back(eoff + Q.tile_estart[t + 1]);
        P.tile_vstart.push_back(tvoff + Q.tile_vstart[t + 1]);
        P.tile_gstart.push_back(goff + Q.tile_gstart[t + 1]);
        tile_mesh.push_back(k);
      }
      for (size_t g = 0; g + 1 < Q.group_estart.size(); ++g) P.group_estart.push_back(eoff + Q.group_estart[g]);
      for (int32_t v : Q.tv_vid) P.tv_vid.push_back(voff + v);
      P.ids.insert(P.ids.end(), Q.ids.begin(), Q.ids.end());
      P.mudv.insert(P.mudv.end(), Q.mudv.begin(), Q.mudv.end());
      P.lamdv.insert(P.lamdv.end(), Q.lamdv.begin(), Q.lamdv.end());
      for (int32_t sl : m->slots[q].slot_of_tv) slot_of_tv.push_back(soff + sl);
      P.n_cells += Q.n_cells;
      P.n_tv += Q.n_tv;
      P.n_tiles += Q.n_tiles;
    }
    mesh_tile0.push_back(P.n_tiles);
    for (int i = 0; i < np; ++i) off.push_back(soff + m->off[i + 1]);
    for (int i = 0; i < np; ++i) uoi.push_back(voff + m->space->user_of_internal[i]);
    fixed.insert(fixed.end(), m->fixed_internal.begin(), m->fixed_internal.end());
    mask.insert(mask.end(), m->mask_internal.begin(), m->mask_internal.end());
    force.insert(force.end(), m->force_internal.begin(), m->force_internal.end());
    any_force = any_force || m->n_force > 0;
    for (int v = 0; v < np; v += chunk_verts) {
      chunk_v0.push_back(voff + std::min(np, v + chunk_verts));
      chunk_mesh.push_back(k);
    }
    mesh_chunk0.push_back((int32_t)chunk_mesh.size());
    b->vert_off.push_back(voff + np);
  }
  P.group_estart.push_back(P.n_cells);
  P.D.assign(9 * (size_t)P.n_cells, 0.0);
  std::vector<double> act_all;
  if (any_muscle) act_all.assign(6 * (size_t)P.n_cells, 0.0);
  {
    size_t eoff = 0;
    for (agb_model* m : b->models)
      for (agb_fem* f : m->fems) {
        const TilePlan& Q = f->plan;
        const bool muscle = f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
        const std::vector<double> DA = muscle ? muscle_D(Q, f->act_internal) : std::vector<double>();
        const std::vector<double>& Dq = muscle ? DA : Q.D;
        for (int c = 0; c < 9; ++c)
          std::memcpy(&P.D[(size_t)c * P.n_cells + eoff], &Dq[(size_t)c * Q.n_cells], sizeof(double) * Q.n_cells);
        if (muscle) std::memcpy(&act_all[6 * eoff], f->act_internal.data(), sizeof(double) * 6 * Q.n_cells);
        eoff += Q.n_cells;
      }
  }
  b->n_slots = off.back();
  const int np = b->vert_off.back();
  const int n_chunks = (int)chunk_mesh.size();
  const size_t v4 = v4_bytes(prec);
  int rc = dupload(&b->d_tile_estart, P.tile_estart);
  if (!rc) rc = dupload(&b->d_tile_vstart, P.tile_vstart);
  if (!rc) rc = dupload(&b->d_tile_gstart, P.tile_gstart);
  if (!rc) rc = dupload(&b->d_group_estart, P.group_estart);
  if (!rc) rc = dupload(&b->d_tv_vid, P.tv_vid);
  if (!rc) rc = upload_records(P, prec, &b->d_rec, &b->d_ids);
  if (!rc && any_muscle) rc = upload_act(act_all, (size_t)P.n_cells, prec, &b->d_act);
  if (!rc) rc = dupload(&b->d_slot_of_tv, slot_of_tv);
  if (!rc) rc = dupload(&b->d_off, off);
  if (!rc) rc = dupload(&b->d_uoi, uoi);
  if (!rc) rc = dupload(&b->d_tile_mesh, tile_mesh);
  if (!rc) rc = dupload(&b->d_mesh_tile0, mesh_tile0);
  if (!rc) rc = dupload(&b->d_chunk_v0, chunk_v0);
  if (!rc) rc = dupload(&b->d_chunk_mesh, chunk_mesh);
  if (!rc) rc = dupload(&b->d_mesh_chunk0, mesh_chunk0);
  if (!rc) rc = dalloc_bytes(&b->d_fixed, v4 * np);
  if (!rc) {
    if (prec == AGB_F64) {
      auto h = pack_v4<double>(fixed, &mask);
      rc = upload(b->d_fixed, h.data(), v4 * np);
    } else {
      auto h = pack_v4<float>(fixed, &mask);
      rc = upload(b->d_fixed, h.data(), v4 * np);
    }
  }
  if (!rc && any_force) {
    rc = dalloc_bytes(&b->d_force, v4 * np);
    if (!rc) {
      if (prec == AGB_F64) {
        auto h = pack_v4<double>(force, nullptr);
        rc = upload(b->d_force, h.data(), v4 * np);
      } else {
        auto h = pack_v4<float>(force, nullptr);
        rc = upload(b->d_force, h.data(), v4 * np);
      }
    }
  }
  if (!rc) rc = dalloc_bytes(&b->d_xa, 2 * v4 * np);
  if (!rc) rc = dalloc_bytes(&b->d_gd, 2 * v4 * np);
  if (!rc) rc = dalloc_bytes(&b->d_p0, v4 * np);
  if (!rc) rc = dalloc_bytes(&b->d_p1, v4 * np);
  if (!rc && delta) rc = dalloc_bytes(&b->d_xref, v4 * np);
  if (!rc && delta) rc = dalloc_bytes(&b->d_gref, v4 * np);
  if (!rc) rc = dalloc_bytes(&b->d_slots, 2 * v4 * (size_t)b->n_slots);
  if (!rc && bmat == AGB_ARAP) rc = dalloc_bytes(&b->d_svd, 2 * 3 * v4 * (size_t)P.n_cells);
  const size_t n_part = (size_t)P.n_tiles * 7 + (size_t)n_chunks * 12;
  if (!rc) rc = dalloc_bytes(&b->d_part, 8 * n_part);
  if (!rc) rc = dalloc(&b->d_state, (size_t)n_models);
  if (!rc) rc = dalloc(&b->d_bstate, 1);
  if (!rc && cudaMallocHost((void**)&b->h_state, sizeof(SolverState) * n_models) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc && cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking) != cudaSuccess) rc = AGB_E_CUDA;
  if (!rc && batch_prepare_kernels(prec) != cudaSuccess) rc = AGB_E_CUDA;
  if (rc) {
    if (rc == AGB_E_CUDA && agb::last_error()[0] == 0) set_error("agb_batch_create: CUDA allocation failed");
    agb_batch_destroy(b);
    return rc;
  }
  BatchArgs& ba = b->args;
  SolveArgs& a = ba.a;
  a.fv.material = bmat;
  a.fv.act = b->d_act;
  a.fv.n_tiles = P.n_tiles;
  a.fv.n_cells = P.n_cells;
  a.fv.tile_estart = b->d_tile_estart;
  a.fv.tile_vstart = b->d_tile_vstart;
  a.fv.tile_gstart = b->d_tile_gstart;
  a.fv.group_estart = b->d_group_estart;
  a.fv.tv_vid = b->d_tv_vid;
  a.fv.rec = b->d_rec;
  a.fv.ids = b->d_ids;
  a.n_points = np;
  a.precision = prec;
  a.xa = b->d_xa;
  a.gd = b->d_gd;
  a.p0 = b->d_p0;
  a.p1 = b->d_p1;
  a.xref = b->d_xref;
  a.gref = b->d_gref;
  a.delta = delta ? 1 : 0;
  a.force = b->d_force;
  a.slot_of_tv = b->d_slot_of_tv;
  a.off = b->d_off;
  a.slots = b->d_slots;
  a.n_slots = b->n_slots;
  a.svd = b->d_svd;
  a.st = nullptr;
  a.max_bt = prm.max_backtracking;
  ba.n_meshes = n_models;
  ba.n_chunks = n_chunks;
  ba.tile_mesh = b->d_tile_mesh;
  ba.mesh_tile0 = b->d_mesh_tile0;
  ba.chunk_v0 = b->d_chunk_v0;
  ba.chunk_mesh = b->d_chunk_mesh;
  ba.mesh_chunk0 = b->d_mesh_chunk0;
  ba.st = b->d_state;
  ba.bs = b->d_bstate;
  char* part = (char*)b->d_part;
  ba.part_dir = part;
  ba.part_grad = part + 8 * (size_t)P.n_tiles * 6;
  ba.part_vert = part + 8 * (size_t)P.n_tiles * 7;
  ba.cond = 0;
  // initial state: done until reset
  std::vector<SolverState> st0(n_models);
  for (auto& st : st0) {
    st = SolverState{};
    st.done = 1;
    st.result = AGB_RUNNING;
  }
  RC(upload(b->d_state, st0.data(), sizeof(SolverState) * n_models));
  *out = b;
  return AGB_OK;
}

int agb_batch_info(agb_batch* b, int32_t* n_points, int32_t* n_cells) {
  AGB_REQUIRE(b, AGB_E_INVALID, "agb_batch_info: null handle");
  if (n_points) *n_points = b->vert_off.back();
  if (n_cells) *n_cells = b->plan.n_cells;
  return AGB_OK;
}

int agb_batch_reset(agb_batch* b, const void* u, void* stream) {
  AGB_REQUIRE(b && u, AGB_E_INVALID, "agb_batch_reset: null argument");
  cudaStream_t s = as_stream(stream);
  SolverState proto{};
  proto.rtol = b->params.rtol;
  proto.atol = b->params.atol;
  proto.armijo_c = b->params.armijo_c;
  proto.overstep = b->params.overstep;
  proto.beta_max = b->params.beta_max;
  proto.max_steps = b->params.max_steps;
  proto.max_bt = b->params.max_backtracking;
  proto.ref_ratio = b->args.a.delta ? b->params.refresh_ratio : 0.0;
  RC(check_launch(launch_batch_init(b->args, u, b->d_fixed, b->d_uoi, proto, s), "batch_init"));
  RC(check_launch(launch_batch_first(b->args, s), "batch_first"));
  return AGB_OK;
}

static int build_batch_graph(agb_batch* b, bool loop) {
  cudaGraph_t g = nullptr;
  AGB_CHECK_CUDA(cudaGraphCreate(&g, 0));
  cudaGraph_t body = g;
  cudaGraphConditionalHandle h = 0;
  cudaError_t e = cudaSuccess;
  if (loop) {
    e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (e == cudaSuccess) body = np.conditional.phGraph_out[0];
  }
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(b->capture_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    BatchArgs a = b->args;
    a.cond = loop ? (unsigned long long)h : 0ull;
    cudaError_t le = launch_batch_iteration(a, b->capture_stream);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(b->capture_stream, &captured);
    if (e == cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(loop ? &b->loop_exec : &b->step_exec, g, 0);
  cudaGraphDestroy(g);
  return check_launch(e, loop ? "batch loop graph" : "batch step graph");
}

int agb_batch_iterate(agb_batch* b, int32_t n_steps, void* stream) {
  AGB_REQUIRE(b && n_steps >= 0, AGB_E_INVALID, "agb_batch_iterate: bad argument");
  if (n_steps == 0) return AGB_OK;
  if (!b->loop_exec) RC(build_batch_graph(b, true));
  cudaStream_t s = as_stream(stream);
  RC(check_launch(launch_batch_set_limit(b->args, n_steps, s), "batch_set_limit"));
  AGB_CHECK_CUDA(cudaGraphLaunch(b->loop_exec, s));
  return AGB_OK;
}

int agb_batch_step(agb_batch* b, void* stream) {
  AGB_REQUIRE(b, AGB_E_INVALID, "agb_batch_step: null handle");
  if (!b->step_exec) RC(build_batch_graph(b, false));
  AGB_CHECK_CUDA(cudaGraphLaunch(b->step_exec, as_stream(stream)));
  return AGB_OK;
}

int agb_batch_read(agb_batch* b, void* u_out, agb_pncg_stats* stats, void* stream) {
  AGB_REQUIRE(b, AGB_E_INVALID, "agb_batch_read: null handle");
  cudaStream_t s = as_stream(stream);
  if (u_out) {
    SolveArgs a = b->args.a;
    RC(check_launch(launch_solver_unpack_x(a, nullptr, b->d_uoi, u_out, s), "batch unpack"));
  }
  RC(check_launch(launch_batch_energy(b->args, s), "batch_energy"));
  const int n = (int)b->models.size();
  AGB_CHECK_CUDA(cudaMemcpyAsync(b->h_state, b->d_state, sizeof(SolverState) * n, cudaMemcpyDeviceToHost, s));
  AGB_CHECK_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    for (int k = 0; k < n; ++k) {
      const SolverState& st = b->h_state[k];
      stats[k].result = st.done ? st.result : AGB_RUNNING;
      stats[k].n_steps = st.iter;
      stats[k].grad_norm = st.gnorm;
      stats[k].grad_norm_first = st.gnorm0;
      stats[k].energy = st.energy;
      stats[k].alpha = st.ls_ok ? st.t : 0.0;
      stats[k].beta = st.beta;
      stats[k].line_search_steps = st.ls_steps;
      stats[k].line_search_ok = st.ls_ok;
      stats[k].hess_diag_mean = hess_diag_mean(st);
    }
  }
  for (int k = 0; k < n; ++k)
    AGB_REQUIRE(b->h_state[k].error == 0, AGB_E_DEVICE, "batch: device guard tripped in model %d", k);
  return AGB_OK;
}

int agb_fem_set_activation(agb_fem* f, const double* activation) {
  AGB_REQUIRE(f && activation, AGB_E_INVALID, "agb_fem_set_activation: null argument");
  AGB_REQUIRE(f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE, AGB_E_INVALID,
              "agb_fem_set_activation: not a muscle potential");
  const TilePlan& P = f->plan;
  const size_t n = (size_t)P.n_cells;
  for (size_t e = 0; e < n; ++e)
    for (int k = 0; k < 6; ++k) f->act_internal[6 * e + k] = activation[6 * (size_t)P.elem_user[e] + k];
  const std::vector<double> D = muscle_D(P, f->act_internal);
  RC(upload_records(P, f->precision, &f->d_rec, &f->d_ids, &D));
  return upload_act(f->act_internal, n, f->precision, &f->d_act);
}

int agb_fem_grad_activation_vjp(agb_fem* f, const void* u, const void* w, void* out_activation, void* stream) {
  AGB_REQUIRE(f && u && w && out_activation, AGB_E_INVALID, "agb_fem_grad_activation_vjp: null argument");
  AGB_REQUIRE(f->material == AGB_STABLE_NEO_HOOKEAN_MUSCLE, AGB_E_INVALID,
              "agb_fem_grad_activation_vjp: not a muscle potential");
  cudaStream_t s = as_stream(stream);
  RC(ensure_vjp_tables(f));
  const int np = f->space->n_points;
  RC(check_launch(launch_pack(f->precision, np, f->space->d_user_of_internal, u, f->d_u, w, f->d_p, s), "pack"));
  RC(check_launch(launch_activation_vjp(f->view(), f->precision, f->d_u, f->d_p, f->d_elem_user, out_activation, s),
                  "activation_vjp"));
  return AGB_OK;
}

}  // extern "C"
