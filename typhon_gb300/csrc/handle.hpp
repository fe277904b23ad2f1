// The ty_mesh handle and the helpers that the host translation units of libtyphon_gpu share.
#pragma once
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/typhon_gpu.h"
#include "devmesh.hpp"
#include "implicit.hpp"
#include "kdif.hpp"
#include "adjoint.hpp"
#include "internal.hpp"

namespace tyi {
inline int cuda_fail(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return TY_ERR_CUDA;
}
inline int pad32(int n) { return (n + 31) / 32 * 32; }
}  // namespace tyi

#define TY_CU(call)                                                  \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return tyi::cuda_fail(e_, #call);         \
  } while (0)

#define MODE_CALL(h, fn, ...) \
  ((h)->o.mode == TY_MODE_FAST ? tyk::kfast::fn(__VA_ARGS__) : tyk::kexact::fn(__VA_ARGS__))

using tyk::DevMesh;
using tyk::DevState;
using tyk::Prof;
using tyk::SpatOpts;

struct ty_mesh {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevMesh m;
  DevState s;
  SpatOpts o{};
  bool has_params = false, has_state = false, prim_valid = false, fast_ready = false;
  bool heat_bc = false;  // the mesh has TY_BC_HEAT (ghost-face) boundaries
  bool inout_bc = false, bcdata_set = false;  // inlets / outlets, and their parameters uploaded
  bool nonperiodic_bc = false;  // a boundary face that is not periodic
  std::vector<double> kd_k;  // host copy of the KDIF conductivity [nci]
  int nslot = 0;
  std::vector<void*> allocs;
  // host copies needed to derive mode-dependent arrays
  std::vector<int> fc1, fc2;
  std::vector<double> ccentre, fcentre, fnormal, fsurf, cvol;
  std::vector<int> cf;  // [nslot][nci]
  int lsq_gradmeth = -1, geo_highres = -1;
  bool visc_ready = false;
  double* dtbits_host = nullptr;  // pinned
  Prof prof;
  tyk::ImpState imp;  // implicit-step matrices and Krylov workspace (allocated on first use)
  tyk::KdifState kd;  // heat-conduction state (ty_kdif_setup)
  double* adj_face = nullptr;  // [10][ldf] adjoint face products (first use)
  double* adj_buf = nullptr;   // [2][5][ldc] adjoint staging
  double* adj_rec2 = nullptr;  // [50][ldf] reversed reconstructions (second-order adjoint, exact mode)
  double* adj_qg2 = nullptr;   // [20][ldc] adjoints of q and of the gradients (exact mode)
  // fast-mode second-order adjoint: cell records [nci][32], face records [nf][44], q adjoints
  // [5][ldc], least-squares terms per face side [nf][2][5], weight tables [3 + 3 nslot][nci]
  double* adj_cell = nullptr;
  double* adj_rec = nullptr;
  double* adj_qg = nullptr;
  double* adj_ctb = nullptr;
  double* adj_w = nullptr;
  int adj_w_gradmeth = -1;
  // fast-mode first-order adjoint: cell records [nci][12] (prim, dt/V lambda), face records [nf][10]
  double* adj_cell1 = nullptr;
  double* adj_face1 = nullptr;
  // ghost-row bookkeeping of explicit runs (ty_ghost_state_set): conservative states [5][ng],
  // stage rows [kMaxStage][5][ng], primitive variables of the last stage's state [5][ng]
  double* mtab_buf = nullptr;  // [nslot][nslot][nci] increment matrices (DevMesh::mtab)
  double* gcons = nullptr;
  double* gres = nullptr;
  double* gprim = nullptr;
  bool ghost_rows = false;
  double* steady_red = nullptr;  // [3 kRedBlocks + 3] partial and final residual sums of ty_steady_iteration
  double* steady_dtloc = nullptr;  // [nci] per-cell time step of ty_steady_iteration (local_dt)
  cudaStream_t own_stream = nullptr;

  template <class T>
  int alloc(T*& p, size_t n) {
    void* q = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) { tyi::set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e)); return TY_ERR_NOMEM; }
    allocs.push_back(q);
    p = (T*)q;
    return TY_OK;
  }
  template <class T>
  int upload(const T*& dst, const std::vector<T>& src) {
    T* d = nullptr;
    int rc = alloc(d, src.size());
    if (rc) return rc;
    if (!src.empty()) TY_CU(cudaMemcpy(d, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    dst = d;
    return TY_OK;
  }
};


namespace tyi {
// shared steps of the pipelines (api.cpp)
int check_err(ty_mesh* h);                       // read and clear the device error word
int set_dt_slot(ty_mesh* h, int slot, double v); // dtbits[slot] = v (stream-ordered)
int ensure_prim(ty_mesh* h);                     // primitive variables of the resident state
int ready(ty_mesh* h);                           // parameters and state present; device set
int stage_faces(ty_mesh* h);                     // ghost states .. face fluxes of s.prim
int ensure_lsq(ty_mesh* h);                      // least-squares factors (LSQ) on the device
}  // namespace tyi
