// Residual on device buffers and its adjoint (vector-Jacobian product), C ABI.
//
// Both act on the handle's resident state U (ty_state_upload_device): ty_residual_device
// writes R = dt/V sum(+-F S) (ty_residual's value) to a caller device buffer, and
// ty_adjoint_vjp writes lambda_U = (dR/dU)^T lambda_R for the inviscid residual, first order
// (HIGHRES = NONE) or second order (MUSCL or MUSCL-UNS with no limiter or van Albada, the
// Barth post-limiter frozen at the state's ratios; periodic meshes).  New: Typhon has no adjoint; the unsteady gradient of a
// functional (RK stages, checkpointing, torch.autograd) is composed from these two calls in
// typhon_gb300/adjoint.py.
#include <vector>

#include "handle.hpp"

using namespace tyk;
using namespace tyi;

#define ADJ_CALL(h, fn, ...) \
  ((h)->o.mode == TY_MODE_FAST ? tyk::kfast::fn(__VA_ARGS__) : tyk::kexact::fn(__VA_ARGS__))

extern "C" {

int ty_residual_device(ty_mesh* h, double dt, double* R) {
  int rc;
  if ((rc = ready(h))) return rc;
  if (!R) return TY_ERR_ARG;
  if ((rc = ensure_prim(h))) return rc;
  if ((rc = stage_faces(h))) return rc;
  cudaError_t e = ADJ_CALL(h, residual_gather, h->m, h->s, dt, nullptr, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "residual gather");
  const size_t n = h->m.nci;
  TY_CU(cudaMemcpy2DAsync(R, n * sizeof(double), h->s.res, h->m.ldc * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToDevice, h->stream));
  return TY_OK;
}

int ty_adjoint_vjp(ty_mesh* h, double dt, const double* lamR, double* lamU) {
  if (int rc = ready(h)) return rc;
  if (!lamR || !lamU) return TY_ERR_ARG;
  const bool second = h->o.highres != TY_HRES_NONE;
  if (h->o.viscous != TY_VISC_NONE ||
      (second && ((h->o.highres != TY_HRES_MUSCL && h->o.highres != TY_HRES_MUSCLUNS) ||
                  (h->o.limiter != TY_LIM_NONE && h->o.limiter != TY_LIM_ALBADA) || h->nonperiodic_bc)) ||
      (!second && h->o.postlim != TY_POSTLIM_NONE)) {
    tyi::set_error("ty_adjoint_vjp: inviscid residual, first order, or MUSCL / MUSCL-UNS with no limiter or van "
                   "Albada and the Barth post-limiter frozen (periodic boundaries)");
    return TY_ERR_UNSUPPORTED;
  }
  if (h->m.frot) {
    tyi::set_error("ty_adjoint_vjp: no adjoint on meshes with rotational periodicity");
    return TY_ERR_UNSUPPORTED;
  }
  if (h->o.scheme == TY_SCH_HLLE || h->o.scheme == TY_SCH_AUSMM || h->o.scheme > TY_SCH_HLLE || h->inout_bc) {
    tyi::set_error("ty_adjoint_vjp: the HLLE and AUSM-M fluxes, the HLLC / HLLE wave-speed variants and inlet / "
                   "outlet boundaries have no adjoint");
    return TY_ERR_UNSUPPORTED;
  }
  DevMesh& m = h->m;
  int rc;
  if (second && h->o.mode == TY_MODE_FAST) {
    // array-of-structures records, lambda read and written in the caller's layout
    if (!h->adj_cell &&
        ((rc = h->alloc(h->adj_cell, 32 * (size_t)m.ldc)) || (rc = h->alloc(h->adj_rec, 44 * (size_t)m.ldf)) ||
         (rc = h->alloc(h->adj_qg, 5 * (size_t)m.ldc)) || (rc = h->alloc(h->adj_ctb, 10 * (size_t)m.ldf)) ||
         (rc = h->alloc(h->adj_w, (3 + 3 * (size_t)m.nslot) * (size_t)m.nci))))
      return rc;
    if (h->adj_w_gradmeth != h->lsq_gradmeth) {
      cudaError_t e = kfast::adjoint_weights_fast(m, h->adj_w, h->stream);
      if (e != cudaSuccess) return cuda_fail(e, "adjoint weights");
      h->adj_w_gradmeth = h->lsq_gradmeth;
    }
    cudaError_t e = kfast::adjoint_vjp_muscl_fast(m, h->s, h->o, h->s.u0, lamR, m.nci, dt, h->adj_cell, h->adj_rec,
                                                  h->adj_qg, h->adj_ctb, h->adj_w, lamU, m.nci, h->stream);
    h->prim_valid = false;  // s.prim now holds this state's primitive variables and ghosts
    if (e != cudaSuccess) return cuda_fail(e, "adjoint");
    return TY_OK;
  }
  if (!second && h->o.mode == TY_MODE_FAST) {
    if (!h->adj_cell1 &&
        ((rc = h->alloc(h->adj_cell1, 12 * (size_t)m.ldc)) || (rc = h->alloc(h->adj_face1, 10 * (size_t)m.ldf))))
      return rc;
    cudaError_t e = kfast::adjoint_vjp_fast(m, h->o, h->s.u0, lamR, m.nci, dt, h->adj_cell1, h->adj_face1, lamU, m.nci,
                                            h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint");
    return TY_OK;
  }
  if (!h->adj_face) {
    if ((rc = h->alloc(h->adj_face, 10 * (size_t)m.ldf)) || (rc = h->alloc(h->adj_buf, 10 * (size_t)m.ldc)))
      return rc;
  }
  const size_t n = m.nci, ld = m.ldc;
  double* bR = h->adj_buf;
  double* bU = h->adj_buf + 5 * ld;
  TY_CU(cudaMemcpy2DAsync(bR, ld * sizeof(double), lamR, n * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToDevice, h->stream));
  cudaError_t e;
  if (second) {
    if (!h->adj_rec2 &&
        ((rc = h->alloc(h->adj_rec2, 50 * (size_t)m.ldf)) || (rc = h->alloc(h->adj_qg2, 20 * (size_t)m.ldc))))
      return rc;
    e = ADJ_CALL(h, adjoint_vjp_muscl, m, h->s, h->o, h->s.u0, bR, dt, h->adj_rec2, h->adj_qg2, bU, h->stream);
    h->prim_valid = false;  // s.prim now holds this state's primitive variables and ghosts
  } else {
    e = ADJ_CALL(h, adjoint_vjp, m, h->o, h->s.u0, bR, dt, h->adj_face, bU, h->stream);
  }
  if (e != cudaSuccess) return cuda_fail(e, "adjoint");
  TY_CU(cudaMemcpy2DAsync(lamU, n * sizeof(double), bU, ld * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToDevice, h->stream));
  return TY_OK;
}

}  // extern "C"
