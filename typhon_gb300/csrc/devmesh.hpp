// Device-resident mesh and state of one ty_mesh handle (plain struct of device pointers,
// passed by value to the kernels).  Layout: structure-of-arrays, one contiguous FP64
// array per component, cells padded to a multiple of 32 so that every component starts
// 256-byte aligned.
//
//   cells  0 .. nci-1        interior cells (Typhon's numbering)
//          nci .. nc-1       ghost cells, one per boundary face
//   faces  0 .. nfi-1        interior faces, nfi .. nf-1 boundary faces
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace tyk {

constexpr int kMaxSlot = 8;    // faces per cell held in the gather list (hexahedra need 6)
constexpr int kMaxStage = 6;   // Runge-Kutta stages

struct DevMesh {
  int dim = 0, nci = 0, nc = 0, nfi = 0, nf = 0, ng = 0, nslot = 0;
  int ldc = 0;  // leading dimension of cell arrays (>= nc, multiple of 32)
  int ldf = 0;  // leading dimension of face arrays (>= nf, multiple of 32)
  // connectivity
  const int* fc1 = nullptr;    // [nf] cell on the normal's tail
  const int* fc2 = nullptr;    // [nf] cell on the normal's head (ghost for boundary faces)
  const int* fbc = nullptr;    // [nf] ty_bc kind
  const int* part = nullptr;   // [nf] periodic partner face or -1
  const int* cf = nullptr;     // [nslot][nci] (face << 1 | side), side 1 = cell is fc2; -1 pad;
                               // slots in Typhon's colour order (summation order)
  const int* gsrc = nullptr;   // [ng] interior cell that feeds each ghost
  const int* gface = nullptr;  // [ng] boundary face of each ghost
  // geometry
  const double* fn = nullptr;     // [3][ldf] unit normal
  const double* fs = nullptr;     // [ldf] surface
  const double* fwall = nullptr;  // [3][ldf] wall velocity
  const double* fbcd = nullptr;   // [6][ldf] inlet / outlet parameters (ty_set_bc_data)
  const double* cvol = nullptr;   // [ldc]
  const double* sumS = nullptr;   // [nci] sum of face surfaces, colour order (time step)
  const double* dcg = nullptr;    // [3][ldf] centre(fc2) - centre(fc1) (LSQ, weighted for W-LSQ)
  const double* lsq = nullptr;    // [6][nci] Cholesky factor L11 L21 L31 L22 L32 L33
  const double* lsqw = nullptr;   // [6][ldf] fast mode: per face, A^-1 d for fc1 (0..2), fc2 (3..5)
  const double* uLR = nullptr;    // [3][ldf] MUSCL direction (unit for MUSCL/-UNS, 1/dLR-scaled for FAST)
  const double* dLR = nullptr;    // [ldf]
  const double* kLF = nullptr;    // [ldf] MUSCL-FAST |F - C_L|
  const double* kRF = nullptr;    // [ldf] MUSCL-FAST -|F - C_R|
  const double* LF = nullptr;     // [3][ldf] MUSCL/-UNS F - C_L
  const double* RF = nullptr;     // [3][ldf] MUSCL/-UNS F - C_R
  const double* recw = nullptr;   // [8][ldf] fast MUSCL/-UNS without limiter: per side w (3), k (1),
                                  // face increment = grad q . w + (q_nb - q_c) k
  const double* invdLR = nullptr; // [ldf] 1 / dLR (fast mode)
  const double* mtab = nullptr;   // [nslot][nslot][nci] fast MUSCL/-UNS without limiter: the face
                                  // increments of a cell are linear in its neighbour differences,
                                  // D_i = sum_j M_ij dq_j (gradient and reconstruction folded);
                                  // null when not built
  const int* cfn = nullptr;       // [nslot][nci] neighbour cell across each gather-list face
  const double* invV = nullptr;   // [nci] 1 / V (fast mode)
  const double* geo2 = nullptr;   // [nci] 2 V / sum S (fast mode time step)
  const double* vgeo = nullptr;   // [5][ldf] viscous flux: HL/(HL+HR), HR/(HL+HR), C_R - C_L (3)
  const double* gdist = nullptr;  // [ng] wall ghosts: |F - C|^2 / |(F - C).n| (setboco_ns_flux.f90)
  const double* frot = nullptr;   // [9][ldf] periodic faces connected by a rotation: the row-major
                                  // rotation bringing the partner's vectors into the face's frame
                                  // (transvec_per); null when no family is rotational
};

struct DevState {
  double* u0 = nullptr;    // [5][ldc] state at the start of the step (the solution between steps)
  double* cur = nullptr;   // [5][ldc] state of the current stage
  double* acc = nullptr;   // [5][ldc] Runge-Kutta combination sum coef(n,s) rhs_s
  double* pk[kMaxStage + 1] = {};  // [5][ldc] partial sums of later stage states
  double* prim = nullptr;  // [5][ldc] rho, p, u, v, w (ghosts included)
  double* grad = nullptr;  // [15][ldc] grad rho, grad p, du_i/dx_j (row i)
  double* cl = nullptr;    // [5][ldf] face states (post-limiter path)
  double* cr = nullptr;    // [5][ldf]
  double* ratio = nullptr; // [3][ldc] post-limiter ratios (rho, p, velocity)
  double* flux = nullptr;  // [5][ldf] face flux times surface
  double* res = nullptr;   // [5][ldc] residual of ty_residual
  double* stage = nullptr; // [5*nci] host-layout staging: rho, rhoE, rhou as (x,y,z) per cell
  unsigned long long* dtbits = nullptr;  // [4] minimum time step slots (bit pattern of a positive double)
  int* err = nullptr;      // [4] error word, first bad cell, ...
};

struct SpatOpts {
  int scheme, highres, limiter, postlim, gradmeth, mode;
  double gamma, entropy_fix;
  double inv_entropy_fix;  // 1 / entropy_fix (fast-mode Roe flux)
  double ig1, gig1;        // 1 / (gamma - 1), gamma / (gamma - 1) (fast-mode fluxes)
  // HLL family (TY_SCH_HLLC / HLLE and their B, K, KB variants): 1 HLLC, 2 HLLE, 0 other;
  // kinetic wave speeds; beta; f1 = sqrt(gamma/2), f2 = 1/(2 sqrt(pi)) of the kinetic estimates
  int hll_family, hll_kin;
  double hll_beta, hll_f1, hll_f2;
  int viscous, visc_law;
  double visc_kin, rgas, prandtl;
  double farfield[5];  // free stream of far-field faces (rho, p, u, v, w)
};

// One Runge-Kutta update applied at the end of a stage: partial sum of the state of stage
// `target`, P_target <- (u0 or P_target) + c * R.  The partial sum of the next stage is the
// next stage state (written to cur); later ones are kept in pk[target].
struct RkOp {
  int target;   // stage index (2..nstage) whose state the term belongs to
  int from_u0;  // 1: first term, start from u0; 0: accumulate into pk[target]
  int is_next;  // 1: target is the next stage (result goes to cur)
  double c;
};
struct RkStagePlan {
  int nops = 0;
  RkOp ops[kMaxStage];
  int acc_init = 0;   // 1: acc = c_acc * R; 0: acc = acc + c_acc * R
  double c_acc = 0;
  int final_stage = 0;  // 1: u0 <- u0 + acc
  int has_acc = 1;
  int store_acc = 0;    // final stage: also store acc (the residual of update_field)
  const double* dtloc = nullptr;  // per-cell time step [nci] (LOCAL_STABILITY_CONDITION), else the global one
};

// Kernel identifiers for the per-kernel timing of ty_profile_read.
enum KernelId {
  K_PRIM = 0, K_GHOST_PRIM, K_GRAD, K_GHOST_GRAD, K_FACE_STATES, K_BARTH, K_FACE_FLUX, K_FACE_FLUX_LIM,
  K_RK_UPDATE, K_GATHER, K_TIMESTEP, K_CELL_FAST, K_FACE_FLUX_FAST, K_IMP_FACE, K_IMP_DIAG, K_IMP_MATVEC,
  K_IMP_PRECOND, K_IMP_ORTHO, K_NUM
};

// Optional CUDA-event timing of every launch (host side only).
struct Prof {
  bool on = false;
  struct Rec { int id; cudaEvent_t a, b; };
  std::vector<Rec> rec;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaEvent_t get() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
  template <class F>
  void launch(int id, cudaStream_t st, F&& f) {
    if (!on) { f(); return; }
    cudaEvent_t a = get(), b = get();
    cudaEventRecord(a, st);
    f();
    cudaEventRecord(b, st);
    rec.push_back(Rec{id, a, b});
  }
  void reset() { rec.clear(); used = 0; }
  ~Prof() { for (auto e : pool) cudaEventDestroy(e); }
};

// Typhon's ghost rows in explicit runs (flux_to_res.f90:90-113, update_field.f90:38): the
// residual row of a ghost cell is the raw flux F S of its face (not scaled by dt/V), and the
// Runge-Kutta combination adds it to the ghost's conservative state like any cell's row.
// One stage of that bookkeeping: the stage's ghost state u0 + sum_{s<stage} cs[s] r_s (its
// primitive variables are kept), the stage's rows r_stage, and after the last stage
// u0 += cf[0] r_0 + ... + cf[n-1] r_{n-1}.
struct GhostRk {
  int stage = 0, nstage = 1;
  double cs[kMaxStage] = {};
  double cf[kMaxStage] = {};
};

// Launch sequences implemented once per arithmetic mode (kernels_exact.cu, kernels_fast.cu).
#define TY_DECLARE_MODE(NS)                                                                        \
  namespace NS {                                                                                   \
  cudaError_t prim_from(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* cons,   \
                        cudaStream_t st, Prof* pr);                                                 \
  cudaError_t residual_faces(const DevMesh& m, const DevState& s, const SpatOpts& o,               \
                             cudaStream_t st, Prof* pr);                                           \
  cudaError_t residual_gather(const DevMesh& m, const DevState& s, double dt,                      \
                              const unsigned long long* dtbits, cudaStream_t st, Prof* pr);        \
  cudaError_t rk_update(const DevMesh& m, const DevState& s, const SpatOpts& o,                    \
                        const RkStagePlan& plan, double dt, const unsigned long long* dtbits,      \
                        unsigned long long* dtbits_next, double cfl, cudaStream_t st, Prof* pr);   \
  cudaError_t timestep(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* cons, \
                       double cfl, unsigned long long* dtbits, cudaStream_t st, Prof* pr);         \
  cudaError_t unpack_state(const DevMesh& m, const DevState& s, cudaStream_t st);                  \
  cudaError_t ghost_rows(const DevMesh& m, const DevState& s, const SpatOpts& o, const GhostRk& r,   \
                         double* gcons, double* gres, double* gprim, cudaStream_t st);             \
  cudaError_t pack_state(const DevMesh& m, const DevState& s, cudaStream_t st);                    \
  }

TY_DECLARE_MODE(kexact)
TY_DECLARE_MODE(kfast)

namespace kfast {
// the per-cell increment matrices of DevMesh::mtab, from lsqw, recw and the gather lists
cudaError_t build_mtab(const DevMesh& m, double* mtab, cudaStream_t st);
}

}  // namespace tyk
