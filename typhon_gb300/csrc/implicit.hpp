// Device state of the implicit (backward Euler) step and the launchers of its kernels.
//
// Matrix: Typhon's block sparse BDLU (SOURCE/MATH/SPMAT_BDLU.f90:27-37): a 5x5 diagonal block
// per interior cell and, per interior face, an upper block (row fc1, column fc2) and a lower
// block (row fc2, column fc1).  Blocks are stored per face / per cell as 26 doubles (25
// row-major entries and one pad, so that every block starts 16-byte aligned) or, for the
// mixed-precision solve, 28 floats.
//
// Vectors of the linear solve are in Typhon's packed layout (GENFIELD.f90 pack_gfield): the
// five conserved variables of a cell side by side, cell after cell, interior cells only.
// Ghost rows of Typhon's system are identity rows with a zero right-hand side, so their
// unknowns stay zero through the whole solve and are not stored.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "devmesh.hpp"

namespace tyk {

constexpr int kBlk = 26;         // FP64 block stride (25 entries + pad)
constexpr int kBlk32 = 28;       // FP32 block stride (25 entries + pad to 16 bytes)
constexpr int kMaxKrylov = 64;   // largest NKRYLOV of Typhon's GMRES
constexpr int kMaxCgs = 32;      // largest restart length of the flexible GMRES (CGS2)
constexpr int kRedBlocks = 1216; // blocks of a reduction (152 SMs x 8), fixed for determinism
constexpr int kRedThreads = 256;
constexpr int kCgsThreads = 128;  // threads of a Krylov basis pass block (sums: (kMaxCgs + 1) x 128 doubles of shared memory)

struct ImpState {
  bool lists = false;
  int nk = 0;                 // Krylov vectors allocated
  bool fp64_blocks = false, fp32_blocks = false, jfnk = false;
  int* cfo = nullptr;         // [nslot][nci] (face << 1 | side) in ascending face order, -1 pad
  int* cfon = nullptr;        // [nslot][nci] cell across that face
  double* dtloc = nullptr;    // [nci] local time step of the step
  double* jacL = nullptr;     // [nf][kBlk] flux Jacobians times S (calc_jac_*, flux_to_res)
  double* jacR = nullptr;
  double* upper = nullptr;    // [nfi][kBlk]
  double* lower = nullptr;
  double* diag = nullptr;     // [nci][kBlk]
  double* dinv = nullptr;     // [nci][kBlk] inverse of the diagonal block (block Jacobi)
  float* upper32 = nullptr;   // [nfi][kBlk32]
  float* lower32 = nullptr;
  float* diag32 = nullptr;    // [nci][kBlk32]
  float* dinv32 = nullptr;
  double* b = nullptr;        // [5 nci] right-hand side (residual of the step)
  double* x = nullptr;        // [5 nci] solution (the update)
  double* r = nullptr;        // [5 nci]
  double* w = nullptr;        // [5 nci]
  double* V = nullptr;        // [nk + 1][5 nci] Krylov basis
  float* V32 = nullptr;       // [nk + 1][5 nci] Krylov basis of the mixed-precision flexible GMRES
  double* Z = nullptr;        // [nk][5 nci] preconditioned basis (flexible GMRES, FP64)
  float* Z32 = nullptr;       // [nk][5 nci] preconditioned basis (mixed precision)
  double* part = nullptr;     // [kMaxKrylov + 1][kRedBlocks] partial sums
  double* scal = nullptr;     // [4 * kMaxKrylov] device scalars (Hessenberg column, step sizes)
  unsigned* done = nullptr;   // [1] blocks finished in a one-launch reduction (zero between launches)
  double* upert = nullptr;    // [5][ldc] perturbed state (Jacobian-free products)
  double* r0 = nullptr;       // [5 nci] residual at the unperturbed state (Jacobian-free)
  double* bs = nullptr;       // [5 nci] right-hand side of the flexible GMRES with its rows scaled
  // Row scale S of the flexible GMRES system (equation v of every cell times rs[v]); the
  // mat-vec kernels return S A z, the preconditioner applies D^-1 S^-1, so the Krylov solve
  // minimises |S (b - A x)| over physical updates x.  Ones (exact no-ops) outside that solve.
  double rs[5] = {1.0, 1.0, 1.0, 1.0, 1.0};
  double rsi[5] = {1.0, 1.0, 1.0, 1.0, 1.0};  // 1 / rs
  double* pinned = nullptr;   // host mirror of scal (pinned)
  int last_local = 1;         // time step of the last step: per cell, or last_dt everywhere
  double last_dt = 0.0;
};

// Five per-variable factors passed by value to the flat vector kernels.
struct Row5 {
  double v[5];
};

// Arguments of the assembly kernels.
struct ImpArgs {
  int local_dt;               // 1: per-cell dtloc, 0: global minimum in dtbits[slot]
  int src;                    // face states: 0 reconstructed, 1 limited (cl/cr + ratio), 2 cl/cr as is
  int want64, want32;         // which block precisions to store
  const unsigned long long* dtg;  // global time step (bit pattern)
};

#define TY_DECLARE_IMPLICIT(NS)                                                                       \
  namespace NS {                                                                                      \
  cudaError_t imp_dtloc(const DevMesh& m, const DevState& s, const SpatOpts& o, const ImpState& im,     \
                        double cfl, unsigned long long* dtbits, cudaStream_t st);                      \
  cudaError_t imp_assemble(const DevMesh& m, const DevState& s, const SpatOpts& o, const ImpState& im,  \
                           const ImpArgs& a, cudaStream_t st, Prof* pr);                                \
  cudaError_t imp_rhs(const DevMesh& m, const DevState& s, const ImpState& im, const ImpArgs& a,        \
                      double* out, cudaStream_t st);                                                    \
  cudaError_t imp_matvec(const DevMesh& m, const ImpState& im, const double* x, const double* z,         \
                         double* y, cudaStream_t st, Prof* pr);                                         \
  cudaError_t imp_matvec32(const DevMesh& m, const ImpState& im, const float* z, double* y,              \
                           cudaStream_t st, Prof* pr);                                                  \
  cudaError_t imp_precond(const DevMesh& m, const ImpState& im, const double* v, const float* v32,       \
                          double* z, float* z32, cudaStream_t st, Prof* pr);                             \
  cudaError_t imp_x0_diag(const DevMesh& m, const ImpState& im, const double* b, double* x,             \
                          cudaStream_t st);                                                             \
  cudaError_t imp_dot(const double* a, const double* b, size_t n, double* part, double* out,              \
                      cudaStream_t st);                                                                 \
  cudaError_t imp_asum(const double* a, size_t n, double* part, double* out, cudaStream_t st);           \
  cudaError_t res_l1(int nci, const double* acc, size_t ld, double* part, double* out, cudaStream_t st);  \
  cudaError_t imp_mgs_pass(const double* vprev, const double* hprev, double* w, const double* vnext,    \
                           size_t n, double* part, double* out, cudaStream_t st);                        \
  cudaError_t imp_basis_pass(double* V, float* V32, size_t ldv, int nv, const double* c,                \
                             const double* src, const double* sp, int extend, size_t n, double* part,   \
                             unsigned* done, double* out, cudaStream_t st, Prof* pr);                   \
  cudaError_t imp_scale(const double* w, double s, double* v, size_t n, cudaStream_t st);                \
  cudaError_t imp_bicgstab_iter(const DevMesh& m, const ImpState& im, double* x, double* r1,             \
                                const double* r2, double* p, double* v, double* s, double* t, int first,  \
                                double* part, double* sc, cudaStream_t st, Prof* pr);                      \
  cudaError_t imp_axpy_multi(double* x, const double* V, const float* V32, size_t ldv, int j,            \
                             const double* y, int descending, size_t n, cudaStream_t st);               \
  cudaError_t imp_update_state(const DevMesh& m, DevState& s, const double* x, double* part,            \
                               double* out, cudaStream_t st);                                           \
  cudaError_t imp_perturb(const DevMesh& m, const double* u0, const double* z, double eps, double* up,   \
                          cudaStream_t st);                                                             \
  cudaError_t imp_fd_combine(const double* z, const float* z32, const double* rp, const double* r0,      \
                             double inv_eps, Row5 rs, double* w, size_t n, cudaStream_t st);             \
  cudaError_t imp_to_f32(const double* x, float* y, size_t n, cudaStream_t st);                          \
  cudaError_t imp_res_norms(const DevMesh& m, const ImpState& im, const ImpArgs& a, const double* b,     \
                            double* part, double* out, cudaStream_t st);                                 \
  }

TY_DECLARE_IMPLICIT(kexact)
TY_DECLARE_IMPLICIT(kfast)

}  // namespace tyk
