/*
 * typhon_gpu.h — C ABI of the GB300 (sm_103a) finite-volume residual-and-update library.
 *
 * Drop-in for the explicit hot path of Typhon (Fortran 90 CFD solver, Haider-BA/typhon):
 * the zone residual, the Runge-Kutta stage and the time step.  Every entry point is
 * extern "C", takes plain pointers and sizes, and returns an int status (TY_OK = 0,
 * negative = TY_ERR_*).  Fortran binds it with ISO_C_BINDING, Python with ctypes.
 *
 * Conventions
 *   - A ty_mesh handle owns all device memory; state stays resident on the GPU between
 *     calls.  One CUDA stream per handle; calls on one handle are not re-entrant, calls on
 *     different handles are independent.
 *   - Index arrays are int32.  Arrays "in Typhon layout" are: facecell column-major
 *     fils(nface,2), 1-based; scalars as separate contiguous arrays; vectors as
 *     array-of-structs (x,y,z) per element, as st_genericfield stores them
 *     (CFDTOOLS/Mesh/Field/BASEFIELD.f90:30-54).
 *   - Conserved variables: rho, rho*E, rho*u (vector); primitive: rho, p, u (vector).
 *   - Errors that Typhon turns into error_stop (negative internal energy, NaN time step)
 *     are returned as status codes; the handle stays usable.
 */
#ifndef TYPHON_GPU_H
#define TYPHON_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define TY_OK 0
#define TY_ERR_ARG -1          /* bad argument (null pointer, size, enum value) */
#define TY_ERR_CUDA -2         /* CUDA runtime error (message in ty_last_error) */
#define TY_ERR_NOMEM -3        /* device allocation failed */
#define TY_ERR_MESH -4         /* inconsistent mesh description */
#define TY_ERR_NEGENERGY -5    /* negative or NaN internal energy in the time step */
#define TY_ERR_NANDT -6        /* NaN time step */
#define TY_ERR_STATE -7        /* call out of order (no state uploaded, no parameters set) */
#define TY_ERR_UNSUPPORTED -8  /* option not available */
#define TY_ERR_LSQ -9          /* least-squares matrix not positive definite */

/* ---- option enums (values match the oracle and the Python binding) ---- */
/* TY_SCH_HLLE: calc_flux_hlle.f90 (beta = 1) with the HLL Jacobian of its wave speeds. */
/* TY_SCH_AUSMM: calc_flux_ausmm.f90 (explicit only: Typhon has no AUSM-M Jacobian). */
/* The wave-speed variants of Typhon's HLLC and HLLE (SCHEME = HLLCB, HLLCK, HLLCKB, HLLEB,
 * HLLEK, HLLEKB; def_spat.f90:68-76, calc_flux_hllc.f90:64-124, calc_flux_hlle.f90:64-120):
 * B takes beta = sqrt((gamma-1)/(2 gamma)) in place of 1 in the outer wave speeds, K the
 * kinetic (EFM) estimates c (m (1 -+ erf m)/2 -+ exp(-m^2)/(2 sqrt pi)), m = u.n/c -+ beta
 * sqrt(gamma/2), c = a / sqrt(gamma/2).  The implicit step uses the HLL Jacobian of the same
 * speeds; the adjoint refuses them.  The K variants call erf and exp, whose device results
 * may differ from the C library's in the last bit: TY_MODE_EXACT is then within 1e-13 of the
 * CPU restatement instead of bit-identical. */
enum ty_scheme {
  TY_SCH_HLLC = 1, TY_SCH_RUSANOV = 2, TY_SCH_ROE = 3, TY_SCH_AUSMM = 4, TY_SCH_HLLE = 5,
  TY_SCH_HLLCB = 6, TY_SCH_HLLCK = 7, TY_SCH_HLLCKB = 8, TY_SCH_HLLEB = 9, TY_SCH_HLLEK = 10, TY_SCH_HLLEKB = 11
};
enum ty_highres { TY_HRES_NONE = 0, TY_HRES_MUSCL = 1, TY_HRES_MUSCLFAST = 2, TY_HRES_MUSCLUNS = 3 };
enum ty_limiter {
  TY_LIM_NONE = 0, TY_LIM_MINMOD = 1, TY_LIM_ALBADA = 2, TY_LIM_VLEER = 3,
  TY_LIM_SUPERBEE = 4, TY_LIM_KIM3 = 5, TY_LIM_LIM03 = 6
};
enum ty_postlim { TY_POSTLIM_NONE = 0, TY_POSTLIM_BARTH = 1, TY_POSTLIM_SUPERBARTH = 2 };
enum ty_gradmeth { TY_GRAD_NONE = 0, TY_GRAD_LSQ = 1, TY_GRAD_LSQW = 2 };
enum ty_rk {
  TY_RK_EXPLICIT = 0,  /* TIME_PARAM METHOD = EXPLICIT (treelevel_explicit.f90): forward Euler */
  TY_RK2 = 1, TY_RK2SSP = 2, TY_RK3SSP = 3, TY_RK4 = 4, TY_LSRK25BB = 5, TY_LSRK26BB = 6,
  TY_LSRK12BS = 7, TY_LSRK13BS = 8
};
/* TY_BC_FARFIELD (new: Typhon parses FAR-FIELD but has no Navier-Stokes implementation):
 * the kind of each far-field face follows the free-stream normal velocity vn = u_inf.n (n
 * outward) against the free-stream sound speed c: vn <= -c supersonic inflow (free stream),
 * vn < -1e-8 c subsonic inflow (free-stream density and velocity, inside pressure), vn < c
 * subsonic outflow (inside density and velocity, free-stream pressure; also a boundary
 * tangent to the free stream), else supersonic outflow (inside state).  The free stream is
 * ty_spat_params.farfield. */
/* TY_BC_NOSLIP (new): the adiabatic wall of TY_BC_WALL with the inside density in its face
 * state.  TY_BC_WALL keeps Typhon's face state, whose density is the inside PRESSURE
 * (setboco_ns_flux.f90:136, "density / weak BC"), for parity with Typhon. */
/* TY_BC_HEAT: a heat-conduction (KDIF) boundary, implemented as Typhon implements every
 * KDIF wall and the EXTRAPOLATE condition: by a ghost FACE (bctype_of_kdifboco, MENU_KDIF.f90:
 * 103-125; bctype_of_boco, MENU_BOCO.f90:126-150; init_ustboco_ghostface.f90), a ghost cell
 * at the face centre with zero volume.  The thermal kind and value of each face come from
 * ty_kdif_setup.  Not a Navier-Stokes boundary: the Navier-Stokes operations (residual,
 * steps, implicit, adjoint) refuse a mesh that has one; ty_set_params still sets the
 * arithmetic mode used by the KDIF calls. */
/* Inlets and outlets (Typhon's SUBSONIC_INLET, SUBSONIC_OUTLET, SUPERSONIC_INLET,
 * SUPERSONIC_OUTLET: setboco_ns_inlet_sub.f90, setboco_ns_outlet_sub.f90,
 * setboco_ns_inlet_sup.f90, setboco_ns_outlet_sup.f90), ghost faces as in Typhon
 * (bctype_of_nsboco, MENU_NS.f90:91-115).  Per-face parameters come from ty_set_bc_data:
 *   TY_BC_INLET_SUB   total pressure, total temperature, flow direction (3): the state of
 *                     those totals and direction at the inside static pressure
 *   TY_BC_OUTLET_SUB  static pressure: the inside state's totals and direction, expanded
 *                     isentropically to it
 *   TY_BC_INLET_SUP   total pressure, total temperature, Mach number, direction (3)
 *   TY_BC_OUTLET_SUP  none: the inside state (its Jacobian folded, ns_bocojacobian.f90)
 * They need ty_spat_params.rgas > 0. */
enum ty_bc {
  TY_BC_INTERIOR = 0, TY_BC_PERIODIC = 1, TY_BC_SYMMETRY = 2, TY_BC_WALL = 3, TY_BC_FARFIELD = 4,
  TY_BC_NOSLIP = 5, TY_BC_HEAT = 6, TY_BC_INLET_SUB = 7, TY_BC_OUTLET_SUB = 8, TY_BC_INLET_SUP = 9,
  TY_BC_OUTLET_SUP = 10
};
/* Arithmetic mode of the kernels.
 *   TY_MODE_EXACT: every FP64 operation in the order Typhon evaluates it, each rounded
 *                  separately (no fused multiply-add); results match the CPU restatement
 *                  bit for bit.
 *   TY_MODE_FAST:  algebraically rearranged (precomputed reciprocals and reconstruction
 *                  weights, fused multiply-add); agrees with EXACT to ~1e-13 relative. */
enum ty_mode { TY_MODE_EXACT = 0, TY_MODE_FAST = 1 };

/* Preprocessed mesh in Typhon's numbering (st_ustmesh after grid_preproc and
 * init_connect_grid): interior faces first, boundary faces last, one ghost cell per
 * boundary face numbered after the interior cells.
 * Replaces the umesh argument of integration_grid (SOURCE/MAIN/integration_grid.f90:8). */
typedef struct ty_mesh_desc {
  int32_t dim;              /* 2 (COORD=2D) or 3 */
  int32_t ncell_int;        /* interior cells */
  int32_t ncell;            /* interior + ghost cells */
  int32_t nface_int;        /* interior faces (first in the face list) */
  int32_t nface;            /* all faces */
  const int32_t* facecell;  /* [2*nface] fils(nface,2), 1-based, column-major */
  const double* face_normal;   /* [3*nface] unit normal from cell 1 to cell 2, AoS */
  const double* face_surface;  /* [nface] */
  const double* face_centre;   /* [3*nface] AoS */
  const double* cell_centre;   /* [3*ncell] AoS, ghost cells included */
  const double* cell_volume;   /* [ncell] */
  const int32_t* face_color;   /* [nface] colour group of each face (coo_colorgroup,
                                  0-based); fixes the summation order of the residual */
  const int32_t* face_bc;      /* [nface] ty_bc kind of each face (0 for interior faces);
                                  TY_BC_WALL: adiabatic wall moving at face_wallvel */
  const int32_t* face_partner; /* [nface] periodic partner face, 1-based, 0 if none */
  const double* face_wallvel;  /* [3*nface] wall velocity of wall faces, or NULL */
} ty_mesh_desc;

typedef struct ty_mesh ty_mesh;

typedef struct ty_spat_params {
  int32_t scheme;     /* ty_scheme   (SPAT_PARAM:SCHEME) */
  int32_t highres;    /* ty_highres  (SPAT_PARAM:HIGHRES) */
  int32_t limiter;    /* ty_limiter  (SPAT_PARAM:LIMITER) */
  int32_t postlim;    /* ty_postlim  (SPAT_PARAM:POST-LIMITER) */
  int32_t gradmeth;   /* ty_gradmeth (SPAT_PARAM:GRADMETH) */
  int32_t mode;       /* ty_mode */
  double gamma;       /* ratio of specific heats (AIR: 1.4) */
  double entropy_fix; /* Roe only: Harten fix width as a fraction of the sound speed */
  /* laminar Navier-Stokes (MODEL: DYNAMICS = LAMINAR); viscous = 0 for Euler */
  int32_t viscous;    /* ty_viscous: face gradient (SPAT_PARAM:DISSIPATIVE_FLUX) */
  int32_t visc_law;   /* ty_visc_law */
  double visc_kin;    /* kinematic viscosity of TY_VISC_KINEMATIC */
  double rgas;        /* gas constant (AIR: 287.14) */
  double prandtl;     /* Prandtl number (AIR: 0.72) */
  double farfield[5]; /* free stream of TY_BC_FARFIELD faces: rho, p, u, v, w */
} ty_spat_params;
/* face gradient of the viscous flux (interpface_gradient_vect.f90, interpface_gradn_scal.f90) */
enum ty_viscous { TY_VISC_NONE = 0, TY_VISC_CELLAVG = 1, TY_VISC_CELLFULL = 2 };
/* viscosity law (EQNS.f90 calc_viscosity): nu*rho, or Sutherland with AIR's constants */
enum ty_visc_law { TY_VISC_KINEMATIC = 0, TY_VISC_SUTHERLAND = 1 };

/* Version string of the library. */
const char* ty_version(void);
/* Text of a status code. */
const char* ty_error_string(int status);
/* Detail of the last error on this thread (CUDA message, failing index, ...). */
const char* ty_last_error(void);

/* Create the device-side mesh: copies the description to HBM and derives the cell->face
 * gather lists (in colour order), the least-squares factors (precalc_grad_lsq.f90:43-159)
 * and the per-face reconstruction geometry.  device: CUDA ordinal.
 * Replaces Typhon's grid set-up consumed by calc_rhs (SOURCE/MAIN/calc_rhs.f90:10). */
int ty_mesh_create(const ty_mesh_desc* desc, int device, ty_mesh** out);
int ty_mesh_destroy(ty_mesh* mesh);
/* Sizes of a device mesh: ncell_int, ncell, nface_int, nface, max faces per cell. */
int ty_mesh_info(const ty_mesh* mesh, int32_t* out5);

/* Spatial scheme (def_spat.f90:58-313 equivalents). */
int ty_set_params(ty_mesh* mesh, const ty_spat_params* params);

/* Conserved state in Typhon layout (field%etatcons): rho[ncell_int], rhoE[ncell_int],
 * rhou[3*ncell_int] (AoS).  Host pointers; the copy is synchronous. */
int ty_state_upload(ty_mesh* mesh, const double* rho, const double* rhoE, const double* rhou);
int ty_state_download(ty_mesh* mesh, double* rho, double* rhoE, double* rhou);
/* Same, SoA device pointers [5][ncell_int] (rho, rhoE, rhou, rhov, rhow) on the handle's
 * device; stream-ordered on the handle's stream. */
int ty_state_upload_device(ty_mesh* mesh, const double* cons_soa);
int ty_state_download_device(ty_mesh* mesh, double* cons_soa);
/* Primitive variables of the current state [5][ncell_int] (rho, p, u, v, w), host. */
int ty_prim_download(ty_mesh* mesh, double* prim_soa);
/* Typhon's ghost rows in explicit runs (replaces the ghost rows of flux_to_res.f90:90-113 and
 * update_field.f90:38, where every cell's row, ghosts included, is updated): the residual row
 * of a ghost cell is the raw flux F S of its face, not scaled by dt/V, and the Runge-Kutta
 * combination adds it to the ghost's conservative state.  In a first-order run Typhon's ghost
 * primitive variables come from that state, and its boundary monitors (integ_ustboco.f90,
 * the histovar files) report them.  ty_ghost_state_set starts the bookkeeping from the ghost
 * conservative states cons_ghost [5][nghost] (host; ghosts in the mesh's ghost order, cell
 * ncell_int + k for ghost k); NULL stops it.  Explicit steps (ty_rk_step, ty_rk_steps,
 * ty_steady_iteration) then keep it; it changes no interior value.  ty_ghost_prim_download
 * gives the primitive variables [5][nghost] (host) of the ghost states the last stage's
 * residual was evaluated with. */
int ty_ghost_state_set(ty_mesh* mesh, const double* cons_ghost);
int ty_ghost_prim_download(ty_mesh* mesh, double* prim_ghost);

/* Global stability time step (calc_ns_timestep.f90:52-103 + min of
 * calc_zonetimestep.f90:95): dt = min_c 2 CFL V_c / sum_f S_f / (|u|+a). */
int ty_timestep(ty_mesh* mesh, double cfl, double* dt_out);

/* One zone residual with a uniform time step dt (calc_rhs explicit part:
 * calc_varprim, boundary states, gradients, high-order face states, fluxes and
 * flux_to_res): R = dt/V * sum(+-F S).  Replaces integration_grid
 * (SOURCE/MAIN/integration_grid.f90:8-121).  R_out: host [5][ncell_int] SoA or NULL. */
int ty_residual(ty_mesh* mesh, double dt, double* R_out);

/* One explicit Runge-Kutta step of size dt (treelevel_rungekutta.f90:8-113 followed by
 * update_field.f90:38), state updated in place on the device. */
int ty_rk_step(ty_mesh* mesh, int32_t rk_method, double dt);

/* nsteps explicit steps, each with the global stability time step at CFL cfl, computed on
 * the device (no host synchronisation between steps).  dt_last: the last step's dt (host)
 * or NULL. */
int ty_rk_steps(ty_mesh* mesh, int32_t rk_method, double cfl, int32_t nsteps, double* dt_last);

/* One iteration of Typhon's steady explicit run (integration_cyclezone.f90:80-170 with
 * TIME = STEADY): the stability time step at CFL cfl (calc_zonetimestep.f90:54-126; global
 * minimum, or per cell when local_dt is non-zero: DTCALC = LOCAL_STABILITY_CONDITION), one
 * step of rk_method, and update_field.f90:45-60's residual terms of the step's update
 * res_l1[3] = (sum |d rho|, sum |d rho E|, sum |d rho u|) over the interior cells (host).
 * dt_out: the (minimum) time step (host) or NULL.  The caller divides by the reference state
 * and runs the cycle logic (the Python side's Grid.ns_steady). */
int ty_steady_iteration(ty_mesh* mesh, int32_t rk_method, double cfl, int32_t local_dt, double* dt_out,
                        double* res_l1);

/* Debug/parity access to intermediate fields of the last residual evaluation (host):
 * which = 0 prim [5][ncell], 1 grad [15][ncell], 2 face flux*S [5][nface],
 *         3 limiter ratios [3][ncell] (Barth post-limiter). */
int ty_debug_get(ty_mesh* mesh, int32_t which, double* out);
/* The fast mode's reciprocal, reciprocal square root and square root (Newton-Raphson
 * iterations from the hardware seeds) on n host values x, results in host y, on the current
 * device; which = 0 1/x, 1 1/sqrt(x), 2 sqrt(x) (fast mode); 3, 4, 5 the same by CUDA's IEEE
 * division and square root; 6, 7 the seeds alone (rcp.approx / rsqrt.approx).  For measuring
 * the fast mode's rounding; no counterpart in the reference. */
int ty_debug_fastmath(int32_t which, int32_t n, const double* x, double* y);

/* Inlet / outlet parameters per face: host [nface][6] (see ty_bc; rows of other faces are
 * ignored).  Required before a Navier-Stokes operation on a mesh with inlets or outlets. */
int ty_set_bc_data(ty_mesh* mesh, const double* data);
/* Rotational periodicity: the rotation of each face [nface][9] (ty_umesh_face_rotation).  Ghost
 * states of rotational periodic faces take the partner cell's state with the velocity rotated
 * (R u), their gradients R g for the scalars and G R^T for the velocity (Typhon's transten_per
 * multiplies on the right only), and the right face states take the partner face's left
 * state with the velocity rotated (calcboco_connect_per_match.f90:56-78).  The implicit step
 * follows; the adjoint and heat conduction refuse such a mesh. */
int ty_mesh_set_face_rotation(ty_mesh* mesh, const double* rot);

/* Wait for the handle's stream. */
int ty_synchronize(ty_mesh* mesh);

/* Run the handle's work on the caller's CUDA stream (a cudaStream_t of the handle's
 * device, e.g. a PyTorch stream), or on the handle's own stream again when stream is NULL.
 * The legacy default stream is named by cudaStreamLegacy ((void*)1), since NULL means the
 * handle's own stream.  Waits for work already queued on the previous stream. */
int ty_set_stream(ty_mesh* mesh, void* stream);

/* Per-kernel CUDA-event timing of every launch issued while enabled (enabling clears the
 * record).  ty_profile_read returns, per kernel id (0 prim, 1 ghost_prim, 2 grad,
 * 3 ghost_grad, 4 face_states, 5 barth, 6 face_flux, 7 face_flux_lim, 8 rk_update,
 * 9 gather, 10 timestep, 11 cell_fast, 12 face_flux_fast, 13 imp_face, 14 imp_diag,
 * 15 imp_matvec, 16 imp_precond, 17 imp_ortho), the summed milliseconds and the number of
 * launches. */
int ty_profile_enable(ty_mesh* mesh, int32_t on);
int ty_profile_read(ty_mesh* mesh, int32_t n, double* ms, int32_t* launches);

/* ---------------------------------------------------------------------------------
 * Implicit (backward Euler) step.  Replaces calc_rhs.f90:121-138 with calc_jacobian set
 * (integration_grid + build_implicit + tstep_implicit/implicit_solve) and update_field.f90:38.
 */
typedef enum {
  TY_KRYLOV_GMRES = 0,   /* Typhon's bdlu_gmres (bdlu_gmres.f90:50-217): MGS, no preconditioner */
  TY_KRYLOV_FGMRES = 1,  /* flexible GMRES(m), right block-Jacobi, assembled matrix (new); the
                            basis' Gram matrix is measured, one host synchronisation per vector */
  TY_KRYLOV_JFNK = 2,    /* the same flexible GMRES(m) on Jacobian-free products (new) */
  TY_KRYLOV_BICGSTAB = 3 /* Typhon's bdlu_bicgstab (bdlu_bicgstab.f90:40-80), its default for the
                            Navier-Stokes implicit method: x0 = b / diag, stopped when
                            sum|alpha p + omega s| < INV_RES sum|x0| or after max_it + 1
                            iterations; nkrylov is not used */
} ty_krylov;
typedef enum {
  TY_PREC_FP64 = 0,      /* everything in FP64 */
  TY_PREC_MIXED = 1,     /* TY_KRYLOV_FGMRES only: FP32 blocks, mat-vec, preconditioner and
                            Krylov basis (swept in FP32, FP64 block sums); FP64 residual of the
                            step and of each restart, Hessenberg algebra and update */
  TY_PREC_MIXED_FP64ORTHO = 2  /* TY_KRYLOV_FGMRES only: FP32 blocks, FP32 Jacobian-vector
                            products and FP32 block-Jacobi preconditioner (FP32 preconditioned
                            vectors); the Krylov basis, its orthogonalisation (two sweeps,
                            measured Gram matrix), the residuals, the Hessenberg algebra and the
                            update in FP64 */
} ty_precision;
typedef enum ty_imp_scaling {
  TY_IMP_SCALE_STATE = 0,  /* equation v divided by the state's RMS magnitude s_v (rho, rhoE,
                              and sqrt(s_rho s_rhoE) for momentum): the Krylov solve minimises
                              the residual in units of the state, not the energy equation's
                              alone (default) */
  TY_IMP_SCALE_NONE = 1    /* the assembled rows as they are */
} ty_imp_scaling;
typedef struct ty_imp_params {
  int32_t krylov;        /* ty_krylov (INVERSION = GMRES is TY_KRYLOV_GMRES) */
  int32_t precision;     /* ty_precision */
  int32_t nkrylov;       /* NKRYLOV: Krylov vectors per cycle (GMRES <= 64, others <= 32) */
  int32_t max_it;        /* IMP_MAX_IT: GMRES stops after 2*max_it+1 cycles (Typhon), the
                            others after max_it cycles */
  int32_t local_dt;      /* DTCALC: 1 = LOCAL_STABILITY_CONDITION, 0 = STABILITY_CONDITION */
  int32_t scaling;       /* ty_imp_scaling of the FGMRES/JFNK system (GMRES: ignored) */
  double inv_res;        /* INV_RES: GMRES uses Typhon's test |r|/|b| < INV_RES |x0|_1; the
                            others |S r|/|S b| <= INV_RES, S their row scale */
  double cfl;            /* stability number of this step (the caller ramps it) */
} ty_imp_params;
typedef struct ty_imp_stats {
  int32_t info;          /* GMRES: cycles - 1 when converged, -1 otherwise (bdlu_gmres info) */
  int32_t restarts;      /* Krylov cycles run */
  int32_t matvecs;       /* operator applications */
  int32_t reserved;
  double dt_min;         /* smallest cell time step of the step */
  double res_l2[5];      /* L2 norm over cells of -sum(F S)/V per variable, before the update */
  double du_l1[5];       /* L1 norm of the update per variable (update_field.f90:54-60) */
  double lin_res;        /* final relative linear residual |S (b - A x)| / |S b| (S = I unless
                            the FGMRES/JFNK system is scaled) */
  double du_mom;         /* sum over cells of the Euclidean norm of the momentum update (the
                            vector part of Typhon's steady residual, update_field.f90:54-60) */
} ty_imp_stats;
/* One implicit step on the resident state: time step (per cell or global at p->cfl),
 * residual with flux Jacobians (HLL for HLLC and Roe, Rusanov's for Rusanov, viscous
 * diagonal, symmetry mirror), BDLU assembly, linear solve, U += dU. */
int ty_implicit_step(ty_mesh* mesh, const ty_imp_params* p, ty_imp_stats* stats);
/* Parity access after ty_implicit_step (host, row-major 5x5 blocks):
 * which = 0 jacL [nface][25], 1 jacR [nface][25] (times S), 2 diagonal blocks [ncell_int][25],
 *         3 upper [nface_int][25], 4 lower [nface_int][25], 5 dtloc [ncell_int],
 *         6 right-hand side [ncell_int][5], 7 solution dU [ncell_int][5]. */
int ty_implicit_get(ty_mesh* mesh, int32_t which, double* out);
/* y = A x with the FP64 BDLU matrix of the last implicit step; x, y host [ncell_int][5]
 * (Typhon's bdlu_yeqax, SPMAT_BDLU.f90:139-157). */
int ty_implicit_matvec(ty_mesh* mesh, const double* x, double* y);

/* ---------------------------------------------------------------------------------
 * Heat conduction (KDIF: SOLVER = HEAT).  The temperature T lives per cell of the handle's
 * mesh; U = Cp T.  Replaces integration_kdif_ust (SOURCE/EQKDIF/integration_kdif_ust.f90) and
 * the implicit step of the HEAT solver (calc_rhs.f90:121-138 with its DLU matrix).
 */
enum ty_kdif_flux {     /* SPAT_PARAM:DISSIPATIVE_FLUX of calc_kdif_flux.f90:106-137 */
  TY_KDIF_COMPACT = 0,  /* two-point: -k (T_R - T_L) (d.n) / |d|^2 */
  TY_KDIF_CELLAVG = 1,  /* -k (a grad T_R + b grad T_L).n */
  TY_KDIF_FULL = 2      /* compact along d plus the averaged gradient across it */
};
enum ty_kdif_bc {       /* boundary kind of each boundary face (periodic faces: from the mesh) */
  TY_KBC_ISOTHERMAL = 1,  /* ISOTHERMAL_WALL: ghost temperature = face value (setboco_kdif_isoth.f90) */
  TY_KBC_FLUX = 2,        /* imposed flux entering the domain = face value; 0 is adiabatic */
  TY_KBC_EXTRAPOLATE = 3  /* ghost temperature = inside temperature */
};
typedef struct ty_kdif_params {
  int32_t flux;          /* ty_kdif_flux */
  int32_t reserved;
  double heat_capacity;  /* MODEL: HEATCAPA (rho Cp per unit volume) */
} ty_kdif_params;
/* conductivity [ncell_int] (new: per cell; the face value is the distance-weighted harmonic
 * mean, or the common value when both cells agree, which is Typhon's uniform CONDUCT);
 * face_kind [nface] ty_kdif_bc of boundary faces (ignored for interior and periodic faces);
 * face_value [nface] wall temperature or imposed flux. */
int ty_kdif_setup(ty_mesh* mesh, const ty_kdif_params* p, const double* conductivity, const int32_t* face_kind,
                  const double* face_value);
int ty_kdif_set_temperature(ty_mesh* mesh, const double* T);   /* host [ncell_int] */
int ty_kdif_get_temperature(ty_mesh* mesh, double* T);         /* host [ncell_int] */
/* residual dt/V sum(+-F S) of U = Cp T (host [ncell_int], may be NULL) */
int ty_kdif_residual(ty_mesh* mesh, double dt, double* R);
typedef enum {
  TY_KSOLVE_CG = 0,          /* conjugate gradients + Jacobi, FP64 (new: Typhon has CGS/BiCG/GMRES):
                                Chronopoulos-Gear single-reduction form, two launches per
                                iteration, no host round trip between checks */
  TY_KSOLVE_CG32_REFINE = 1, /* FP32 conjugate gradients inside FP64 iterative refinement */
  TY_KSOLVE_CG_MIXED = 2     /* TY_KSOLVE_CG on the face conductances stored in FP32 (FP64
                                vectors and arithmetic; the difference form keeps the matrix
                                spectrally within 1e-7 of the FP64 one) until the relative
                                residual is below 1e-6, then restarted on the FP64 matrix from
                                the FP64 system's residual (stats.refinements = 1 when it
                                switched) */
} ty_kdif_solver;
typedef struct ty_kdif_solve {
  int32_t solver;        /* ty_kdif_solver */
  int32_t max_it;        /* iterations (CG) or inner iterations per refinement (CG32) */
  double tol;            /* relative residual of the symmetrised system */
  double inner_tol;      /* CG32: relative residual of each inner FP32 solve */
} ty_kdif_solve;
typedef struct ty_kdif_stats {
  int32_t iterations;    /* CG iterations (all inner iterations for CG32) */
  int32_t refinements;   /* outer FP64 refinements (CG32) */
  double rel_res;        /* final |b - S x| / |b| */
  double du_l1;          /* sum over cells of |dU| (U = Cp T), Typhon's steady residual
                            (update_field.f90:45-52) before its division by the reference */
} ty_kdif_stats;
/* One backward-Euler step of size dt: residual, symmetrised matrix diag(V/dt) A, solve,
 * T += dU / Cp. */
int ty_kdif_implicit_step(ty_mesh* mesh, double dt, const ty_kdif_solve* s, ty_kdif_stats* stats);
/* Typhon's stability time step of the heat equation (calc_kdif_timestep.f90:38-62 with the
 * global minimum of calc_zonetimestep.f90): min over cells of 2 fourier V^2 / sum_f S^2 times
 * Cp / k, k the cell's conductivity (Typhon's linear material: one k). */
int ty_kdif_fourier_dt(ty_mesh* mesh, double fourier, double* dt);
/* Parity access (host): which = 0 T [ncell] (ghosts included), 1 grad T [3][ncell_int],
 * 2 flux*S [nface], 3 J_R*S [nface], 4 diagonal [ncell_int], 5 flux balance [ncell_int]. */
int ty_kdif_get(ty_mesh* mesh, int32_t which, double* out);
/* y = S x with the last assembled symmetrised matrix, host [ncell_int]. */
int ty_kdif_matvec(ty_mesh* mesh, const double* x, double* y);

/* ---------------------------------------------------------------------------------
 * Adjoint (new: Typhon has no adjoint).  Both calls act on the resident state set by
 * ty_state_upload_device and work on caller DEVICE buffers [5][ncell_int] (rho, rhoE, rhou,
 * rhov, rhow), queued on the handle's stream.
 *   ty_residual_device: R = dt/V sum(+-F S), ty_residual's value.
 *   ty_adjoint_vjp:     lambda_U = (dR/dU)^T lambda_R of the inviscid residual, first order
 *                       (HIGHRES = NONE, any boundary) or second order (least-squares
 *                       gradients, HIGHRES = MUSCL or MUSCL-UNS with no limiter or van
 *                       Albada, POST-LIMITER = BARTH / SUPERBARTH frozen: its ratios are
 *                       those of the state and are not differentiated; periodic
 *                       boundaries); TY_ERR_UNSUPPORTED otherwise.  A reversed face loop
 *                       (hand-written reverse-mode flux derivatives, reversed
 *                       reconstruction) and per-cell gathers, no atomics. */
int ty_residual_device(ty_mesh* mesh, double dt, double* R);
int ty_adjoint_vjp(ty_mesh* mesh, double dt, const double* lambda_R, double* lambda_U);

/* Global stability time step for callers that cannot let the library allocate device
 * memory (a host code that owns all device memory through its own allocator, a solver loop
 * that must not allocate between steps).  No counterpart in the reference: it computes the
 * same value as ty_timestep in TY_MODE_EXACT, without a ty_mesh handle.
 *   cons        device [5][ld] conserved state (rho, rhoE, rhou, rhov, rhow), ld >= ncell
 *   volume      device [ncell] cell volumes
 *   sum_surface device [ncell] sum of the face surfaces of each cell
 *   stream      cudaStream_t of the current device (NULL: the default stream)
 *   dt_out      host: the minimum over cells of CFL*2*V/sum S/(|u|+a)
 * Allocates nothing: its scratch (a partial minimum per 256 cells, the result and an error
 * word) lives in a static device array of the library, at most 4,194,304 cells per call
 * (larger ncell returns TY_ERR_ARG).  Every call looks up the array's address in the CUDA
 * context current on the calling thread.  The first call in a context loads the library's
 * module (CUDA loads modules lazily) and that load allocates device memory for the code and
 * the array: make one call at set-up, before any stream capture and before the phase that
 * must not allocate.  Calls share the array: calls that overlap on the GPU race.
 * Synchronises the stream; returns TY_ERR_NEGENERGY / TY_ERR_NANDT like ty_timestep. */
int ty_timestep_static(int32_t ncell, const double* cons, int32_t ld, const double* volume,
                       const double* sum_surface, double gamma, double cfl, void* stream, double* dt_out);

/* ---------------------------------------------------------------------------------
 * Host mesh preprocessing (no GPU): builds the ty_mesh_desc arrays from an element mesh
 * the way Typhon's grid_preproc and init_connect_grid do (face creation and order,
 * geometry, colouring, ghost cells, periodic matching).  Counterpart of
 * create_face_connect (CFDTOOLS/Mesh/MESHCONNECT.f90:34), calc_meshgeom
 * (CFDTOOLS/Mesh/MESHGEOM.f90:421) and coo_colorgroup (CFDTOOLS/Base/COLOR.f90:33). */
typedef struct ty_umesh ty_umesh;
int ty_umesh_new(ty_umesh** out);
int ty_umesh_free(ty_umesh* um);
/* nodes: [3*nvtex]; element sections (cells of the highest dimension and boundary face
 * elements) with their element numbers and 1-based vertex lists, as in a .tym file. */
int ty_umesh_set_nodes(ty_umesh* um, int32_t nvtex, const double* xyz);
int ty_umesh_add_section(ty_umesh* um, int32_t elemtype, int32_t nelem, const int32_t* ielem,
                         const int32_t* vtex);
/* A boundary family given by face element numbers (a .tym mark, a CGNS FaceCenter or
 * ElementList BC), or by vertex numbers: every boundary face whose vertices are all in the
 * list (a CGNS Vertex BC; CFDTOOLS/Mesh/seek_bcface_vtex.f90:38-45). */
int ty_umesh_add_mark(ty_umesh* um, const char* family, int32_t ntag, const int32_t* tags);
int ty_umesh_add_vertex_mark(ty_umesh* um, const char* family, int32_t ntag, const int32_t* tags);
/* Boundary definitions, then preprocessing.  kind: ty_bc; periodic families give their
 * partner family and the translation from this family to the partner. */
int ty_umesh_add_bc(ty_umesh* um, const char* family, int32_t kind, const char* partner,
                    const double* translation3, const double* wallvel3);
/* Makes the periodic definition of `family` (added by ty_umesh_add_bc) a rotation: BLOCK:
 * PERIODICITY TYPE = ROTATION with ROTATION_CENTER, ROTATION_AXIS (normalised here) and
 * ROTATION_ANGLE in degrees (def_mesh.f90:230-247), from this family to its partner.  The
 * faces are matched after rotating their centres (transloc_per, MESHPARAMS.f90:125-146) and
 * each ghost centre is the face centre plus the partner's face-to-cell vector rotated back
 * (init_connect_grid.f90:210-225). */
int ty_umesh_set_rotation(ty_umesh* um, const char* family, const double* centre3, const double* axis3,
                          double angle_deg);
/* The rotation of each face [nface*9], row-major: the one that brings vectors of the
 * partner's frame into the face's frame on faces of rotational periodic families (calc_rot of
 * transvec_per, VEC3D.f90:652-674), the identity elsewhere.  Returns 1 when a family is
 * rotational, 0 otherwise (then pass nothing to ty_mesh_set_face_rotation). */
int ty_umesh_face_rotation(const ty_umesh* um, double* out);
int ty_umesh_build(ty_umesh* um, int32_t dim);
/* Pointers into the built description (valid until ty_umesh_free). */
int ty_umesh_desc(const ty_umesh* um, ty_mesh_desc* out);
/* Face -> vertex lists of the built mesh: [nface*4] 1-based, 0 padded. */
int ty_umesh_facevtex(const ty_umesh* um, int32_t* out);
/* Reverse Cuthill-McKee order of the cells of each cell section (new: a numbering for
 * locality; Typhon keeps the file's order): out [ncell_int], for every cell
 * section in ty_umesh_add_section order, the 0-based positions of its elements in their new
 * order, computed on the cells the section's interior faces connect.  Rebuilding the mesh
 * with each section's element rows taken in this order (element numbers kept in place)
 * numbers neighbouring cells, and so the faces created from them, close together. */
int ty_umesh_rcm_order(const ty_umesh* um, int32_t* out);
/* Boundary definition of each face [nface]: the index (0-based, in ty_umesh_add_bc order)
 * of the definition its family matched, -1 for interior faces.  Lets a caller give per-face
 * values (KDIF wall kinds and temperatures, ...) by family. */
int ty_umesh_face_family(const ty_umesh* um, int32_t* out);

#ifdef __cplusplus
}
#endif
#endif /* TYPHON_GPU_H */
