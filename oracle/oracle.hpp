// Typhon CPU oracle — TEST INFRASTRUCTURE ONLY.
//
// A literal C++ restatement of the Fortran routines of Typhon (Haider-BA/typhon)
// on the unstructured finite-volume residual-and-update path.  It exists to
// check the GPU library: only tests/, __graft_entry__.smoke() and the CPU leg
// of bench.py may build, load or run it, and never as the thing measured or
// shipped.  Every function cites the Fortran file:line it restates; the loop
// and summation orders follow the Fortran so that results can be compared
// bit for bit where the GPU path runs in its exact mode.
//
// Parity pin: the oracle reproduces the golden monitor files of Typhon's own
// non-regression suite (NRG/TIME/RUNGEKUTTA/*/RHOERR.tmon,
// NRG/MESH/CON/PER2D-TRANS/RHODEV.tmon) to their printed precision; see
// tests/test_oracle_golden.py.
//
// Indices are 0-based here.  Ghost cells are numbered after the interior
// cells, in the order Typhon assigns them (init_connect_grid.f90).
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace ory {

struct V3 {
  double x = 0, y = 0, z = 0;
};
inline V3 v3(double a, double b, double c) { V3 v; v.x = a; v.y = b; v.z = c; return v; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
// v3d_scalar_product (CFDTOOLS/Math/VEC3D.f90:555-561)
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// v3d_sqrnorme (VEC3D.f90:529-535)
inline double sqrabs(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// v3d_norme (VEC3D.f90:503-509)
inline double vabs(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// v3d_vectorial_product (VEC3D.f90:583-591)
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Element type codes of CFDTOOLS/Mesh/ELEMVTEX.f90:17-37.
enum ElemType {
  ELEM_BAR2 = 2, ELEM_TRI3 = 13, ELEM_QUAD4 = 24, ELEM_TETRA4 = 101,
  ELEM_PYRA5 = 121, ELEM_PENTA6 = 131, ELEM_HEXA8 = 141
};
int elem_dim(int type);
int elem_nvtex(int type);

struct ElemSection {
  int type = 0;
  std::vector<int> ielem;  // element numbers (1-based, as stored in the file)
  std::vector<int> vtex;   // nelem * nv vertex numbers (1-based)
  int nv() const { return elem_nvtex(type); }
  int nelem() const { return (int)ielem.size(); }
};

struct Mark {
  std::string family;
  std::vector<int> tags;  // element numbers of boundary face elements, or vertex numbers
  bool vertex = false;    // tags are vertices (a CGNS Vertex BC)
};

// Content of a Typhon .tym mesh (TYFMT_MESH.f90 reader) or of a generator.
struct RawMesh {
  std::vector<V3> vtex;
  std::vector<ElemSection> sections;  // cell and face element sections in file order
  std::vector<Mark> marks;
};

bool read_tym(const std::string& path, RawMesh& out, std::string& err);

// Boundary families and how the solver treats them.
// BC_NOSLIP (new): BC_WALL with the inside density in the face state (BC_WALL keeps Typhon's
// face state, whose density is the inside pressure, setboco_ns_flux.f90:136)
// BC_HEAT: a KDIF boundary with a ghost face (init_ustboco_ghostface.f90), as Typhon
// implements every KDIF wall and EXTRAPOLATE
// Inlets and outlets (setboco_ns_inlet_sub.f90, setboco_ns_outlet_sub.f90,
// setboco_ns_inlet_sup.f90, setboco_ns_outlet_sup.f90), ghost faces as in Typhon
// (bctype_of_nsboco, MENU_NS.f90:91-115).  Parameters (BcDef::data):
//   BC_INLET_SUB  total pressure, total temperature, direction (3)
//   BC_OUTLET_SUB static pressure
//   BC_INLET_SUP  total pressure, total temperature, Mach number, direction (3)
enum BcKind { BC_PERIODIC = 1, BC_SYMMETRY = 2, BC_WALL = 3, BC_FARFIELD = 4, BC_NOSLIP = 5, BC_HEAT = 6,
              BC_INLET_SUB = 7, BC_OUTLET_SUB = 8, BC_INLET_SUP = 9, BC_OUTLET_SUP = 10 };
inline bool ghost_face_kind(int k) { return k == BC_HEAT || (k >= BC_INLET_SUB && k <= BC_OUTLET_SUP); }
struct BcDef {
  std::string family;   // family name as in the mesh marks
  int kind = 0;
  // periodic: partner family and the translation from this family to the partner
  std::string partner;
  V3 translation;
  // wall: wall velocity
  V3 wall_velocity;
  double data[6] = {0, 0, 0, 0, 0, 0};  // inlet / outlet parameters (BcKind)
  // periodic by rotation (BLOCK:PERIODICITY TYPE = ROTATION, MESHPARAMS.f90:125-205): centre,
  // unit axis, angle in radians from this family to the partner (translation then unused)
  bool rotation = false;
  V3 rot_centre, rot_axis;
  double rot_angle = 0.0;
};

// calc_rot (CFDTOOLS/Math/VEC3D.f90:652-674): row-major rotation about the unit axis
void calc_rot(V3 axis, double angle, double* M);
// M v, summed in column order
V3 rot_apply(const double* M, V3 v);

struct Boco {
  std::string family;
  std::vector<int> iface;  // mesh faces of the family (0-based), in mark order
  int kind = 0;
  int def = -1;            // index into the BcDef list
  double rlink = 0;        // +1 for FAMILY1 side, -1 for FAMILY2 side
  std::vector<int> partner_face;  // periodic: partner face of each face
  V3 wall_velocity;
  double data[6] = {0, 0, 0, 0, 0, 0};
  // periodic by rotation: the rotation bringing the partner's vectors into this family's
  // frame (calc_rot of the angle -rlink * angle, transvec_per), row-major
  bool rotation = false;
  double rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
};

// Preprocessed mesh in Typhon's numbering (st_ustmesh).
struct UMesh {
  int dim = 2;        // geometric dimension (2: COORD=2D, 3: 3D)
  int ncell_int = 0, ncell = 0, nface_int = 0, nface = 0, nface_lim = 0;
  std::vector<int> fc1, fc2;        // face -> cells (fc2 is a ghost index for boundary faces)
  std::vector<std::vector<int>> facevtex;
  std::vector<V3> fnormal, fcentre;
  std::vector<double> fsurf;
  std::vector<V3> ccentre;          // ncell (ghosts included once connections are set)
  std::vector<double> cvol;
  std::vector<std::vector<int>> colors;  // coo_colorgroup: faces of each colour, ascending
  std::vector<Boco> bocos;
};

// create_face_connect + calc_ustmesh + grid_postproc + init_connect_grid.
bool build_umesh(const RawMesh& raw, int geo_dim, const std::vector<BcDef>& bcs, UMesh& m,
                 std::string& err);

// ---------------------------------------------------------------------------
// Solver
// HLLC and HLLE with Typhon's wave-speed variants (def_spat.f90:68-76): B = the beta of
// calc_flux_hllc.f90:70-72 / calc_flux_hlle.f90:68-70, K = the kinetic (EFM) estimates
enum Scheme { SCH_HLLC = 1, SCH_RUSANOV = 2, SCH_ROE = 3, SCH_AUSMM = 4, SCH_HLLE = 5, SCH_HLLCB = 6, SCH_HLLCK = 7,
              SCH_HLLCKB = 8, SCH_HLLEB = 9, SCH_HLLEK = 10, SCH_HLLEKB = 11 };
inline bool is_hllc(int s) { return s == SCH_HLLC || (s >= SCH_HLLCB && s <= SCH_HLLCKB); }
inline bool is_hlle(int s) { return s == SCH_HLLE || (s >= SCH_HLLEB && s <= SCH_HLLEKB); }
enum HighRes { HRES_NONE = 0, HRES_MUSCL = 1, HRES_MUSCLFAST = 2, HRES_MUSCLUNS = 3 };
enum Limiter { LIM_NONE = 0, LIM_MINMOD = 1, LIM_ALBADA = 2, LIM_VLEER = 3, LIM_SBEE = 4,
               LIM_KIM3 = 5, LIM_LIM03 = 6 };
enum PostLim { POSTLIM_NONE = 0, POSTLIM_BARTH = 1, POSTLIM_SUPERBARTH = 2 };
enum GradMeth { GRAD_NONE = 0, GRAD_LSQ = 1, GRAD_LSQW = 2 };
enum RkMethod { EXPLICIT = 0, RK2 = 1, RK2SSP = 2, RK3SSP = 3, RK4 = 4, LSRK25BB = 5, LSRK26BB = 6,
                LSRK12BS = 7, LSRK13BS = 8 };

struct SpatParams {
  int scheme = SCH_HLLC;
  int highres = HRES_NONE;
  int limiter = LIM_ALBADA;
  int postlim = POSTLIM_NONE;
  int gradmeth = GRAD_NONE;
  double gamma = 1.4;
  double roe_entropy_fix = 0.1;  // Harten fix width (fraction of local sound speed), Roe only
  // laminar Navier-Stokes (DYNAMICS = LAMINAR)
  int viscous = 0;        // 0 Euler, 1 DISSIPATIVE_FLUX = CELL-AVERAGE, 2 = FULL
  int visc_law = 0;       // 0 KINEMATIC-CONSTANT (mu = nu rho), 1 Sutherland (AIR)
  double visc_kin = 0.0;  // nu for KINEMATIC-CONSTANT
  double rgas = 287.14;   // AIR
  double prandtl = 0.72;
  // far field (new: Typhon parses FAR-FIELD but has no Navier-Stokes implementation):
  // free-stream primitive state rho, p, u, v, w
  double farfield[5] = {1.0, 1.0 / 1.4, 0.0, 0.0, 0.0};
};

// Far-field ghost state (new).  The kind of each far-field face is fixed by the free-stream
// normal velocity vn = u_inf . n (n outward) against the free-stream sound speed c:
//   vn <= -c  supersonic inflow:  the free stream
//   vn < -1e-8 c  subsonic inflow: free-stream density and velocity, pressure from inside
//   vn <  c   subsonic outflow:   inside density and velocity, free-stream pressure (a face
//             tangent to the free stream counts as outflow, whatever the rounding of n)
//   else      supersonic outflow: the inside state
// q: inside primitive state (rho, p, u, v, w); out: ghost primitive state.
void farfield_state(double gamma, const double* qinf, V3 n, const double* q, double* out);
// inlet / outlet state (BcKind 7..10) from the inside primitive state
void inout_state(int kind, double g, double r, const double* data, const double* qi, double* qo);
bool farfield_jacobian(double gamma, const double* qinf, V3 n, const double* q, double* M);
void noslip_jacobian(V3 uw, double* M);
enum ViscMeth { VISC_NONE = 0, VISC_CELLAVG = 1, VISC_CELLFULL = 2 };

struct RkTable {
  int nstage = 0;
  std::vector<double> coef;  // nstage x nstage, row-major: coef[(i-1)*n + (j-1)] = coef(i,j)
  double c(int i, int j) const { return coef[(i - 1) * nstage + (j - 1)]; }
};
RkTable rk_table(int method);

// Field layout: [var][cell], var 0=rho, 1=p or rhoE, 2..4 = vector components.
struct Solver {
  const UMesh* m = nullptr;
  SpatParams sp;
  RkTable rk;
  double cfl = 1.0;
  std::vector<double> cons, prim;      // 5*ncell
  std::vector<double> grad;            // 15*ncell: grad rho (3), grad p (3), du_i/dx_j (9, row i)
  std::vector<double> cell_l, cell_r;  // 5*nface
  std::vector<double> flux;            // 5*nface
  std::vector<double> residu;          // 5*ncell
  std::vector<double> dtloc;           // ncell
  std::vector<double> gradcond;        // 9*ncell_int, Cholesky factors (column-major 3x3)
  bool gradcond_ok = false;
  std::vector<double> limratio;        // 3*ncell: Barth ratios of the last stage (rho, p, vector)
  double cur_res = 0;

  void init(const UMesh* mesh, const SpatParams& p, int rk_method, double cfl_);
  void varprim();
  void varcons();
  void boco_cell_state();
  void boco_cell_grad();
  void boco_face_state();
  void precalc_grad_lsq();
  void calc_gradient();
  void hres_states();
  void postlimit_barth(double klim);
  void face_fluxes();
  double viscosity(double rho, double T) const;
  void viscous_fluxes();
  void ns_bocoflux();
  void flux_to_res();
  void calc_rhs();               // one residual evaluation at dtloc

  // ---- implicit (backward Euler) step: HLL flux Jacobians, BDLU, GMRES ----
  // ns_bocojacobian: symmetry (Typhon) and far-field (new) fold J_R dQ_ghost/dQ_inside into J_L
  bool calc_jac = false;
  std::vector<double> jacL, jacR;         // 25*nface, row-major 5x5 per face (times S after flux_to_res)
  std::vector<double> bdiag;              // 25*ncell
  std::vector<double> bupper, blower;     // 25*nface
  int nkrylov = 50, imp_max_it = 50;
  double inv_res = 1.e-4;
  int gmres_iters = 0;
  std::vector<double> rhs_b;              // right-hand side of the last implicit solve (per cell)
  void ns_bocojacobian();
  void build_implicit_bdlu();
  void bdlu_yeqax(const double* x, double* y) const;
  void bdlu_yeqmaxpz(const double* x, const double* z, double* y) const;
  int bdlu_gmres(double* sol);                   // sol: RHS in, solution out (5*ncell, per cell)
  int bdlu_bicgstab(double* sol);                // bdlu_bicgstab.f90, same convention
  int inversion = 0;                             // 0 GMRES, 1 BICGSTAB
  // one implicit step: time step (global min or local), residual + Jacobians, solve, update;
  // returns GMRES restarts (info) and the L1 norm of the update per variable in l1[5]
  int implicit_step(double cfl_, bool local_dt, double* l1);
  double timestep();             // stab_cond: global min dt over interior cells
  void rk_step(double dt, bool local = false);  // treelevel_rungekutta + update_field
};

// ---------------------------------------------------------------------------
// Heat conduction (KDIF), oracle_kdif.cpp
enum KdifScheme { KDIF_COMPACT = 0, KDIF_CELLAVG = 1, KDIF_FULL = 2 };
// boundary kinds of KDIF faces (periodic faces come from the mesh)
enum KdifBc { KBC_NONE = 0, KBC_ISOTHERMAL = 1, KBC_FLUX = 2, KBC_EXTRAPOLATE = 3, KBC_PERIODIC = 4 };
struct KdifSolver {
  const UMesh* m = nullptr;
  int scheme = KDIF_FULL;
  double cp = 1.0;
  std::vector<double> kcell;   // ncell conductivity (ghosts: the inside cell's)
  std::vector<int> fkind;      // nface KdifBc
  std::vector<double> fval;    // nface wall temperature or imposed flux
  std::vector<double> T;       // ncell temperature
  std::vector<double> grad;    // 3*ncell
  std::vector<double> flux;    // nface flux times S
  std::vector<double> jac;     // nface J_R times S (0 on imposed-flux faces)
  std::vector<double> residu;  // ncell dt/V sum(+-F S)
  std::vector<double> balance; // ncell_int sum(+-F S)
  std::vector<double> diag;    // ncell_int diagonal of the symmetrised implicit matrix
  Solver lsq;                  // least-squares gradient machinery of the NS path
  void init(const UMesh* mesh, int flux_scheme, double heat_capacity, const double* kc, const int* kind,
            const double* value);
  void ghosts();
  void gradient();
  double face_k(int f, double dHL, double dHR) const;
  void fluxes();
  void rhs(double dt);
  void assemble(double dt);
  void matvec(const double* x, double* y) const;
  int cg(const std::vector<double>& b, std::vector<double>& x, double tol, int max_it, double* rel);
  int implicit_step(double dt, double tol, int max_it, double* rel);
  // Typhon's own implicit iteration: DLU system I + dt/V J, CGS, steady cycles
  std::vector<double> dlu_diag, dlu_upper, dlu_lower;  // ncell, nface, nface
  double fourier_dt(double fourier, double conduct) const;
  void typhon_dlu(double dt);
  void dlu_yeqax(const double* x, double* y) const;
  void dlu_yeqmaxpz(const double* x, const double* z, double* y) const;
  void dlu_yeqatx(const double* x, double* y) const;
  int dlu_cgs(std::vector<double>& sol, double maxres, int max_it) const;
  int dlu_bicg(std::vector<double>& sol, double maxres, int max_it) const;
  int dlu_gmres(std::vector<double>& sol, double maxres, int max_it, int nkrylov) const;
};

// Typhon's steady driver for one KDIF zone (integration.f90, integration_cycle.f90,
// integration_cyclezone.f90, check_end_cycle.f90), implicit DLU + CGS.
struct KdifSteadyParams {
  double fourier = 1.0, conduct = 1.0;
  double cycle_res = 0.1, global_res = 1e-5;  // TIME_PARAM and PROJECT RESIDUALS
  double cgs_maxres = 1e-4;                    // INV_RES
  int cgs_max_it = 10;                         // IMP_MAX_IT
  int inversion = 0;                           // INVERSION: 0 CGS, 1 BICG, 2 GMRES
  int nkrylov = 10;                            // NKRYLOV (GMRES)
  int max_iters = 100000, max_cycles = 1000;
};
struct KdifSteadyOut {
  std::vector<double> log_res;    // log10 of the residual of every iteration (monres)
  std::vector<double> cycle_avg;  // volume-averaged temperature after each cycle
  std::vector<int> cycle_end;     // total iterations at the end of each cycle
};
void kdif_typhon_steady(KdifSolver& k, std::vector<double>& U, const KdifSteadyParams& p, KdifSteadyOut& out);

// Typhon's steady driver for one Navier-Stokes zone with the implicit step (integration.f90,
// integration_cycle.f90, integration_cyclezone.f90, check_end_cycle.f90, calc_zonetimestep.f90
// CFL law, update_field.f90 residual) and the boundary histories of one family
// (integ_ustboco.f90, write_bocohisto.f90).
struct NsSteadyParams {
  double cfl = 1.0, cfl_max = 1.0;             // TIME_PARAM CFL, CFL_MAX
  double cycle_res = 0.1, global_res = 1e-5;   // TIME_PARAM and PROJECT RESIDUALS
  int max_iters = 100000, max_cycles = 1000;
  std::vector<int> history_faces;              // faces of the family with SAVE_HISTORY
  int rk_method = -1;                          // >= 0: explicit steps (0 = METHOD EXPLICIT), else implicit
  bool local_dt = false;                       // explicit: DTCALC = LOCAL_STABILITY_CONDITION
};
struct NsSteadyOut {
  std::vector<double> log_res;      // log10 residual of every iteration
  std::vector<double> flux_sum;     // per cycle: sum over the family of F S (5 values)
  std::vector<double> ghost_avg;    // per cycle: S-weighted average of the ghost primitive state (5)
  std::vector<int> cycle_end;
};
void ns_typhon_steady(Solver& s, const NsSteadyParams& p, NsSteadyOut& out);

}  // namespace ory
