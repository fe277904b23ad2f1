// Typhon CPU oracle — C entry points for the tests (ctypes).  TEST INFRASTRUCTURE ONLY.
//
// Also holds the drivers of Typhon's own non-regression cases whose meshes are readable
// here (.tym): the cycle loop of SOURCE/MAIN/integration.f90:59-142 and
// SOURCE/MAIN/integration_cyclezone.f90:80-170 (unsteady, global time step), and the
// volume-average probes of CFDTOOLS/Mesh/PROBECALC.f90:66-90 written by
// SOURCE/MAIN/write_monitors_cycle.f90:40-67 after calc_varprim.
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "oracle.hpp"

using namespace ory;

namespace {
struct MeshHandle {
  RawMesh raw;
  UMesh m;
  std::vector<BcDef> rotations;  // periodic families by rotation (family, centre, axis, angle)
};
void set_err(char* buf, int len, const std::string& s) {
  if (buf && len > 0) {
    std::strncpy(buf, s.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
}
std::vector<BcDef> make_bcs(int nbc, const char* const* fam, const int* kind, const char* const* partner,
                            const double* trans, const double* wallvel, const double* data = nullptr) {
  std::vector<BcDef> bcs(nbc);
  for (int i = 0; i < nbc; ++i) {
    bcs[i].family = fam[i];
    bcs[i].kind = kind[i];
    if (partner && partner[i]) bcs[i].partner = partner[i];
    if (trans) bcs[i].translation = v3(trans[3 * i], trans[3 * i + 1], trans[3 * i + 2]);
    if (wallvel) bcs[i].wall_velocity = v3(wallvel[3 * i], wallvel[3 * i + 1], wallvel[3 * i + 2]);
    if (data)
      for (int q = 0; q < 6; ++q) bcs[i].data[q] = data[6 * i + q];
  }
  return bcs;
}
}  // namespace

extern "C" {

// ---- raw meshes ----
void* ory_raw_new() { return new MeshHandle(); }
void ory_raw_free(void* h) { delete (MeshHandle*)h; }
int ory_raw_read_tym(void* h, const char* path, char* err, int errlen) {
  std::string e;
  if (!read_tym(path, ((MeshHandle*)h)->raw, e)) { set_err(err, errlen, e); return -1; }
  return 0;
}
void ory_raw_set_vtex(void* h, int n, const double* xyz) {
  auto& r = ((MeshHandle*)h)->raw;
  r.vtex.resize(n);
  for (int i = 0; i < n; ++i) r.vtex[i] = v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}
void ory_raw_add_section(void* h, int type, int nelem, const int* ielem, const int* vtex) {
  ElemSection s;
  s.type = type;
  s.ielem.assign(ielem, ielem + nelem);
  s.vtex.assign(vtex, vtex + (size_t)nelem * elem_nvtex(type));
  ((MeshHandle*)h)->raw.sections.push_back(std::move(s));
}
void ory_raw_add_mark(void* h, const char* name, int ntag, const int* tags) {
  Mark mk;
  mk.family = name;
  mk.tags.assign(tags, tags + ntag);
  ((MeshHandle*)h)->raw.marks.push_back(std::move(mk));
}
void ory_raw_add_vertex_mark(void* h, const char* name, int ntag, const int* tags) {
  ory_raw_add_mark(h, name, ntag, tags);
  ((MeshHandle*)h)->raw.marks.back().vertex = true;
}
int ory_raw_counts(void* h, int* out) {  // nvtex, nsections, nmarks
  auto& r = ((MeshHandle*)h)->raw;
  out[0] = (int)r.vtex.size();
  out[1] = (int)r.sections.size();
  out[2] = (int)r.marks.size();
  return 0;
}

// ---- preprocessing ----
// bcdata: 6 parameters per boundary definition (inlets and outlets), may be NULL
int ory_mesh_build(void* h, int geo_dim, int nbc, const char* const* fam, const int* kind,
                   const char* const* partner, const double* trans, const double* wallvel, const double* bcdata,
                   char* err, int errlen) {
  auto* mh = (MeshHandle*)h;
  std::string e;
  std::vector<BcDef> bcs = make_bcs(nbc, fam, kind, partner, trans, wallvel, bcdata);
  for (auto& b : bcs)
    for (const auto& r : mh->rotations)
      if (r.family == b.family) {
        b.rotation = true;
        b.rot_centre = r.rot_centre;
        b.rot_axis = r.rot_axis;
        b.rot_angle = r.rot_angle;
      }
  if (!build_umesh(mh->raw, geo_dim, bcs, mh->m, e)) {
    set_err(err, errlen, e);
    return -1;
  }
  return 0;
}
// A periodic family connected to its partner by a rotation (BLOCK:PERIODICITY TYPE =
// ROTATION): centre, axis (normalised here), angle in degrees (def_mesh.f90:242-247), from
// this family to the partner.  Call before ory_mesh_build.
void ory_raw_set_rotation(void* h, const char* family, const double* centre, const double* axis, double angle_deg) {
  BcDef r;
  r.family = family;
  r.rot_centre = v3(centre[0], centre[1], centre[2]);
  V3 a = v3(axis[0], axis[1], axis[2]);
  r.rot_axis = a / vabs(a);
  r.rot_angle = angle_deg / 180.0 * 3.141592653589793238462643;
  ((MeshHandle*)h)->rotations.push_back(r);
}
// Rotation of each face [nface][9], row-major: the one bringing the partner's vectors into
// this face's frame on faces of rotational periodic families, identity elsewhere.
void ory_mesh_face_rotation(void* h, double* out) {
  auto& m = ((MeshHandle*)h)->m;
  for (int f = 0; f < m.nface; ++f)
    for (int k = 0; k < 9; ++k) out[9 * f + k] = (k % 4 == 0) ? 1.0 : 0.0;
  for (auto& b : m.bocos)
    if (b.rotation)
      for (int f : b.iface)
        for (int k = 0; k < 9; ++k) out[9 * f + k] = b.rot[k];
}
// sizes: ncell_int, ncell, nface_int, nface, ncolors, dim, nboco
void ory_mesh_sizes(void* h, int* out) {
  auto& m = ((MeshHandle*)h)->m;
  out[0] = m.ncell_int; out[1] = m.ncell; out[2] = m.nface_int; out[3] = m.nface;
  out[4] = (int)m.colors.size(); out[5] = m.dim; out[6] = (int)m.bocos.size();
}
// Export Typhon's preprocessed arrays (0-based).  face_color: colour of each face;
// face_partner: periodic partner face (-1 otherwise); face_bckind: 0 interior, else BcKind.
void ory_mesh_export(void* h, int* fc1, int* fc2, double* fnormal, double* fcentre, double* fsurf,
                     double* ccentre, double* cvol, int* face_color, int* face_partner, int* face_bckind,
                     double* face_wallvel) {
  auto& m = ((MeshHandle*)h)->m;
  for (int f = 0; f < m.nface; ++f) {
    fc1[f] = m.fc1[f]; fc2[f] = m.fc2[f];
    fnormal[3 * f] = m.fnormal[f].x; fnormal[3 * f + 1] = m.fnormal[f].y; fnormal[3 * f + 2] = m.fnormal[f].z;
    fcentre[3 * f] = m.fcentre[f].x; fcentre[3 * f + 1] = m.fcentre[f].y; fcentre[3 * f + 2] = m.fcentre[f].z;
    fsurf[f] = m.fsurf[f];
    face_partner[f] = -1;
    face_bckind[f] = 0;
    face_wallvel[3 * f] = face_wallvel[3 * f + 1] = face_wallvel[3 * f + 2] = 0.0;
  }
  for (int c = 0; c < m.ncell; ++c) {
    ccentre[3 * c] = m.ccentre[c].x; ccentre[3 * c + 1] = m.ccentre[c].y; ccentre[3 * c + 2] = m.ccentre[c].z;
    cvol[c] = m.cvol[c];
  }
  for (size_t ic = 0; ic < m.colors.size(); ++ic)
    for (int f : m.colors[ic]) face_color[f] = (int)ic;
  for (auto& b : m.bocos)
    for (size_t k = 0; k < b.iface.size(); ++k) {
      int f = b.iface[k];
      face_bckind[f] = b.kind;
      if (b.kind == BC_PERIODIC) face_partner[f] = b.partner_face[k];
      face_wallvel[3 * f] = b.wall_velocity.x;
      face_wallvel[3 * f + 1] = b.wall_velocity.y;
      face_wallvel[3 * f + 2] = b.wall_velocity.z;
    }
}
void ory_mesh_facevtex(void* h, int maxv, int* out) {  // nface x maxv, 1-based vertices, 0 pad
  auto& m = ((MeshHandle*)h)->m;
  for (int f = 0; f < m.nface; ++f)
    for (int k = 0; k < maxv; ++k) out[f * maxv + k] = k < (int)m.facevtex[f].size() ? m.facevtex[f][k] : 0;
}

// ---- solver ----
// iparams: scheme, highres, limiter, postlim, gradmeth, rk_method, viscous, visc_law
// dparams: gamma, cfl, roe_entropy_fix, visc_kin, rgas, prandtl, far-field rho, p, u, v, w
void* ory_solver_new(void* mesh, const int* ip, const double* dp) {
  auto* s = new Solver();
  SpatParams sp;
  sp.scheme = ip[0]; sp.highres = ip[1]; sp.limiter = ip[2]; sp.postlim = ip[3]; sp.gradmeth = ip[4];
  sp.viscous = ip[6]; sp.visc_law = ip[7];
  sp.gamma = dp[0];
  sp.roe_entropy_fix = dp[2];
  sp.visc_kin = dp[3]; sp.rgas = dp[4]; sp.prandtl = dp[5];
  for (int v = 0; v < 5; ++v) sp.farfield[v] = dp[6 + v];
  s->init(&((MeshHandle*)mesh)->m, sp, ip[5], dp[1]);
  return s;
}
void ory_solver_free(void* s) { delete (Solver*)s; }
void ory_solver_set_cons(void* s, const double* c) {
  auto* S = (Solver*)s;
  std::memcpy(S->cons.data(), c, S->cons.size() * sizeof(double));
}
void ory_solver_set_prim(void* s, const double* p) {
  auto* S = (Solver*)s;
  std::memcpy(S->prim.data(), p, S->prim.size() * sizeof(double));
  S->varcons();
}
// which: 0 cons, 1 prim, 2 grad, 3 residu, 4 flux, 5 cell_l, 6 cell_r, 7 dtloc, 8 limratio,
//        9 jacL, 10 jacR (25 per face, row-major), 11 BDLU diag (25 per cell), 12 upper, 13 lower,
//        14 right-hand side of the last implicit solve (5 per cell)
int ory_solver_get(void* s, int which, double* out) {
  auto* S = (Solver*)s;
  const std::vector<double>* v = nullptr;
  switch (which) {
    case 0: v = &S->cons; break;
    case 1: v = &S->prim; break;
    case 2: v = &S->grad; break;
    case 3: v = &S->residu; break;
    case 4: v = &S->flux; break;
    case 5: v = &S->cell_l; break;
    case 6: v = &S->cell_r; break;
    case 7: v = &S->dtloc; break;
    case 8: v = &S->limratio; break;
    case 9: v = &S->jacL; break;
    case 10: v = &S->jacR; break;
    case 11: v = &S->bdiag; break;
    case 12: v = &S->bupper; break;
    case 13: v = &S->blower; break;
    case 14: v = &S->rhs_b; break;
    default: return -1;
  }
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return (int)v->size();
}
double ory_solver_timestep(void* s) { return ((Solver*)s)->timestep(); }
// one residual evaluation with a uniform dtloc = dt (calc_rhs)
void ory_solver_rhs(void* s, double dt) {
  auto* S = (Solver*)s;
  std::fill(S->dtloc.begin(), S->dtloc.end(), dt);
  S->calc_rhs();
}
void ory_solver_rk_step(void* s, double dt) { ((Solver*)s)->rk_step(dt); }
// n explicit steps with the global stability time step; dts receives each dt (may be null)
int ory_solver_run_steps(void* s, int n, double* dts) {
  auto* S = (Solver*)s;
  for (int i = 0; i < n; ++i) {
    double dt = S->timestep();
    if (!(dt > 0.0)) return -1;
    if (dts) dts[i] = dt;
    S->rk_step(dt);
  }
  return 0;
}

// ---- implicit step (backward Euler, BDLU matrix, restarted GMRES) ----
// cfl: stability number of the step; local_dt: 1 = LOCAL_STABILITY_CONDITION, 0 = global minimum;
// nkrylov, max_it, inv_res: NKRYLOV, IMP_MAX_IT, INV_RES.  l1 (5, may be null) receives the L1
// norm of the update per variable, iters (may be null) the GMRES restarts taken.
// Returns GMRES info (restarts - 1, or -1 when not converged), -2 on a bad time step.
int ory_solver_implicit_step(void* s, double cfl, int local_dt, int nkrylov, int max_it, double inv_res,
                             double* l1, int* iters) {
  auto* S = (Solver*)s;
  S->nkrylov = nkrylov; S->imp_max_it = max_it; S->inv_res = inv_res;
  int info = S->implicit_step(cfl, local_dt != 0, l1);
  if (iters) *iters = S->gmres_iters;
  return info;
}
// Typhon's steady implicit run (ns_typhon_steady).  dp: cfl, cfl_max, cycle_res, global_res,
// inv_res; ip: nkrylov, imp_max_it, max_iters, max_cycles; hist: faces of the history family.
// Writes up to cap log10 residuals and, per cycle, 5 flux sums, 5 ghost averages and the end
// iteration; returns the iteration count and the cycle count in *ncycle.
int ory_solver_typhon_steady(void* s, const double* dp, const int* ip, int nhist, const int* hist, int cap,
                             double* log_res, double* flux_sum, double* ghost_avg, int* cycle_end, int* ncycle) {
  auto* S = (Solver*)s;
  NsSteadyParams p;
  p.cfl = dp[0]; p.cfl_max = dp[1]; p.cycle_res = dp[2]; p.global_res = dp[3];
  S->inv_res = dp[4]; S->nkrylov = ip[0]; S->imp_max_it = ip[1];
  p.max_iters = ip[2]; p.max_cycles = ip[3]; p.rk_method = ip[4]; p.local_dt = ip[5] != 0;
  p.history_faces.assign(hist, hist + nhist);
  NsSteadyOut out;
  ns_typhon_steady(*S, p, out);
  const int n = (int)out.log_res.size(), ncy = (int)out.cycle_end.size();
  for (int i = 0; i < n && i < cap; ++i) log_res[i] = out.log_res[i];
  for (int i = 0; i < ncy && i < cap; ++i) {
    cycle_end[i] = out.cycle_end[i];
    for (int v = 0; v < 5; ++v) { flux_sum[5 * i + v] = out.flux_sum[5 * i + v]; ghost_avg[5 * i + v] = out.ghost_avg[5 * i + v]; }
  }
  *ncycle = ncy;
  return n;
}
// linear solver of the implicit step: 0 Typhon's GMRES, 1 Typhon's BiCGSTAB
void ory_solver_set_inversion(void* s, int kind) { ((Solver*)s)->inversion = kind; }
// y = A x with the BDLU matrix of the last implicit step (x, y: 5 per cell, per-cell blocks)
void ory_solver_bdlu_matvec(void* s, const double* x, double* y) { ((Solver*)s)->bdlu_yeqax(x, y); }

// ---- Typhon non-regression cases with .tym meshes ----
// case 1: NRG/TIME/RUNGEKUTTA/<method>  (HLLC, MUSCL-FAST, van Albada, periodic),
//         probe RHOERR = vol-avg (rho - rho_exact(x - 50 t, y))^2
// case 2: NRG/MESH/CON/PER2D-TRANS     (Rusanov, first order, periodic),
// case 3: NRG/MESH/ELEM/TYM-QUAD       (HLLC, first order, symmetry on all sides), probe PAVG = vol-avg p
// case 4/5: NRG/NS/NUM/FLUX/VISCOUS/CELLAVG | CELLFULL (laminar, nu = 1, moving adiabatic walls);
//         out[0:ncycle] = VXERR, out[ncycle:2 ncycle] = DELTA
//         probe RHODEV = vol-avg (rho - 1.25)^2
// Writes ncycle probe values into out; returns the number of time steps taken, < 0 on error.
int ory_run_nrg(int which, void* mesh, int rk_method, double cfl, int ncycle, double duration, double* out) {
  auto& m = ((MeshHandle*)mesh)->m;
  Solver S;
  SpatParams sp;
  if (which == 1) {
    sp.scheme = SCH_HLLC; sp.highres = HRES_MUSCLFAST; sp.limiter = LIM_ALBADA; sp.gradmeth = GRAD_LSQ;
  } else if (which == 2) {
    sp.scheme = SCH_RUSANOV; sp.highres = HRES_NONE; sp.gradmeth = GRAD_NONE;
  } else if (which == 3) {
    sp.scheme = SCH_HLLC; sp.highres = HRES_NONE; sp.gradmeth = GRAD_NONE;
  } else if (which == 4 || which == 5) {
    sp.scheme = SCH_HLLC; sp.highres = HRES_MUSCLFAST; sp.limiter = LIM_ALBADA; sp.gradmeth = GRAD_LSQ;
    sp.viscous = which == 4 ? VISC_CELLAVG : VISC_CELLFULL;
    sp.visc_law = 0;
    sp.visc_kin = 1.;
  } else {
    return -1;
  }
  S.init(&m, sp, rk_method, cfl);
  const double pi = 3.14159265358979323846;
  const int nc = m.ncell;
  for (int c = 0; c < nc; ++c) {  // BLOCK:INIT at cell centres, ghosts included (init_ns_ust.f90)
    double x = m.ccentre[c].x, y = m.ccentre[c].y;
    double rho, vx;
    if (which == 4 || which == 5) {  // DENSITY = 1, P = 100/1.4, VX = erf(y/2/sqrt(1))
      S.prim[c] = 1.;
      S.prim[nc + c] = 100 / 1.4;
      S.prim[2 * nc + c] = std::erf(y / 2 / std::sqrt(1.));
      S.prim[3 * nc + c] = 0.;
      S.prim[4 * nc + c] = 0.;
      continue;
    }
    if (which == 3) {  // P = 1e5, T = 300, MACH = 0.2 along x (init_ns_ust.f90: density from p/(r T))
      const double p = 1.0E5, T = 300., rcst = 287.14, gam = 1.4;
      rho = p / (rcst * T);
      double vel = std::sqrt((gam * p / rho)) * .2;
      S.prim[c] = rho;
      S.prim[nc + c] = p;
      S.prim[2 * nc + c] = (vel / 1.0) * 1.;
      S.prim[3 * nc + c] = (vel / 1.0) * 0.;
      S.prim[4 * nc + c] = (vel / 1.0) * 0.;
      continue;
    }
    if (which == 1) {
      double s = std::sin(2 * pi * x) * std::sin(2 * pi * y);
      rho = 1 + (s * s) / 2;
      vx = 50.;
    } else {
      rho = 1. + 9 * x * (x - 1) * y * (y - 1);
      vx = 10.;
    }
    S.prim[c] = rho;
    S.prim[nc + c] = 100000 / 14.;
    S.prim[2 * nc + c] = vx;
    S.prim[3 * nc + c] = 0.;
    S.prim[4 * nc + c] = 0.;
  }
  S.varcons();
  const double dtbase = duration / ncycle;
  double curtps = 0.0;
  int nsteps = 0;
  for (int icycle = 1; icycle <= ncycle; ++icycle) {
    double cycle_time = 0.0;
    bool end_cycle = false;
    while (!end_cycle) {
      double dtmax = dtbase - cycle_time;
      double dt = S.timestep();
      if (!(dt > 0.0)) return -2;
      dt = std::min(dt, dtmax);
      if (dt >= dtbase - cycle_time) { end_cycle = true; dt = dtbase - cycle_time; }
      S.rk_step(dt);
      cycle_time = cycle_time + dt;
      ++nsteps;
    }
    curtps = curtps + dtbase;
    S.varprim();
    double num = 0.0, num2 = 0.0, vol = 0.0;
    for (int c = 0; c < m.ncell_int; ++c) {
      double q, q2 = 0.0;
      if (which == 4 || which == 5) {  // VXERR and DELTA probes
        double y = m.ccentre[c].y, vx = S.prim[2 * nc + c];
        double e = vx - std::erf(y / 2 / std::sqrt(curtps + 1.));
        q = e * e;
        q2 = 2 * 50 * (1 - vx * vx);
      } else if (which == 3) {
        q = S.prim[nc + c];
      } else if (which == 1) {
        double x = m.ccentre[c].x, y = m.ccentre[c].y;
        double s = std::sin(2 * pi * (x - 50 * curtps)) * std::sin(2 * pi * y);
        double e = S.prim[c] - (1 + (s * s) / 2);
        q = e * e;
      } else {
        double e = S.prim[c] - 1.25;
        q = e * e;
      }
      num += q * m.cvol[c];
      num2 += q2 * m.cvol[c];
      vol += m.cvol[c];
    }
    out[icycle - 1] = num / vol;
    if (which == 4 || which == 5) out[ncycle + icycle - 1] = num2 / vol;
  }
  return nsteps;
}

}  // extern "C"

// ---- heat conduction (KDIF) ----
extern "C" {
// scheme: 0 compact, 1 cell-average, 2 full; kc[ncell_int] conductivity; kind/value[nface]:
// KdifBc and the wall temperature or imposed flux of each boundary face
void* ory_kdif_new(void* mesh, int scheme, double cp, const double* kc, const int* kind, const double* value) {
  auto* k = new KdifSolver();
  k->init(&((MeshHandle*)mesh)->m, scheme, cp, kc, kind, value);
  return k;
}
void ory_kdif_free(void* k) { delete (KdifSolver*)k; }
void ory_kdif_set_T(void* k, const double* T) {
  auto* K = (KdifSolver*)k;
  for (int c = 0; c < K->m->ncell_int; ++c) K->T[c] = T[c];
}
void ory_kdif_rhs(void* k, double dt) { ((KdifSolver*)k)->rhs(dt); }
void ory_kdif_assemble(void* k, double dt) { ((KdifSolver*)k)->assemble(dt); }
void ory_kdif_matvec(void* k, const double* x, double* y) { ((KdifSolver*)k)->matvec(x, y); }
// which: 0 T [ncell], 1 grad [3][ncell], 2 flux*S [nface], 3 J_R*S [nface], 4 residu [ncell],
//        5 flux balance [ncell_int], 6 diagonal [ncell_int]
int ory_kdif_get(void* k, int which, double* out) {
  auto* K = (KdifSolver*)k;
  const std::vector<double>* v = nullptr;
  switch (which) {
    case 0: v = &K->T; break;
    case 1: v = &K->grad; break;
    case 2: v = &K->flux; break;
    case 3: v = &K->jac; break;
    case 4: v = &K->residu; break;
    case 5: v = &K->balance; break;
    case 6: v = &K->diag; break;
    default: return -1;
  }
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return (int)v->size();
}
// Typhon's steady KDIF run from the temperature set by ory_kdif_set_T.  dp: fourier,
// conduct, cycle_res, global_res, inv_res; ip: imp_max_it, max_iters, max_cycles, inversion
// (0 CGS, 1 BICG, 2 GMRES), nkrylov.  Writes
// up to cap iterations' log10 residuals and cycles' averages and end iterations; returns the
// iteration count (negative cycle count in *ncycle_out).
int ory_kdif_typhon_steady(void* k, const double* dp, const int* ip, int cap, double* log_res, double* cycle_avg,
                           int* cycle_end, int* ncycle_out) {
  KdifSolver* s = (KdifSolver*)k;
  KdifSteadyParams p;
  p.fourier = dp[0]; p.conduct = dp[1]; p.cycle_res = dp[2]; p.global_res = dp[3]; p.cgs_maxres = dp[4];
  p.cgs_max_it = ip[0]; p.max_iters = ip[1]; p.max_cycles = ip[2]; p.inversion = ip[3]; p.nkrylov = ip[4];
  std::vector<double> U(s->T.begin(), s->T.begin() + s->m->ncell_int);
  for (auto& u : U) u = u * s->cp;
  KdifSteadyOut out;
  kdif_typhon_steady(*s, U, p, out);
  const int n = (int)out.log_res.size(), nc = (int)out.cycle_avg.size();
  for (int i = 0; i < n && i < cap; ++i) log_res[i] = out.log_res[i];
  for (int i = 0; i < nc && i < cap; ++i) { cycle_avg[i] = out.cycle_avg[i]; cycle_end[i] = out.cycle_end[i]; }
  *ncycle_out = nc;
  return n;
}
int ory_kdif_implicit_step(void* k, double dt, double tol, int max_it, double* rel) {
  return ((KdifSolver*)k)->implicit_step(dt, tol, max_it, rel);
}
}
