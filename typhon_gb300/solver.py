"""Host-side mirror of Typhon's zone-integration interface on top of the C ABI.

``Grid`` plays the role of Typhon's st_grid for one zone on one GPU: it owns the device
mesh (ty_mesh) and its resident state, and exposes the calls that Typhon's drivers make,
under the same names and with the same meaning:

  calc_zonetimestep      SOURCE/ZONE/calc_zonetimestep.f90:10 (global stability dt)
  integration_grid       SOURCE/MAIN/integration_grid.f90:8 (zone residual dt/V sum F S)
  treelevel_rungekutta   SOURCE/MAIN/treelevel_rungekutta.f90:8 + update_field.f90:9
  integration_cyclezone  SOURCE/MAIN/integration_cyclezone.f90:11 (unsteady cycle loop)

Errors that Typhon turns into error_stop are raised as TyphonError with the library's
status code.
"""
import ctypes as C

import numpy as np

from . import _capi
from .umesh import MeshDesc

# option names as in Typhon's SPAT_PARAM / TIME_PARAM blocks (SOURCE/PARAM/def_spat.f90,
# def_time.f90) -> C ABI enum values
SCHEME = {"HLLC": 1, "RUSANOV": 2, "ROE": 3, "AUSMM": 4, "HLLE": 5, "HLL": 5, "HLLCB": 6, "HLLCK": 7, "HLLCKB": 8,
          "HLLEB": 9, "HLLEK": 10, "HLLEKB": 11}
HIGHRES = {"NONE": 0, "MUSCL": 1, "MUSCL-FAST": 2, "MUSCL-UNS": 3}
LIMITER = {"NONE": 0, "MINMOD": 1, "ALBADA": 2, "VAN_ALBADA": 2, "VAN_LEER": 3, "VANLEER": 3, "SUPERBEE": 4,
           "KIM3": 5, "LIM03": 6}
POSTLIM = {"NONE": 0, "BARTH": 1, "SUPERBARTH": 2}
GRADMETH = {"NONE": 0, "LSQ": 1, "W-LSQ": 2}
RK_METHOD = {"EXPLICIT": 0, "RK2": 1, "RK2-SSP": 2, "RK3-SSP": 3, "RK4": 4, "RK25BB": 5, "RK26BB": 6, "RK12BS": 7, "RK13BS": 8}
MODE = {"exact": 0, "fast": 1}
DISSIPATIVE_FLUX = {"NONE": 0, "CELL-AVERAGE": 1, "FULL": 2}
VISC_LAW = {"KINEMATIC-CONSTANT": 0, "SUTHERLAND": 1}
KRYLOV = {"GMRES": 0, "FGMRES": 1, "JFNK": 2, "BICGSTAB": 3}
PRECISION = {"fp64": 0, "mixed": 1, "mixed-fp64ortho": 2}
KDIF_FLUX = {"COMPACT": 0, "CELL-AVERAGE": 1, "FULL": 2}
KBC_ISOTHERMAL, KBC_FLUX, KBC_EXTRAPOLATE = 1, 2, 3


def prim_to_cons(prim, gamma=1.4):
    """calc_varcons_ns (SOURCE/EQNS/calc_varcons_ns.f90:37-46), same operation order."""
    rho, p, u, v, w = prim
    ig1 = 1.0 / (gamma - 1.0)
    cons = np.empty_like(prim)
    cons[0] = rho
    cons[1] = ig1 * p + 0.5 * rho * (u * u + v * v + w * w)
    cons[2], cons[3], cons[4] = rho * u, rho * v, rho * w
    return cons


class Grid:
    """One zone grid resident on one GPU."""

    def __init__(self, mesh: MeshDesc, device=0):
        self.mesh = mesh
        self.lib = _capi.lib()
        self._desc = mesh.to_c()
        h = C.c_void_p()
        _capi.check(self.lib.ty_mesh_create(C.byref(self._desc), int(device), C.byref(h)), "ty_mesh_create")
        self.h = h
        if getattr(mesh, "face_rotation", None) is not None:
            rot = np.ascontiguousarray(mesh.face_rotation, np.float64)
            _capi.check(self.lib.ty_mesh_set_face_rotation(h, rot.ctypes.data), "ty_mesh_set_face_rotation")
        self.nci = mesh.ncell_int
        self.gamma = 1.4
        self.gradmeth = "NONE"
        self.time = 0.0

    def close(self):
        if getattr(self, "h", None):
            self.lib.ty_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def info(self):
        out = np.zeros(5, np.int32)
        _capi.check(self.lib.ty_mesh_info(self.h, out.ctypes.data), "ty_mesh_info")
        return dict(zip(("ncell_int", "ncell", "nface_int", "nface", "max_faces_per_cell"), map(int, out)))

    # -- def_spat --------------------------------------------------------------------------
    def set_spat(self, scheme="HLLC", highres="NONE", limiter="ALBADA", postlim="NONE", gradmeth=None,
                 mode="exact", gamma=1.4, entropy_fix=0.1, dissipative_flux="NONE", viscosity="KINEMATIC-CONSTANT",
                 kin_visc=0.0, rgas=287.14, prandtl=0.72, farfield=(1.0, 1.0 / 1.4, 0.0, 0.0, 0.0)):
        """SPAT_PARAM: SCHEME, HIGHRES, LIMITER, POST-LIMITER, GRADMETH (LSQ by default with
        MUSCL or a viscous flux, none otherwise, as get_gradientmethod in
        SOURCE/PARAM/MENU_NUM.f90); DISSIPATIVE_FLUX (CELL-AVERAGE | FULL) turns on the laminar
        viscous flux with MODEL: VISCOSITY (KINEMATIC-CONSTANT with KIN_VISC, or SUTHERLAND).
        farfield: free-stream primitive state (rho, p, u, v, w) of far-field boundaries."""
        visc = DISSIPATIVE_FLUX[dissipative_flux]
        if gradmeth is None:
            gradmeth = "NONE" if (highres == "NONE" and visc == 0) else "LSQ"
        p = _capi.SpatParams(SCHEME[scheme], HIGHRES[highres], LIMITER[limiter], POSTLIM[postlim],
                             GRADMETH[gradmeth], MODE[mode], float(gamma), float(entropy_fix), visc,
                             VISC_LAW[viscosity], float(kin_visc), float(rgas), float(prandtl),
                             (C.c_double * 5)(*map(float, farfield)))
        _capi.check(self.lib.ty_set_params(self.h, C.byref(p)), "ty_set_params")
        self.gamma = gamma
        self.gradmeth = gradmeth

    # -- state -----------------------------------------------------------------------------
    def set_cons(self, cons):
        """Conserved state [5][ncell_int] (rho, rhoE, rhou, rhov, rhow), host array."""
        cons = np.ascontiguousarray(cons, np.float64).reshape(5, -1)[:, :self.nci]
        rho = np.ascontiguousarray(cons[0])
        rhoE = np.ascontiguousarray(cons[1])
        rhou = np.ascontiguousarray(cons[2:5].T)
        _capi.check(self.lib.ty_state_upload(self.h, rho.ctypes.data, rhoE.ctypes.data, rhou.ctypes.data),
                    "ty_state_upload")

    def set_prim(self, prim):
        self.set_cons(prim_to_cons(np.asarray(prim, np.float64).reshape(5, -1)[:, :self.nci], self.gamma))

    def set_ghost_prim(self, prim_ghost):
        """Start Typhon's ghost-row bookkeeping of explicit runs (ty_ghost_state_set) from the
        ghost primitive states [5][nghost] (cells ncell_int.. of the mesh), converted as
        calc_varcons_ns does; None stops it."""
        if prim_ghost is None:
            _capi.check(self.lib.ty_ghost_state_set(self.h, None), "ty_ghost_state_set")
            return
        ng = self.mesh.ncell - self.nci
        cons = np.ascontiguousarray(prim_to_cons(np.asarray(prim_ghost, np.float64).reshape(5, ng), self.gamma))
        _capi.check(self.lib.ty_ghost_state_set(self.h, cons.ctypes.data), "ty_ghost_state_set")
        self._ghost_rows = True

    def ghost_prim(self):
        """Primitive variables [5][nghost] of the ghost states of the last stage (the ghost
        primitive variables of a first-order Typhon run)."""
        out = np.zeros((5, self.mesh.ncell - self.nci))
        _capi.check(self.lib.ty_ghost_prim_download(self.h, out.ctypes.data), "ty_ghost_prim_download")
        return out

    def upload_typhon(self, rho, rhoE, rhou):
        """Upload a conserved state given in Typhon's layout without any conversion:
        rho[ncell_int], rhoE[ncell_int], rhou[ncell_int, 3] (contiguous float64, pinned or not)."""
        for a in (rho, rhoE, rhou):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        _capi.check(self.lib.ty_state_upload(self.h, rho.ctypes.data, rhoE.ctypes.data, rhou.ctypes.data),
                    "ty_state_upload")

    def download_typhon(self, rho, rhoE, rhou):
        """Download the conserved state into caller arrays in Typhon's layout."""
        for a in (rho, rhoE, rhou):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        _capi.check(self.lib.ty_state_download(self.h, rho.ctypes.data, rhoE.ctypes.data, rhou.ctypes.data),
                    "ty_state_download")

    def get_cons(self):
        rho = np.zeros(self.nci)
        rhoE = np.zeros(self.nci)
        rhou = np.zeros((self.nci, 3))
        _capi.check(self.lib.ty_state_download(self.h, rho.ctypes.data, rhoE.ctypes.data, rhou.ctypes.data),
                    "ty_state_download")
        return np.vstack([rho, rhoE, rhou.T])

    def get_prim(self):
        out = np.zeros((5, self.nci))
        _capi.check(self.lib.ty_prim_download(self.h, out.ctypes.data), "ty_prim_download")
        return out

    def probe(self, kind, quantity, time=0.0):
        """A volume probe of the resident state (BLOCK:PROBE, TYPE = VOL_MIN | VOL_MAX |
        VOL_AVERAGE, QUANTITY an expression of RHO, PS, V, V_X, V_Y, V_Z, x, y, z, t;
        PROBECALC.f90:22-212) over the interior cells."""
        from . import probes
        m = self.mesh
        env = probes.ns_environment(self.get_prim(), m.cell_centre[:self.nci], time)
        return probes.vol_probe(kind, quantity, env, m.cell_volume[:self.nci])

    def write_vtk(self, path, raw, binary=False):
        """The resident state as Typhon's OUTPUT FORMAT = VTK | VTK-BIN file
        (output_zone.f90): the mesh `raw` (the RawMesh this grid was preprocessed from) and
        the primitive fields RHO, PS, V of the interior cells, downloaded from the device."""
        from . import vtk
        q = self.get_prim()
        vtk.write_vtk(path, raw, scalars=[("RHO", q[0]), ("PS", q[1])], vectors=[("V", q[2:5])], binary=binary)

    def set_cons_device(self, ptr):
        _capi.check(self.lib.ty_state_upload_device(self.h, C.c_void_p(ptr)), "ty_state_upload_device")

    def get_cons_device(self, ptr):
        _capi.check(self.lib.ty_state_download_device(self.h, C.c_void_p(ptr)), "ty_state_download_device")

    # -- Typhon calls ------------------------------------------------------------------------
    def calc_zonetimestep(self, cfl):
        dt = C.c_double()
        _capi.check(self.lib.ty_timestep(self.h, float(cfl), C.byref(dt)), "ty_timestep")
        return dt.value

    def integration_grid(self, dt, out=True):
        R = np.zeros((5, self.nci)) if out else None
        _capi.check(self.lib.ty_residual(self.h, float(dt), R.ctypes.data if out else None), "ty_residual")
        return R

    def treelevel_rungekutta(self, method, dt):
        _capi.check(self.lib.ty_rk_step(self.h, RK_METHOD[method], float(dt)), "ty_rk_step")
        self.time += dt

    def run_steps(self, method, cfl, nsteps):
        """nsteps steps with the global stability time step, all on the device."""
        dt = C.c_double()
        _capi.check(self.lib.ty_rk_steps(self.h, RK_METHOD[method], float(cfl), int(nsteps), C.byref(dt)),
                    "ty_rk_steps")
        return dt.value

    def integration_cyclezone(self, method, cfl, cycle_dt):
        """Integrate one unsteady cycle of length cycle_dt: global stability dt, the last step
        cut to end the cycle exactly (integration_cyclezone.f90:80-170)."""
        cycle_time = 0.0
        nstep = 0
        while True:
            dtmax = cycle_dt - cycle_time
            dt = min(self.calc_zonetimestep(cfl), dtmax)
            end = dt >= cycle_dt - cycle_time
            if end:
                dt = cycle_dt - cycle_time
            self.treelevel_rungekutta(method, dt)
            cycle_time = cycle_time + dt
            nstep += 1
            if end:
                return nstep

    # -- implicit step (calc_rhs.f90:121-138 with the Jacobians, implicit_solve, update_field) --
    def implicit_step(self, cfl, inversion="GMRES", nkrylov=50, max_it=50, inv_res=1e-4, local_dt=False,
                      precision="fp64", scaling="state"):
        """One backward-Euler step on the resident state.  inversion: GMRES (Typhon's
        bdlu_gmres), FGMRES (block Jacobi, measured Gram matrix) or JFNK; precision fp64 | mixed-fp64ortho
        (FGMRES: FP32 matrix, mat-vec and block Jacobi, FP64 basis) | mixed (FGMRES: FP32 basis too);
        scaling (FGMRES, JFNK): "state" divides equation v by the state's RMS magnitude of
        variable v, "none" solves the rows as assembled.  Returns the ty_imp_stats fields as a dict."""
        p = _capi.ImpParams(KRYLOV[inversion], PRECISION[precision], int(nkrylov), int(max_it), int(local_dt),
                            {"state": 0, "none": 1}[scaling], float(inv_res), float(cfl))
        st = _capi.ImpStats()
        _capi.check(self.lib.ty_implicit_step(self.h, C.byref(p), C.byref(st)), "ty_implicit_step")
        return dict(info=st.info, restarts=st.restarts, matvecs=st.matvecs, dt_min=st.dt_min,
                    res_l2=np.array(st.res_l2[:]), du_l1=np.array(st.du_l1[:]), lin_res=st.lin_res,
                    du_mom=st.du_mom)

    def set_boundary_params(self, params):
        """Inlet / outlet parameters by family: {family: values} with, per kind (BCS of
        Typhon's BOCO blocks), SUBSONIC_INLET (PI, TI, dir_x, dir_y, dir_z), SUBSONIC_OUTLET
        (P,), SUPERSONIC_INLET (PI, TI, MACH, dir_x, dir_y, dir_z)."""
        m = self.mesh
        data = np.zeros((m.nface, 6))
        for fam, vals in params.items():
            vals = tuple(map(float, vals))
            data[m.faces_of(fam), :len(vals)] = vals
        _capi.check(self.lib.ty_set_bc_data(self.h, np.ascontiguousarray(data).ctypes.data), "ty_set_bc_data")

    def ns_steady(self, cfl, cfl_max=None, cycle_res=0.1, global_res=1e-4, inversion="GMRES", nkrylov=50,
                  max_it=50, inv_res=1e-4, precision="fp64", history=None, max_iters=100000, max_cycles=1000,
                  cycle_max_it=None, method="IMPLICIT", local_dt=False):
        """Typhon's steady run of one zone from the resident state (integration.f90,
        integration_cycle.f90, integration_cyclezone.f90, check_end_cycle.f90; the CFL law of
        calc_zonetimestep.f90, cfl (1 - log10 of the zone's and the world's residual drops,
        at least 1) capped at cfl_max; the residual of update_field.f90 with the reference
        state of calc_refcons.f90).  method: IMPLICIT (TIME_PARAM METHOD = IMPLICIT, one
        implicit_step per iteration with inversion / nkrylov / max_it / inv_res / precision)
        or an explicit method (EXPLICIT, RK2, ..., one ty_steady_iteration: global stability
        time step, one step, the update's residual sums).  local_dt: DTCALC =
        LOCAL_STABILITY_CONDITION (per-cell time steps) for either method.  history: a family whose summed
        face fluxes F S (integ_ustboco.f90's histoflux file) and the S-weighted average of
        the ghost primitive states the fluxes were computed from after each cycle are
        returned.  The second equals Typhon's histovar file when Typhon writes the boundary
        states into its ghost cells (runs with gradients); in a first-order run Typhon's
        ghost cells instead carry conservative states that accumulate the raw boundary
        fluxes F S (flux_to_res.f90 adds them unscaled to the ghost rows, update_field.f90
        adds those rows): with set_ghost_prim called before an explicit first-order run the
        ghost primitive states come from that bookkeeping (ty_ghost_prim_download), as
        Typhon's do.  Three scalars per iteration come back to the host.  Returns
        dict(log_res, cycle_end, flux, ghost)."""
        m, nci = self.mesh, self.nci
        V = m.cell_volume[:nci]
        U = self.get_cons()[:, :nci]
        tot = float(np.sum(V))
        ref0, ref1 = float(np.sum(U[0] * V)) / tot, float(np.sum(U[1] * V)) / tot
        refv = np.sqrt(ref0 * ref1)
        hist = m.faces_of(history) if history else None
        tiny = np.finfo(np.float64).tiny
        cfl_max = cfl if cfl_max is None else cfl_max
        w_ref, w_cur, z_reforig = 1.0, 1.0, None
        log_res, cycle_end, flux, ghost = [], [], [], []
        res3 = np.zeros(3)
        iters = 0
        for icycle in range(1, max_cycles + 1):
            wcur_res, wres_ref = w_cur, w_ref
            w_cur = tiny
            z_ref = z_cur = w_cur
            maxit = min(cycle_max_it or max_iters, max_iters - iters)
            it_loc = 0
            while True:
                it_loc += 1
                iters += 1
                c = cfl * max(1.0, 1.0 - np.log10(z_cur / z_ref) - np.log10(wcur_res / wres_ref))
                if method == "IMPLICIT":
                    st = self.implicit_step(min(c, cfl_max), inversion=inversion, nkrylov=nkrylov, max_it=max_it,
                                            inv_res=inv_res, precision=precision, local_dt=local_dt)
                    z_cur = st["du_l1"][0] / ref0 + st["du_l1"][1] / ref1 + st["du_mom"] / refv
                else:
                    dt = C.c_double()
                    _capi.check(self.lib.ty_steady_iteration(self.h, RK_METHOD[method], float(min(c, cfl_max)),
                                                             int(bool(local_dt)), C.byref(dt), res3.ctypes.data),
                                "ty_steady_iteration")
                    z_cur = res3[0] / ref0 + res3[1] / ref1 + res3[2] / refv
                z_ref = max(z_ref, z_cur)
                log_res.append(np.log10(z_cur))
                if z_cur / z_ref <= cycle_res or it_loc == maxit:
                    break
            if icycle == 1:
                z_reforig = z_ref
            if z_cur / z_reforig >= w_cur / w_ref:
                w_cur, w_ref = z_cur, z_reforig
            if hist is not None:
                # integ_ustboco.f90: sum of F S over the family's faces, and the S-weighted
                # average of the ghost primitive states, face by face
                fl, q = self.debug("flux"), self.debug("prim")
                if getattr(self, "_ghost_rows", False) and method != "IMPLICIT" and self.gradmeth == "NONE":
                    q = q.copy()
                    q[:, nci:] = self.ghost_prim()
                fs, qa, area = np.zeros(5), np.zeros(5), 0.0
                for f in hist:
                    fs = fs + fl[:, f]
                    qa = qa + m.face_surface[f] * q[:, m.fc2[f]]
                for f in hist:
                    area = area + m.face_surface[f]
                flux.append(fs)
                ghost.append(qa / area)
            cycle_end.append(iters)
            if w_cur / w_ref <= global_res or iters >= max_iters:
                break
        return dict(log_res=np.array(log_res), cycle_end=np.array(cycle_end), flux=np.array(flux),
                    ghost=np.array(ghost))

    def implicit_get(self, which):
        """Blocks and vectors of the last implicit step (row-major 5x5 blocks)."""
        m = self.mesh
        code, shape = {"jacL": (0, (m.nface, 5, 5)), "jacR": (1, (m.nface, 5, 5)), "diag": (2, (m.ncell_int, 5, 5)),
                       "upper": (3, (m.nface_int, 5, 5)), "lower": (4, (m.nface_int, 5, 5)),
                       "dtloc": (5, (m.ncell_int,)), "rhs": (6, (m.ncell_int, 5)), "du": (7, (m.ncell_int, 5))}[which]
        out = np.zeros(shape)
        _capi.check(self.lib.ty_implicit_get(self.h, code, out.ctypes.data), "ty_implicit_get")
        return out

    def implicit_matvec(self, x):
        """y = A x with the FP64 BDLU matrix of the last implicit step; x is (ncell_int, 5)."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        _capi.check(self.lib.ty_implicit_matvec(self.h, x.ctypes.data, y.ctypes.data), "ty_implicit_matvec")
        return y

    # -- heat conduction (SOLVER = HEAT) ------------------------------------------------------
    def kdif_setup(self, conductivity, face_kind, face_value, flux="FULL", heat_capacity=1.0):
        """KDIF on this mesh: per-cell conductivity [ncell_int], boundary kind (KBC) and value
        (wall temperature or imposed flux) per face [nface]; flux COMPACT | CELL-AVERAGE | FULL
        (SPAT_PARAM:DISSIPATIVE_FLUX), heat_capacity (MODEL:HEATCAPA)."""
        kc = np.ascontiguousarray(conductivity, np.float64)
        fk = np.ascontiguousarray(face_kind, np.int32)
        fv = np.ascontiguousarray(face_value, np.float64)
        p = _capi.KdifParams(KDIF_FLUX[flux], 0, float(heat_capacity))
        self._kdif_cp = float(heat_capacity)
        _capi.check(self.lib.ty_kdif_setup(self.h, C.byref(p), kc.ctypes.data, fk.ctypes.data, fv.ctypes.data),
                    "ty_kdif_setup")

    def kdif_set_temperature(self, T):
        t = np.ascontiguousarray(np.asarray(T, np.float64)[:self.nci])
        _capi.check(self.lib.ty_kdif_set_temperature(self.h, t.ctypes.data), "ty_kdif_set_temperature")

    def kdif_temperature(self):
        out = np.zeros(self.nci)
        _capi.check(self.lib.ty_kdif_get_temperature(self.h, out.ctypes.data), "ty_kdif_get_temperature")
        return out

    def kdif_write_vtk(self, path, raw, binary=False):
        """The resident temperature as Typhon's VTK output of a heat-conduction zone (TS)."""
        from . import vtk
        vtk.write_vtk(path, raw, scalars=[("TS", self.kdif_temperature())], binary=binary)

    def kdif_residual(self, dt):
        R = np.zeros(self.nci)
        _capi.check(self.lib.ty_kdif_residual(self.h, float(dt), R.ctypes.data), "ty_kdif_residual")
        return R

    def kdif_implicit_step(self, dt, solver="CG", tol=1e-12, max_it=20000, inner_tol=1e-5):
        """One backward-Euler step; solver CG (FP64, Jacobi), CG-MIXED (the same on FP32 face
        conductances to 1e-6, then restarted on the FP64 matrix) or CG32 (FP32 CG inside FP64 iterative refinement).
        Returns iterations, refinements, final relative residual."""
        s = _capi.KdifSolve({"CG": 0, "CG32": 1, "CG-MIXED": 2}[solver], int(max_it), float(tol), float(inner_tol))
        st = _capi.KdifStats()
        _capi.check(self.lib.ty_kdif_implicit_step(self.h, float(dt), C.byref(s), C.byref(st)),
                    "ty_kdif_implicit_step")
        return dict(iterations=st.iterations, refinements=st.refinements, rel_res=st.rel_res, du_l1=st.du_l1)

    def kdif_fourier_dt(self, fourier):
        """Typhon's heat-equation time step for a Fourier number (TIME_PARAM:FOURIER)."""
        dt = C.c_double()
        _capi.check(self.lib.ty_kdif_fourier_dt(self.h, float(fourier), C.byref(dt)), "ty_kdif_fourier_dt")
        return dt.value

    def kdif_steady(self, fourier, cycle_res=0.1, global_res=1e-5, solver="CG", tol=1e-13, max_it=20000,
                    max_iters=100000, max_cycles=1000, cycle_max_it=None):
        """Typhon's steady implicit heat-conduction run from the current temperature
        (integration.f90, integration_cycle.f90, integration_cyclezone.f90, check_end_cycle.f90,
        update_field.f90 for one zone): the time step of `fourier` (stability condition, global
        minimum); each iteration one backward-Euler step; the residual sum|dU| / U_ref with U_ref
        the initial volume average of U = Cp T (calc_refcons.f90); a cycle ends when the residual
        falls to cycle_res times the cycle's largest (TIME_PARAM:RESIDUALS) or after
        cycle_max_it iterations; the run ends when the last cycle's residual falls to
        global_res times the first cycle's largest (PROJECT:RESIDUALS).  Returns dict(log_res:
        log10 residual per iteration as Typhon's monres file, cycle_avg: volume-averaged
        temperature after each cycle as a VOL_AVERAGE probe, cycle_end: iterations at each
        cycle's end).  The linear solves run on the GPU (solver, tol, max_it as in
        kdif_implicit_step); only two scalars per iteration come back to the host."""
        V = self.mesh.cell_volume[:self.nci]
        T = self.kdif_temperature()
        cp = self._kdif_cp
        u_ref = float(np.sum(cp * T * V)) / float(np.sum(V))
        dt = self.kdif_fourier_dt(fourier)
        tiny = np.finfo(np.float64).tiny
        w_ref, z_reforig = 1.0, None
        log_res, cycle_avg, cycle_end = [], [], []
        iters = 0
        for icycle in range(1, max_cycles + 1):
            w_cur = tiny
            z_ref, z_cur = w_cur, w_cur
            maxit = min(cycle_max_it or max_iters, max_iters - iters)
            it_loc = 0
            while True:
                it_loc += 1
                iters += 1
                st = self.kdif_implicit_step(dt, solver=solver, tol=tol, max_it=max_it)
                z_cur = st["du_l1"] / u_ref
                z_ref = max(z_ref, z_cur)
                log_res.append(np.log10(z_cur))
                if z_cur / z_ref <= cycle_res or it_loc == maxit:
                    break
            if icycle == 1:
                z_reforig = z_ref
            if z_cur / z_reforig >= w_cur / w_ref:
                w_cur, w_ref = z_cur, z_reforig
            T = self.kdif_temperature()
            cycle_avg.append(float(np.sum(T * V)) / float(np.sum(V)))
            cycle_end.append(iters)
            if w_cur / w_ref <= global_res or iters >= max_iters:
                break
        return dict(log_res=np.array(log_res), cycle_avg=np.array(cycle_avg), cycle_end=np.array(cycle_end))

    def kdif_get(self, which):
        m = self.mesh
        code, shape = {"T": (0, (m.ncell,)), "grad": (1, (3, m.ncell_int)), "flux": (2, (m.nface,)),
                       "jac": (3, (m.nface,)), "diag": (4, (m.ncell_int,)), "balance": (5, (m.ncell_int,))}[which]
        out = np.zeros(shape)
        _capi.check(self.lib.ty_kdif_get(self.h, code, out.ctypes.data), "ty_kdif_get")
        return out

    def kdif_matvec(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        _capi.check(self.lib.ty_kdif_matvec(self.h, x.ctypes.data, y.ctypes.data), "ty_kdif_matvec")
        return y

    def debug(self, which):
        m = self.mesh
        shapes = {"prim": (0, 5, m.ncell), "grad": (1, 15, m.ncell), "flux": (2, 5, m.nface),
                  "ratio": (3, 3, m.ncell)}
        code, rows, n = shapes[which]
        out = np.zeros((rows, n))
        _capi.check(self.lib.ty_debug_get(self.h, code, out.ctypes.data), "ty_debug_get")
        return out

    def synchronize(self):
        _capi.check(self.lib.ty_synchronize(self.h), "ty_synchronize")
