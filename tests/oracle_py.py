"""ctypes binding of the CPU oracle (oracle/build/liboracle.so) for the tests.

The oracle is the checker: tests compare the GPU library against it, never the
other way round.  ``load()`` builds it with make on first use.
"""
import ctypes as C
import pathlib
import subprocess

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]
LIB = ROOT / "oracle" / "build" / "liboracle.so"

# enums of oracle/oracle.hpp
BC_PERIODIC, BC_SYMMETRY, BC_WALL, BC_FARFIELD, BC_NOSLIP, BC_HEAT = 1, 2, 3, 4, 5, 6
BC_INLET_SUB, BC_OUTLET_SUB, BC_INLET_SUP, BC_OUTLET_SUP = 7, 8, 9, 10
SCH_HLLC, SCH_RUSANOV, SCH_ROE, SCH_AUSMM, SCH_HLLE = 1, 2, 3, 4, 5
SCH_HLLCB, SCH_HLLCK, SCH_HLLCKB, SCH_HLLEB, SCH_HLLEK, SCH_HLLEKB = 6, 7, 8, 9, 10, 11
HRES_NONE, HRES_MUSCL, HRES_MUSCLFAST, HRES_MUSCLUNS = 0, 1, 2, 3
LIM_NONE, LIM_MINMOD, LIM_ALBADA, LIM_VLEER, LIM_SBEE, LIM_KIM3, LIM_LIM03 = range(7)
POSTLIM_NONE, POSTLIM_BARTH, POSTLIM_SUPERBARTH = 0, 1, 2
GRAD_NONE, GRAD_LSQ, GRAD_LSQW = 0, 1, 2
VISC_NONE, VISC_CELLAVG, VISC_CELLFULL = 0, 1, 2
RK = {"EXPLICIT": 0, "RK2": 1, "RK2-SSP": 2, "RK3-SSP": 3, "RK4": 4, "RK25BB": 5, "RK26BB": 6, "RK12BS": 7, "RK13BS": 8}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        lib.ory_raw_new.restype = vp
        lib.ory_raw_free.argtypes = [vp]
        lib.ory_raw_read_tym.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int]
        lib.ory_raw_set_vtex.argtypes = [vp, C.c_int, vp]
        lib.ory_raw_add_section.argtypes = [vp, C.c_int, C.c_int, vp, vp]
        lib.ory_raw_add_mark.argtypes = [vp, C.c_char_p, C.c_int, vp]
        lib.ory_raw_add_vertex_mark.argtypes = [vp, C.c_char_p, C.c_int, vp]
        lib.ory_mesh_build.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, C.c_char_p, C.c_int]
        lib.ory_raw_set_rotation.argtypes = [vp, C.c_char_p, vp, vp, C.c_double]
        lib.ory_mesh_face_rotation.argtypes = [vp, vp]
        lib.ory_mesh_sizes.argtypes = [vp, vp]
        lib.ory_mesh_export.argtypes = [vp] + [vp] * 11
        lib.ory_mesh_facevtex.argtypes = [vp, C.c_int, vp]
        lib.ory_solver_new.restype = vp
        lib.ory_solver_new.argtypes = [vp, vp, vp]
        lib.ory_solver_free.argtypes = [vp]
        lib.ory_solver_set_cons.argtypes = [vp, vp]
        lib.ory_solver_set_prim.argtypes = [vp, vp]
        lib.ory_solver_get.argtypes = [vp, C.c_int, vp]
        lib.ory_solver_timestep.argtypes = [vp]
        lib.ory_solver_timestep.restype = C.c_double
        lib.ory_solver_rhs.argtypes = [vp, C.c_double]
        lib.ory_solver_rk_step.argtypes = [vp, C.c_double]
        lib.ory_solver_run_steps.argtypes = [vp, C.c_int, vp]
        lib.ory_solver_implicit_step.argtypes = [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, vp, vp]
        lib.ory_solver_typhon_steady.argtypes = [vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp, vp, vp]
        lib.ory_solver_typhon_steady.restype = C.c_int
        lib.ory_solver_set_inversion.argtypes = [vp, C.c_int]
        lib.ory_solver_implicit_step.restype = C.c_int
        lib.ory_solver_bdlu_matvec.argtypes = [vp, vp, vp]
        lib.ory_kdif_new.argtypes = [vp, C.c_int, C.c_double, vp, vp, vp]
        lib.ory_kdif_new.restype = vp
        lib.ory_kdif_free.argtypes = [vp]
        lib.ory_kdif_set_T.argtypes = [vp, vp]
        lib.ory_kdif_rhs.argtypes = [vp, C.c_double]
        lib.ory_kdif_assemble.argtypes = [vp, C.c_double]
        lib.ory_kdif_matvec.argtypes = [vp, vp, vp]
        lib.ory_kdif_get.argtypes = [vp, C.c_int, vp]
        lib.ory_kdif_implicit_step.argtypes = [vp, C.c_double, C.c_double, C.c_int, vp]
        lib.ory_kdif_implicit_step.restype = C.c_int
        lib.ory_kdif_typhon_steady.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp, vp]
        lib.ory_kdif_typhon_steady.restype = C.c_int
        lib.ory_run_nrg.argtypes = [C.c_int, vp, C.c_int, C.c_double, C.c_int, C.c_double, vp]
        lib.ory_roe_flux.argtypes = [C.c_double, C.c_double, C.c_int, vp, vp, vp, vp]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def roe_flux(L, R, nrm, gamma=1.4, entropy_fix=0.1):
    """The oracle's Roe flux per unit area on arrays of face states: L, R [n][5] primitive
    (rho, p, u, v, w), nrm [n][3] unit normals -> [n][5] (mass, energy, momentum)."""
    lib = load()
    L = np.ascontiguousarray(L, np.float64)
    R = np.ascontiguousarray(R, np.float64)
    nrm = np.ascontiguousarray(nrm, np.float64)
    F = np.zeros_like(L)
    lib.ory_roe_flux(float(gamma), float(entropy_fix), L.shape[0], _p(L), _p(R), _p(nrm), _p(F))
    return F


class Mesh:
    """Raw mesh + Typhon preprocessing inside the oracle."""

    def __init__(self):
        self.lib = load()
        self.h = C.c_void_p(self.lib.ory_raw_new())

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ory_raw_free(self.h)
            self.h = None

    @classmethod
    def from_tym(cls, path):
        m = cls()
        err = C.create_string_buffer(256)
        if m.lib.ory_raw_read_tym(m.h, str(path).encode(), err, 256) != 0:
            raise RuntimeError(err.value.decode())
        return m

    @classmethod
    def from_raw(cls, raw):
        """raw: typhon_gb300.umesh.RawMesh-like object (vtex, sections, marks)."""
        m = cls()
        vt = np.ascontiguousarray(raw.vtex, dtype=np.float64)
        m.lib.ory_raw_set_vtex(m.h, vt.shape[0], _p(vt))
        for typ, ielem, conn in raw.sections:
            ie = np.ascontiguousarray(ielem, dtype=np.int32)
            cv = np.ascontiguousarray(conn, dtype=np.int32)
            m.lib.ory_raw_add_section(m.h, int(typ), ie.shape[0], _p(ie), _p(cv))
        for name, tags, *loc in raw.marks:
            t = np.ascontiguousarray(tags, dtype=np.int32)
            add = m.lib.ory_raw_add_vertex_mark if loc and loc[0] == "vertex" else m.lib.ory_raw_add_mark
            add(m.h, name.encode(), t.shape[0], _p(t))
        return m

    def build(self, dim, bcs, rotations=None):
        """bcs: list of (family, kind, partner, translation(3)[, wall_velocity(3)[, data(6)]]),
        data the inlet / outlet parameters of BcKind; rotations: {family: (centre(3), axis(3),
        angle in degrees)} for periodic families connected by a rotation."""
        for fam_, (ctr, ax, ang) in (rotations or {}).items():
            c3 = np.ascontiguousarray(ctr, np.float64)
            a3 = np.ascontiguousarray(ax, np.float64)
            self.lib.ory_raw_set_rotation(self.h, fam_.upper().encode(), _p(c3), _p(a3), float(ang))
        n = len(bcs)
        fam = (C.c_char_p * n)(*[b[0].encode() for b in bcs])
        kind = np.array([b[1] for b in bcs], dtype=np.int32)
        par = (C.c_char_p * n)(*[(b[2] or "").encode() for b in bcs])
        tr = np.array([b[3] for b in bcs], dtype=np.float64).reshape(-1)
        wv = np.array([b[4] if len(b) > 4 else (0, 0, 0) for b in bcs], dtype=np.float64).reshape(-1)
        bd = np.array([tuple(b[5]) + (0.0,) * (6 - len(b[5])) if len(b) > 5 else (0.0,) * 6 for b in bcs],
                      dtype=np.float64).reshape(-1)
        err = C.create_string_buffer(256)
        rc = self.lib.ory_mesh_build(self.h, dim, n, C.cast(fam, C.c_void_p), _p(kind),
                                     C.cast(par, C.c_void_p), _p(tr), _p(wv), _p(bd), err, 256)
        if rc != 0:
            raise RuntimeError(err.value.decode())
        s = np.zeros(7, dtype=np.int32)
        self.lib.ory_mesh_sizes(self.h, _p(s))
        (self.ncell_int, self.ncell, self.nface_int, self.nface, self.ncolors, self.dim,
         self.nboco) = map(int, s)
        return self

    def face_rotation(self):
        """[nface, 3, 3]: the rotation into each face's frame (identity off rotational faces)."""
        out = np.zeros(9 * self.nface)
        self.lib.ory_mesh_face_rotation(self.h, _p(out))
        return out.reshape(self.nface, 3, 3)

    def export(self):
        nf, nc = self.nface, self.ncell
        d = dict(
            fc1=np.zeros(nf, np.int32), fc2=np.zeros(nf, np.int32),
            fnormal=np.zeros((nf, 3)), fcentre=np.zeros((nf, 3)), fsurf=np.zeros(nf),
            ccentre=np.zeros((nc, 3)), cvol=np.zeros(nc),
            face_color=np.zeros(nf, np.int32), face_partner=np.zeros(nf, np.int32),
            face_bckind=np.zeros(nf, np.int32), face_wallvel=np.zeros((nf, 3)))
        self.lib.ory_mesh_export(self.h, *[_p(d[k]) for k in (
            "fc1", "fc2", "fnormal", "fcentre", "fsurf", "ccentre", "cvol", "face_color",
            "face_partner", "face_bckind", "face_wallvel")])
        d.update(ncell_int=self.ncell_int, ncell=self.ncell, nface_int=self.nface_int,
                 nface=self.nface, dim=self.dim)
        return d


class Solver:
    def __init__(self, mesh, scheme=SCH_HLLC, highres=HRES_NONE, limiter=LIM_ALBADA,
                 postlim=POSTLIM_NONE, gradmeth=GRAD_NONE, rk="RK4", gamma=1.4, cfl=1.0,
                 entropy_fix=0.1, viscous=0, visc_law=0, visc_kin=0.0, rgas=287.14, prandtl=0.72,
                 farfield=(1.0, 1.0 / 1.4, 0.0, 0.0, 0.0)):
        self.lib = load()
        self.mesh = mesh
        ip = np.array([scheme, highres, limiter, postlim, gradmeth, RK[rk], viscous, visc_law], np.int32)
        dp = np.array([gamma, cfl, entropy_fix, visc_kin, rgas, prandtl, *farfield], np.float64)
        self.h = C.c_void_p(self.lib.ory_solver_new(mesh.h, _p(ip), _p(dp)))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ory_solver_free(self.h)
            self.h = None

    def set_cons(self, cons):
        c = np.ascontiguousarray(cons, dtype=np.float64)
        assert c.size == 5 * self.mesh.ncell
        self.lib.ory_solver_set_cons(self.h, _p(c))

    def set_prim(self, prim):
        c = np.ascontiguousarray(prim, dtype=np.float64)
        assert c.size == 5 * self.mesh.ncell
        self.lib.ory_solver_set_prim(self.h, _p(c))

    _SIZES = {0: "c5", 1: "c5", 2: "c15", 3: "c5", 4: "f5", 5: "f5", 6: "f5", 7: "c1", 8: "c3"}

    def get(self, which):
        code = {"cons": 0, "prim": 1, "grad": 2, "residu": 3, "flux": 4, "cell_l": 5,
                "cell_r": 6, "dtloc": 7, "limratio": 8}[which]
        kind = self._SIZES[code]
        n = self.mesh.ncell if kind[0] == "c" else self.mesh.nface
        k = int(kind[1:])
        out = np.zeros(k * n)
        self.lib.ory_solver_get(self.h, code, _p(out))
        return out.reshape(k, n)

    def timestep(self):
        return self.lib.ory_solver_timestep(self.h)

    def get_implicit(self, which):
        """Jacobians and BDLU blocks of the last implicit step: jacL, jacR, upper, lower are
        (nface, 5, 5), diag (ncell, 5, 5); rows are (rho, rhoE, rhou, rhov, rhow)."""
        code, n = {"jacL": (9, self.mesh.nface), "jacR": (10, self.mesh.nface), "diag": (11, self.mesh.ncell),
                   "upper": (12, self.mesh.nface), "lower": (13, self.mesh.nface)}[which]
        out = np.zeros(25 * n)
        assert self.lib.ory_solver_get(self.h, code, _p(out)) == 25 * n
        return out.reshape(n, 5, 5)

    def implicit_rhs(self):
        """Right-hand side of the last implicit solve, (ncell, 5)."""
        out = np.zeros(5 * self.mesh.ncell)
        assert self.lib.ory_solver_get(self.h, 14, _p(out)) == out.size
        return out.reshape(self.mesh.ncell, 5)

    def implicit_step(self, cfl, local_dt=False, nkrylov=50, max_it=50, inv_res=1e-4):
        """One backward-Euler step; returns (info, gmres restarts, L1 of the update per variable)."""
        l1 = np.zeros(5)
        it = C.c_int()
        info = self.lib.ory_solver_implicit_step(self.h, float(cfl), int(local_dt), int(nkrylov), int(max_it),
                                                 float(inv_res), _p(l1), C.byref(it))
        if info == -2:
            raise RuntimeError("oracle implicit step: bad time step")
        return info, it.value, l1

    def set_inversion(self, name):
        """Linear solver of the implicit step: GMRES or BICGSTAB (Typhon's bdlu_*)."""
        self.lib.ory_solver_set_inversion(self.h, {"GMRES": 0, "BICGSTAB": 1}[name])

    def typhon_steady(self, cfl, cfl_max=None, cycle_res=0.1, global_res=1e-4, nkrylov=50, max_it=50,
                      inv_res=1e-4, history_faces=(), max_iters=100000, max_cycles=1000, method="IMPLICIT",
                      local_dt=False):
        """Typhon's steady run from the current state (implicit, or an explicit method of RK):
        log10 residual per iteration, per cycle the flux sums (F S) and S-weighted ghost
        primitive averages over history_faces, and the iteration count at each cycle's end."""
        cap = max_iters + 1
        dp = np.array([cfl, cfl if cfl_max is None else cfl_max, cycle_res, global_res, inv_res], np.float64)
        ip = np.array([nkrylov, max_it, max_iters, max_cycles, -1 if method == "IMPLICIT" else RK[method],
                       int(local_dt)], np.int32)
        hist = np.ascontiguousarray(history_faces, np.int32)
        lr, fs, ga, end = np.zeros(cap), np.zeros(5 * cap), np.zeros(5 * cap), np.zeros(cap, np.int32)
        nc = C.c_int()
        n = self.lib.ory_solver_typhon_steady(self.h, _p(dp), _p(ip), hist.size, _p(hist), cap, _p(lr), _p(fs),
                                              _p(ga), _p(end), C.byref(nc))
        k = nc.value
        return lr[:n], fs[:5 * k].reshape(k, 5), ga[:5 * k].reshape(k, 5), end[:k]

    def bdlu_matvec(self, x):
        """y = A x with the BDLU matrix of the last implicit step; x is (ncell, 5)."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.lib.ory_solver_bdlu_matvec(self.h, _p(x), _p(y))
        return y

    def rhs(self, dt):
        self.lib.ory_solver_rhs(self.h, dt)

    def rk_step(self, dt):
        self.lib.ory_solver_rk_step(self.h, dt)

    def run_steps(self, n):
        dts = np.zeros(n)
        rc = self.lib.ory_solver_run_steps(self.h, n, _p(dts))
        if rc != 0:
            raise RuntimeError("oracle step failed (negative energy or NaN)")
        return dts


def run_nrg(which, mesh, rk, cfl, ncycle=100, duration=0.1):
    lib = load()
    out = np.zeros(2 * ncycle)
    ns = lib.ory_run_nrg(which, mesh.h, RK[rk], cfl, ncycle, duration, _p(out))
    if ns < 0:
        raise RuntimeError(f"oracle NRG case failed ({ns})")
    if which in (4, 5):
        return (out[:ncycle], out[ncycle:]), ns
    return out[:ncycle], ns


PERIODIC_UNIT_SQUARE = [("IMIN", BC_PERIODIC, "IMAX", (1.0, 0.0, 0.0)),
                        ("JMIN", BC_PERIODIC, "JMAX", (0.0, 1.0, 0.0))]


KDIF_COMPACT, KDIF_CELLAVG, KDIF_FULL = 0, 1, 2
KBC_ISOTHERMAL, KBC_FLUX, KBC_EXTRAPOLATE = 1, 2, 3


class Kdif:
    """Heat-conduction oracle (oracle_kdif.cpp) on a built Mesh."""

    def __init__(self, mesh, scheme, cp, conductivity, face_kind, face_value):
        self.lib = load()
        self.mesh = mesh
        kc = np.ascontiguousarray(conductivity, np.float64)
        fk = np.ascontiguousarray(face_kind, np.int32)
        fv = np.ascontiguousarray(face_value, np.float64)
        self.h = C.c_void_p(self.lib.ory_kdif_new(mesh.h, int(scheme), float(cp), _p(kc), _p(fk), _p(fv)))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ory_kdif_free(self.h)
            self.h = None

    def set_T(self, T):
        t = np.ascontiguousarray(T[:self.mesh.ncell_int], np.float64)
        self.lib.ory_kdif_set_T(self.h, _p(t))

    def rhs(self, dt):
        self.lib.ory_kdif_rhs(self.h, float(dt))

    def assemble(self, dt):
        self.lib.ory_kdif_assemble(self.h, float(dt))

    def get(self, which):
        m = self.mesh
        code, n = {"T": (0, m.ncell), "grad": (1, 3 * m.ncell), "flux": (2, m.nface), "jac": (3, m.nface),
                   "residu": (4, m.ncell), "balance": (5, m.ncell_int), "diag": (6, m.ncell_int)}[which]
        out = np.zeros(n)
        assert self.lib.ory_kdif_get(self.h, code, _p(out)) == n
        return out.reshape(3, m.ncell) if which == "grad" else out

    def matvec(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.lib.ory_kdif_matvec(self.h, _p(x), _p(y))
        return y

    def implicit_step(self, dt, tol=1e-12, max_it=10000):
        rel = C.c_double()
        it = self.lib.ory_kdif_implicit_step(self.h, float(dt), float(tol), int(max_it), C.byref(rel))
        return it, rel.value

    def typhon_steady(self, fourier, conduct, cycle_res=0.1, global_res=1e-5, cgs_maxres=1e-4, cgs_max_it=10,
                      max_iters=100000, max_cycles=1000, inversion="CGS", nkrylov=10):
        """Typhon's steady implicit run (DLU + CGS) from the current temperature: log10 residual
        per iteration, volume-averaged temperature and total iterations after each cycle."""
        cap = max_iters + 1
        dp = np.array([fourier, conduct, cycle_res, global_res, cgs_maxres], np.float64)
        ip = np.array([cgs_max_it, max_iters, max_cycles, {"CGS": 0, "BICG": 1, "GMRES": 2}[inversion], nkrylov],
                      np.int32)
        lr, avg, end = np.zeros(cap), np.zeros(cap), np.zeros(cap, np.int32)
        nc = C.c_int()
        n = self.lib.ory_kdif_typhon_steady(self.h, _p(dp), _p(ip), cap, _p(lr), _p(avg), _p(end), C.byref(nc))
        return lr[:n], avg[:nc.value], end[:nc.value]
