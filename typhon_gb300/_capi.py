"""ctypes binding of libtyphon_gpu.so (the C ABI declared in include/typhon_gpu.h).

The library is built in-tree (typhon_gb300/build.py).  Loading fails loudly when it is
missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_lib" / "libtyphon_gpu.so"

TY_OK = 0
STATUS = {
    0: "TY_OK", -1: "TY_ERR_ARG", -2: "TY_ERR_CUDA", -3: "TY_ERR_NOMEM", -4: "TY_ERR_MESH",
    -5: "TY_ERR_NEGENERGY", -6: "TY_ERR_NANDT", -7: "TY_ERR_STATE", -8: "TY_ERR_UNSUPPORTED",
    -9: "TY_ERR_LSQ",
}


class TyphonError(RuntimeError):
    """A non-zero status returned by the library."""

    def __init__(self, status, where, detail):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} ({detail})")


class MeshDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("ncell_int", C.c_int32), ("ncell", C.c_int32),
        ("nface_int", C.c_int32), ("nface", C.c_int32),
        ("facecell", C.c_void_p), ("face_normal", C.c_void_p), ("face_surface", C.c_void_p),
        ("face_centre", C.c_void_p), ("cell_centre", C.c_void_p), ("cell_volume", C.c_void_p),
        ("face_color", C.c_void_p), ("face_bc", C.c_void_p), ("face_partner", C.c_void_p),
        ("face_wallvel", C.c_void_p),
    ]


class SpatParams(C.Structure):
    _fields_ = [
        ("scheme", C.c_int32), ("highres", C.c_int32), ("limiter", C.c_int32),
        ("postlim", C.c_int32), ("gradmeth", C.c_int32), ("mode", C.c_int32),
        ("gamma", C.c_double), ("entropy_fix", C.c_double),
        ("viscous", C.c_int32), ("visc_law", C.c_int32), ("visc_kin", C.c_double), ("rgas", C.c_double),
        ("prandtl", C.c_double), ("farfield", C.c_double * 5),
    ]


_lib = None

class ImpParams(C.Structure):
    """ty_imp_params"""
    _fields_ = [("krylov", C.c_int32), ("precision", C.c_int32), ("nkrylov", C.c_int32), ("max_it", C.c_int32),
                ("local_dt", C.c_int32), ("scaling", C.c_int32), ("inv_res", C.c_double), ("cfl", C.c_double)]


class ImpStats(C.Structure):
    """ty_imp_stats"""
    _fields_ = [("info", C.c_int32), ("restarts", C.c_int32), ("matvecs", C.c_int32), ("reserved", C.c_int32),
                ("dt_min", C.c_double), ("res_l2", C.c_double * 5), ("du_l1", C.c_double * 5),
                ("lin_res", C.c_double), ("du_mom", C.c_double)]


class KdifParams(C.Structure):
    """ty_kdif_params"""
    _fields_ = [("flux", C.c_int32), ("reserved", C.c_int32), ("heat_capacity", C.c_double)]


class KdifSolve(C.Structure):
    """ty_kdif_solve"""
    _fields_ = [("solver", C.c_int32), ("max_it", C.c_int32), ("tol", C.c_double), ("inner_tol", C.c_double)]


class KdifStats(C.Structure):
    """ty_kdif_stats"""
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("rel_res", C.c_double),
                ("du_l1", C.c_double)]


_SIGS = {
    "ty_version": ([], C.c_char_p),
    "ty_error_string": ([C.c_int], C.c_char_p),
    "ty_last_error": ([], C.c_char_p),
    "ty_mesh_create": ([C.POINTER(MeshDesc), C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "ty_mesh_destroy": ([C.c_void_p], C.c_int),
    "ty_mesh_info": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_set_params": ([C.c_void_p, C.POINTER(SpatParams)], C.c_int),
    "ty_state_upload": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_state_download": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_state_upload_device": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_state_download_device": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_prim_download": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_timestep": ([C.c_void_p, C.c_double, C.POINTER(C.c_double)], C.c_int),
    "ty_residual": ([C.c_void_p, C.c_double, C.c_void_p], C.c_int),
    "ty_rk_step": ([C.c_void_p, C.c_int32, C.c_double], C.c_int),
    "ty_rk_steps": ([C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_double)], C.c_int),
    "ty_steady_iteration": ([C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_double), C.c_void_p],
                            C.c_int),
    "ty_debug_get": ([C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_ghost_state_set": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_ghost_prim_download": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_debug_fastmath": ([C.c_int32, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "ty_set_bc_data": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_mesh_set_face_rotation": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_synchronize": ([C.c_void_p], C.c_int),
    "ty_set_stream": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_profile_enable": ([C.c_void_p, C.c_int32], C.c_int),
    "ty_profile_read": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "ty_timestep_static": ([C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                            C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "ty_implicit_step": ([C.c_void_p, C.POINTER(ImpParams), C.POINTER(ImpStats)], C.c_int),
    "ty_implicit_get": ([C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_implicit_matvec": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_kdif_setup": ([C.c_void_p, C.POINTER(KdifParams), C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_kdif_set_temperature": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_kdif_get_temperature": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_kdif_residual": ([C.c_void_p, C.c_double, C.c_void_p], C.c_int),
    "ty_kdif_implicit_step": ([C.c_void_p, C.c_double, C.POINTER(KdifSolve), C.POINTER(KdifStats)], C.c_int),
    "ty_kdif_fourier_dt": ([C.c_void_p, C.c_double, C.POINTER(C.c_double)], C.c_int),
    "ty_kdif_get": ([C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_kdif_matvec": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_residual_device": ([C.c_void_p, C.c_double, C.c_void_p], C.c_int),
    "ty_adjoint_vjp": ([C.c_void_p, C.c_double, C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_new": ([C.POINTER(C.c_void_p)], C.c_int),
    "ty_umesh_free": ([C.c_void_p], C.c_int),
    "ty_umesh_set_nodes": ([C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_umesh_add_section": ([C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_add_mark": ([C.c_void_p, C.c_char_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_umesh_add_vertex_mark": ([C.c_void_p, C.c_char_p, C.c_int32, C.c_void_p], C.c_int),
    "ty_umesh_face_family": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_set_rotation": ([C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_double], C.c_int),
    "ty_umesh_face_rotation": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_add_bc": ([C.c_void_p, C.c_char_p, C.c_int32, C.c_char_p, C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_build": ([C.c_void_p, C.c_int32], C.c_int),
    "ty_umesh_desc": ([C.c_void_p, C.POINTER(MeshDesc)], C.c_int),
    "ty_umesh_facevtex": ([C.c_void_p, C.c_void_p], C.c_int),
    "ty_umesh_rcm_order": ([C.c_void_p, C.c_void_p], C.c_int),
}


KERNEL_NAMES = ["prim", "ghost_prim", "grad", "ghost_grad", "face_states", "barth", "face_flux",
                "face_flux_lim", "rk_update", "gather", "timestep", "cell_fast", "face_flux_fast",
                "imp_face", "imp_diag", "imp_matvec", "imp_precond", "imp_ortho"]


def exported_names():
    return list(_SIGS)


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status, where):
    if status != TY_OK:
        detail = lib().ty_last_error().decode(errors="replace")
        raise TyphonError(status, where, detail)
    return status
