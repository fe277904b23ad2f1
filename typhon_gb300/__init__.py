"""typhon_gb300 — GB300-native (sm_103a) residual-and-update path of the Typhon
unstructured finite-volume solver, behind a C ABI (include/typhon_gpu.h)."""
from . import _capi, umesh
from ._capi import TyphonError
from .solver import Grid, prim_to_cons
from .umesh import (BC_FARFIELD, BC_HEAT, BC_INLET_SUB, BC_INLET_SUP, BC_NOSLIP, BC_OUTLET_SUB, BC_OUTLET_SUP,
                    BC_PERIODIC, BC_SYMMETRY, BC_WALL, RawMesh, gen_grid2d, gen_tet_box, periodic_box_bcs, preprocess, read_tym, reorder_rcm, write_tym)

__all__ = ["BC_FARFIELD", "BC_HEAT", "BC_INLET_SUB", "BC_INLET_SUP", "BC_NOSLIP", "BC_OUTLET_SUB", "BC_OUTLET_SUP", "BC_PERIODIC", "BC_SYMMETRY", "BC_WALL", "Grid", "RawMesh", "TyphonError", "gen_grid2d", "gen_tet_box", "periodic_box_bcs", "preprocess", "reorder_rcm",
           "prim_to_cons", "read_tym", "write_tym", "umesh"]
