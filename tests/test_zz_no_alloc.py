"""ty_timestep_static: the stability time step for callers that cannot let the library
allocate device memory (a host code that owns all device memory through its own
allocator, or a solver loop that must not allocate between steps).

The entry point takes caller-owned device arrays and keeps its scratch in a static device
array of the library.  These tests call it through the C ABI with device buffers owned by
PyTorch and compare it with ty_timestep on the same state, on two calls in a row: bit for
bit against the exact mode (same operations, same order) and within the fast-mode
tolerance of the test suite (1e-12 relative) against the fast mode.  The file is named to
be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FAST_RTOL = 1e-12


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300 as ty
    from typhon_gb300 import _capi, cases
    md = cases.make_mesh("tgv3d", 8)
    prim = cases.taylor_green(md.cell_centre)
    return torch, ty, _capi, md, prim


def sum_surface_colour_order(md):
    """Sum of face surfaces of each interior cell, accumulated in colour order (as the library
    and Typhon's calc_ns_timestep do)."""
    nci = md.ncell_int
    fc1, fc2, col, S = md.fc1, md.fc2, md.face_color, md.face_surface
    out = np.zeros(nci)
    for colour in range(int(col.max()) + 1):
        f = np.where(col == colour)[0]
        a = fc1[f]
        out[a] = out[a] + S[f]          # one face per colour per cell: no repeated index
        b = fc2[f]
        keep = b < nci
        out[b[keep]] = out[b[keep]] + S[f[keep]]
    return out


def static_dt(torch, _capi, cons_dev, vol_dev, sums_dev, nci, cfl, stream=None):
    dt = C.c_double()
    st = stream.cuda_stream if stream is not None else None
    rc = _capi.lib().ty_timestep_static(nci, cons_dev.data_ptr(), nci, vol_dev.data_ptr(), sums_dev.data_ptr(),
                                        1.4, cfl, st, C.byref(dt))
    return rc, dt.value


def test_static_timestep_matches_ty_timestep_twice(env):
    torch, ty, _capi, md, prim = env
    nci = md.ncell_int
    g = ty.Grid(md)
    g.set_spat("ROE", "MUSCL-UNS", "NONE", "BARTH", mode="exact")
    g.set_prim(prim)
    vol = torch.tensor(md.cell_volume[:nci], dtype=torch.float64, device="cuda")
    sums = torch.tensor(sum_surface_colour_order(md), dtype=torch.float64, device="cuda")
    cons = torch.empty((5, nci), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    for call in range(2):                       # two calls in a row, on two different states
        g.get_cons_device(cons.data_ptr())
        g.synchronize()
        ref_exact = g.calc_zonetimestep(0.8)
        rc, dt = static_dt(torch, _capi, cons, vol, sums, nci, 0.8, stream)
        assert rc == 0, _capi.lib().ty_last_error()
        assert dt == ref_exact, (call, dt, ref_exact)
        g.set_spat("ROE", "MUSCL-UNS", "NONE", "BARTH", mode="fast")
        ref_fast = g.calc_zonetimestep(0.8)
        assert abs(dt - ref_fast) <= FAST_RTOL * ref_fast
        g.set_spat("ROE", "MUSCL-UNS", "NONE", "BARTH", mode="exact")
        g.treelevel_rungekutta("RK3-SSP", ref_exact)   # next call sees a new state
    g.close()


def test_static_timestep_errors_and_recovery(env):
    torch, ty, _capi, md, prim = env
    nci = md.ncell_int
    cons = torch.tensor(ty.prim_to_cons(prim[:, :nci]), dtype=torch.float64, device="cuda").contiguous()
    vol = torch.tensor(md.cell_volume[:nci], dtype=torch.float64, device="cuda")
    sums = torch.tensor(sum_surface_colour_order(md), dtype=torch.float64, device="cuda")
    bad = cons.clone()
    bad[1, 7] = -1.0                            # negative total energy in cell 7
    rc, _ = static_dt(torch, _capi, bad, vol, sums, nci, 0.8)
    assert rc == -5 and "cell 7" in _capi.lib().ty_last_error().decode()
    rc, dt = static_dt(torch, _capi, cons, vol, sums, nci, 0.8)   # the error word was cleared
    assert rc == 0 and dt > 0
    # sizes beyond the static scratch are refused before anything is launched
    big = 256 * 16384 + 1
    dtv = C.c_double()
    rc = _capi.lib().ty_timestep_static(big, cons.data_ptr(), big, vol.data_ptr(), sums.data_ptr(), 1.4, 0.8,
                                        None, C.byref(dtv))
    assert rc == -1 and "static scratch limit" in _capi.lib().ty_last_error().decode()


def test_static_timestep_allocates_nothing(env):
    """After a first call has loaded the library's module in this context, further calls
    leave the GPU's free memory and PyTorch's allocator statistics unchanged."""
    torch, ty, _capi, md, prim = env
    nci = md.ncell_int
    cons = torch.tensor(ty.prim_to_cons(prim[:, :nci]), dtype=torch.float64, device="cuda").contiguous()
    vol = torch.tensor(md.cell_volume[:nci], dtype=torch.float64, device="cuda")
    sums = torch.tensor(sum_surface_colour_order(md), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    rc, dt0 = static_dt(torch, _capi, cons, vol, sums, nci, 0.8, stream)      # warm-up call
    assert rc == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    for _ in range(3):
        rc, dt = static_dt(torch, _capi, cons, vol, sums, nci, 0.8, stream)
        assert rc == 0 and dt == dt0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == reserved0
