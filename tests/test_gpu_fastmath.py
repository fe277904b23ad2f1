"""The fast mode's Newton-Raphson reciprocal, reciprocal square root and square root
(typhon_gb300/csrc/fastmath.cuh) against CUDA's IEEE division and square root, through
ty_debug_fastmath: within 2 units in the last place over the whole range of normal positive
doubles, and within 1 unit for most values."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import _capi, build
    build.build()
    return _capi.lib()


def run(lib, which, x):
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    assert lib.ty_debug_fastmath(which, x.size, x.ctypes.data, y.ctypes.data) == 0
    return y


def ulps(a, b):
    """Distance in units in the last place between positive doubles a and b."""
    return np.abs(a.view(np.int64) - b.view(np.int64))


def samples():
    rng = np.random.default_rng(5)
    wide = 10.0 ** rng.uniform(-300, 300, 200_000)      # the range of normal doubles
    flow = 10.0 ** rng.uniform(-4, 4, 200_000)          # densities, pressures, speeds
    edges = np.array([1.0, 2.0, 4.0, 0.5, 0.25, 1.4, 71.4, np.nextafter(1.0, 2), np.nextafter(2.0, 1)])
    return np.concatenate([wide, flow, edges])


@pytest.mark.parametrize("fast,ieee,name", [(0, 3, "1/x"), (1, 4, "1/sqrt(x)"), (2, 5, "sqrt(x)")])
def test_newton_raphson_against_ieee(lib, fast, ieee, name):
    x = samples()
    a, b = run(lib, fast, x), run(lib, ieee, x)
    d = ulps(a, b)
    assert d.max() <= 2, (name, int(d.max()))
    assert np.mean(d == 0) > 0.5, (name, float(np.mean(d == 0)))


def test_square_root_of_zero(lib):
    assert run(lib, 2, np.array([0.0]))[0] == 0.0


def test_seeds_are_approximations(lib):
    """The hardware seeds alone are far from full precision (so the iterations matter), but
    close enough for two Newton-Raphson iterations (relative error below 2^-13)."""
    x = samples()
    for seed, ieee in ((6, 3), (7, 4)):
        rel = np.abs(run(lib, seed, x) / run(lib, ieee, x) - 1.0)
        assert rel.max() < 2.0 ** -13
        assert rel.max() > 2.0 ** -40
