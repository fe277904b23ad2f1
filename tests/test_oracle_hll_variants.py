"""The oracle's HLLC / HLLE wave-speed variants (Typhon's SCHEME = HLLCB, HLLCK, HLLCKB,
HLLEB, HLLEK, HLLEKB: calc_flux_hllc.f90:64-124, calc_flux_hlle.f90:64-120) on the CPU: every
variant is consistent (a uniform state on a periodic mesh has a zero residual, subsonic and
supersonic), and the beta variants stay close to the plain schemes."""
import numpy as np
import pytest

import oracle_py as op

VARIANTS = [op.SCH_HLLCB, op.SCH_HLLCK, op.SCH_HLLCKB, op.SCH_HLLEB, op.SCH_HLLEK, op.SCH_HLLEKB]


def periodic_mesh():
    import typhon_gb300 as ty
    raw = ty.gen_grid2d(10, 10, 1.0, 1.0, "tri", jitter=0.1, seed=3)
    return op.Mesh.from_raw(raw).build(2, op.PERIODIC_UNIT_SQUARE)


@pytest.mark.parametrize("scheme", VARIANTS)
def test_uniform_state_has_zero_residual(scheme):
    om = periodic_mesh()
    s = op.Solver(om, scheme, cfl=1.0)
    for q in ((1.0, 0.7, 0.3, -0.2, 0.0), (0.5, 2.0, 3.0, 1.0, 0.0)):   # subsonic, supersonic
        s.set_prim(np.tile(np.array(q)[:, None], (1, om.ncell)))
        s.rhs(1e-3)
        R = s.get("residu")[:, :om.ncell_int]
        F = s.get("flux")
        assert np.abs(R).max() <= 1e-13 * np.abs(F).max()


@pytest.mark.parametrize("scheme,plain", [(op.SCH_HLLCB, op.SCH_HLLC), (op.SCH_HLLEB, op.SCH_HLLE)])
def test_beta_variant_changes_only_the_wave_speeds(scheme, plain):
    """On a smooth state the B variants (beta < 1 shrinks the outer estimates vn -+ beta a,
    so the Roe-average speeds decide) give fluxes close to the plain scheme's but not equal."""
    om = periodic_mesh()
    d = om.export()
    x, y = d["ccentre"][:, 0], d["ccentre"][:, 1]
    prim = np.stack([1 + 0.1 * np.sin(6.28 * x), 0.7 + 0.05 * np.cos(6.28 * y), 0.3 + 0 * x, 0.1 + 0 * x, 0 * x])
    out = []
    for sch in (scheme, plain):
        s = op.Solver(om, sch, cfl=1.0)
        s.set_prim(prim)
        s.rhs(1e-3)
        out.append(s.get("flux"))
    diff = np.abs(out[0] - out[1]).max(axis=0)
    assert (diff > 0).any()
    assert np.abs(out[0] - out[1]).max() < 0.1 * np.abs(out[1]).max()
