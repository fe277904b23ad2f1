"""Binomial checkpointing and the complex-step reference, without a GPU."""
import numpy as np
import pytest

import residual_cs as cs
from typhon_gb300 import adjoint


class ToyStepper:
    """U' = U + dt sin(U) elementwise; its adjoint needs the right U."""

    def __init__(self):
        self.steps = 0

    def step(self, U, dt):
        self.steps += 1
        return U + dt * np.sin(U)

    def step_adjoint(self, U, dt, lam):
        return lam * (1.0 + dt * np.cos(U))


@pytest.mark.parametrize("n,snaps", [(1, 0), (7, 0), (20, 1), (50, 3), (64, 20), (100, 5)])
def test_checkpointed_adjoint_equals_stored_sweep(n, snaps):
    rng = np.random.default_rng(n)
    dts = list(rng.uniform(0.01, 0.1, n))
    U0 = rng.standard_normal(8)
    lam = rng.standard_normal(8)
    states = [U0]
    for dt in dts:
        states.append(states[-1] + dt * np.sin(states[-1]))
    ref = lam
    for i in reversed(range(n)):
        ref = ref * (1.0 + dts[i] * np.cos(states[i]))
    st = ToyStepper()
    got = adjoint.adjoint_steps(st, U0, dts, lam, snaps)
    assert np.allclose(got, ref, rtol=1e-14, atol=0)
    assert st.steps == adjoint.checkpoint_cost(n, min(snaps, n))


def test_checkpoint_cost_bounds():
    for n in (2, 5, 17, 60):
        costs = [adjoint.checkpoint_cost(n, s) for s in range(n)]
        assert costs[0] == n * (n - 1) // 2              # nothing stored: recompute from U0
        assert costs[n - 1] == n - 1                     # every state stored: one sweep
        assert all(a >= b for a, b in zip(costs, costs[1:]))
    # 20 snapshots over 500 steps: a few sweeps, not the quadratic count
    assert adjoint.checkpoint_cost(500, 20) < 3 * 500


def test_complex_step_reference_matches_real_residual(golden_dir):
    import oracle_py as op
    import typhon_gb300 as ty
    md = ty.preprocess(ty.read_tym(golden_dir / "quad10x10.tym"), 2, op.PERIODIC_UNIT_SQUARE)
    om = op.Mesh.from_tym(golden_dir / "quad10x10.tym").build(2, op.PERIODIC_UNIT_SQUARE)
    x, y = md.cell_centre[:, 0], md.cell_centre[:, 1]
    prim = np.stack([1 + 0.1 * np.sin(6.28 * x), 0.7 + 0.05 * np.cos(6.28 * y), 0.3 + 0 * x, 0.1 + 0 * x, 0 * x])
    for scheme, osch in (("RUSANOV", op.SCH_RUSANOV), ("ROE", op.SCH_ROE)):
        s = op.Solver(om, osch, cfl=1.0)
        s.set_prim(prim)
        s.rhs(1e-3)
        U = s.get("cons")[:, :md.ncell_int]
        R = cs.residual(md, U, 1e-3, scheme)
        Ro = s.get("residu")[:, :md.ncell_int]
        assert np.allclose(R, Ro, rtol=1e-12, atol=1e-14 * np.abs(Ro).max())
