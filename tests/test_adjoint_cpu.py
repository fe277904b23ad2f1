"""Binomial checkpointing and the complex-step reference, without a GPU."""
import numpy as np
import pytest

import residual_cs as cs
from typhon_gb300 import adjoint


class ToyStepper:
    """U' = U + dt sin(U) elementwise; its adjoint needs the right U."""

    def __init__(self):
        self.steps = 0

    def step(self, U, dt, tape=None):
        self.steps += 1
        if tape is not None:
            tape.append([U])
        return U + dt * np.sin(U)

    def step_adjoint(self, U, dt, lam, Us=None):
        if Us is not None:
            U = Us[0]
        return lam * (1.0 + dt * np.cos(U))


def test_stored_stage_sweep_equals_checkpointed():
    rng = np.random.default_rng(11)
    n = 30
    dts = list(rng.uniform(0.01, 0.1, n))
    U0, lam = rng.standard_normal(8), rng.standard_normal(8)
    st = ToyStepper()
    Uf, tape = adjoint.forward_steps_stored(st, U0, dts)
    assert len(tape) == n and st.steps == n
    got = adjoint.adjoint_steps_stored(st, dts, lam, tape)
    assert st.steps == n                                 # the reverse sweep recomputes nothing
    ref = adjoint.adjoint_steps(ToyStepper(), U0, dts, lam, 4)
    assert np.array_equal(got, ref)
    assert np.array_equal(Uf, adjoint.forward_steps(ToyStepper(), U0, dts))


def test_storage_plan():
    nci, stages = 1000, 3
    state = 5 * nci * 8
    assert adjoint.plan_storage(nci, stages, 100, budget_bytes=100 * stages * state) == "stages"
    assert adjoint.plan_storage(nci, stages, 100, budget_bytes=100 * stages * state - 1) == 100
    assert adjoint.plan_storage(nci, stages, 100, budget_bytes=20 * state + 5) == 20
    assert adjoint.plan_storage(nci, stages, 100, budget_bytes=0) == 1


def test_hand_written_flux_derivatives_match_dual_numbers(tmp_path):
    """The reverse-mode flux derivatives of the adjoint kernels against forward-mode dual
    numbers through the same flux templates, compiled for the host."""
    import shutil
    import subprocess
    from pathlib import Path
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = Path(__file__).with_name("adjoint_flux_check.cpp")
    exe = tmp_path / "adjoint_flux_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = {ln.split()[0]: ln.split()[1:] for ln in out if ln.strip()}
    assert set(rows) == {"RUSANOV", "HLLC", "ROE"}
    for name, (ncase, err, *hits) in rows.items():
        assert int(ncase) > 0 and float(err) < 1e-12, (name, err)
        covered = [int(h) for h in hits]
        # every branch of the flux is taken: both Rusanov wave speeds; HLLC supersonic left,
        # right and star; Roe with and without the entropy fix
        want = 3 if name == "HLLC" else 2
        assert all(c > 0 for c in covered[:want]), (name, covered)


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
    for scheme, osch in (("RUSANOV", op.SCH_RUSANOV), ("HLLC", op.SCH_HLLC), ("ROE", op.SCH_ROE)):
        s = op.Solver(om, osch, cfl=1.0)
        s.set_prim(prim)
        s.rhs(1e-3)
        U = s.get("cons")[:, :md.ncell_int]
        R = cs.residual(md, U, 1e-3, scheme)
        Ro = s.get("residu")[:, :md.ncell_int]
        assert np.allclose(R, Ro, rtol=1e-12, atol=1e-14 * np.abs(Ro).max())


@pytest.mark.parametrize("scheme,oscheme", [("HLLC", 1), ("ROE", 3), ("RUSANOV", 2)])
@pytest.mark.parametrize("limiter", ["ALBADA", "NONE"])
@pytest.mark.parametrize("highres,postlim", [("MUSCL", "NONE"), ("MUSCL-UNS", "NONE"), ("MUSCL-UNS", "BARTH"),
                                             ("MUSCL", "SUPERBARTH")])
def test_complex_step_reference_matches_muscl_residual(scheme, oscheme, limiter, highres, postlim):
    """The second-order restatement (least-squares gradients, MUSCL or MUSCL-UNS, van Albada,
    Barth post-limiters) against the oracle's residual on a jittered periodic mesh."""
    import oracle_py as op
    import typhon_gb300 as ty
    raw = ty.gen_grid2d(10, 10, 1.0, 1.0, "tri", jitter=0.1, seed=3)
    md = ty.preprocess(raw, 2, op.PERIODIC_UNIT_SQUARE)
    om = op.Mesh.from_raw(raw).build(2, op.PERIODIC_UNIT_SQUARE)
    x, y = md.cell_centre[:, 0], md.cell_centre[:, 1]
    prim = np.stack([1 + 0.1 * np.sin(6.28 * x + 0.3) * np.sin(6.28 * y + 1.1), 0.7 + 0.05 * np.cos(6.28 * (x + y)),
                     0.3 + 0.1 * np.sin(6.28 * y), 0.1 * np.cos(6.28 * x), 0 * x])
    olim = op.LIM_ALBADA if limiter == "ALBADA" else op.LIM_NONE
    ohres = {"MUSCL": op.HRES_MUSCL, "MUSCL-UNS": op.HRES_MUSCLUNS}[highres]
    opost = {"NONE": op.POSTLIM_NONE, "BARTH": op.POSTLIM_BARTH, "SUPERBARTH": op.POSTLIM_SUPERBARTH}[postlim]
    s = op.Solver(om, oscheme, ohres, olim, opost, op.GRAD_LSQ, cfl=1.0)
    s.set_prim(prim)
    s.rhs(1e-3)
    U = s.get("cons")[:, :md.ncell_int]
    R = cs.residual(md, U, 1e-3, scheme, highres=highres, limiter=limiter, postlim=postlim)
    if postlim != "NONE":   # the limiter is active somewhere on this state
        assert (s.get("limratio")[:, :md.ncell_int] < 1.0).any()
    Ro = s.get("residu")[:, :md.ncell_int]
    assert np.abs(R - Ro).max() <= 1e-12 * np.abs(Ro).max()
