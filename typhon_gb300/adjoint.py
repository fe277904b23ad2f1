"""Unsteady adjoint of the explicit path: gradients of a functional of the final state with
respect to the initial state, through the library's residual and its vector-Jacobian product.

New: Typhon has no adjoint (its inverse mode differentiates by finite differences,
SOURCE/MAIN/inverse_calc_sensi.f90:62-114).

* One Runge-Kutta step in Butcher form (treelevel_rungekutta.f90:48-113, the tables of
  SOURCE/PARAM/MENU_NUM.f90:368-449): U_1 = U0, U_k = U0 + sum_{s<k} c(k-1, s) R(U_s),
  U' = U0 + sum_s c(n, s) R(U_s), each R a residual dt/V sum(+-F S) at a fixed dt.
* Its adjoint runs the stages backwards: lambda_R_s = c(n, s) lambda' + sum_{k>s} c(k-1, s)
  lambda_k, lambda_s = (dR/dU at U_s)^T lambda_R_s (ty_adjoint_vjp), lambda_U0 = lambda' +
  sum_s lambda_s.  The stage states of a step are recomputed from the step's initial state.
* Storage: when every stage state of the run fits in device memory (5 x ncell_int doubles
  per stage and step; a few GB for hundreds of steps on a million cells) the forward pass
  keeps them and the reverse sweep recomputes nothing.  Otherwise the steps are reversed
  with binomial checkpointing: the schedule minimises the number of recomputed steps for a
  given number of stored states (Griewank's recursion, solved here by dynamic programming).
* ``RKSolve`` is a ``torch.autograd.Function`` over CUDA tensors [5, ncell_int] (rho, rhoE,
  rhou, rhov, rhow), so a functional written in torch differentiates through the solver.

The residual must be inviscid: first order, or least-squares gradients with MUSCL
(HIGHRES = MUSCL) and no limiter or van Albada's, on a periodic mesh (the derivative of the
smooth van Albada limiter is exact; there is no post-limiter).  The time steps are fixed (the
stability time step is not differentiated).
"""
import ctypes as C
from functools import lru_cache

import numpy as np

from . import _capi

# Butcher lower-triangular tables coef(i, j), i = 1..n (MENU_NUM.f90:368-449)
RK_TABLES = {
    "RK2": [[.5], [0., 1.]],
    "RK2-SSP": [[1.], [.5, .5]],
    "RK3-SSP": [[1.], [.25, .25], [1. / 6., 1. / 6., 4. / 6.]],
    "RK4": [[.5], [0., .5], [0., 0., 1.], [1. / 6., 2. / 6., 2. / 6., 1. / 6.]],
    "RK25BB": [[0.1815754863270908], [0., 0.238260222208392], [0., 0., 0.330500707328], [0., 0., 0., 0.5],
               [0., 0., 0., 0., 1.]],
    "RK26BB": [[0.11797990162882], [0., 0.18464696649448], [0., 0., 0.24662360430959],
               [0., 0., 0., 0.33183954253762], [0., 0., 0., 0., 0.5], [0., 0., 0., 0., 0., 1.]],
    "RK12BS": [[1.], [0., 1.]],
    "RK13BS": [[.15], [0., .4], [0., 0., 1.]],
}


class Stepper:
    """Runge-Kutta steps and their adjoints on a Grid, on CUDA tensors [5, ncell_int]."""

    def __init__(self, grid, method):
        import torch
        self.torch = torch
        self.g = grid
        self.lib = grid.lib
        self.table = RK_TABLES[method]
        self.n = len(self.table)
        self.nci = grid.nci
        self.stream = torch.cuda.current_stream()
        # torch's default stream is the legacy default stream (handle 0), which the library
        # takes as "its own stream": name it by cudaStreamLegacy (1) instead
        handle = self.stream.cuda_stream or 1
        _capi.check(self.lib.ty_set_stream(grid.h, C.c_void_p(handle)), "ty_set_stream")

    def _set(self, U):
        _capi.check(self.lib.ty_state_upload_device(self.g.h, C.c_void_p(U.data_ptr())), "ty_state_upload_device")

    def residual(self, U, dt):
        R = self.torch.empty_like(U)
        self._set(U)
        _capi.check(self.lib.ty_residual_device(self.g.h, float(dt), C.c_void_p(R.data_ptr())), "ty_residual_device")
        return R

    def vjp(self, U, dt, lamR):
        lamR = lamR.contiguous()
        out = self.torch.empty_like(U)
        self._set(U)
        _capi.check(self.lib.ty_adjoint_vjp(self.g.h, float(dt), C.c_void_p(lamR.data_ptr()),
                                            C.c_void_p(out.data_ptr())), "ty_adjoint_vjp")
        return out

    def stages(self, U0, dt, last_residual=True):
        """Stage states U_1..U_n and residuals R_1..R_n of one step (R_n only when asked)."""
        Us, Rs = [], []
        for k in range(self.n):
            U = U0.clone()
            for s in range(k):
                c = self.table[k - 1][s]
                if c != 0.0:
                    U.add_(Rs[s], alpha=c)
            Us.append(U)
            if k < self.n - 1 or last_residual:
                Rs.append(self.residual(U, dt))
        return Us, Rs

    def step(self, U0, dt, tape=None):
        """U0 -> U' (one step); the step's stage states are appended to `tape` when given."""
        Us, Rs = self.stages(U0, dt)
        U = U0.clone()
        for s, c in enumerate(self.table[-1]):
            if c != 0.0:
                U.add_(Rs[s], alpha=c)
        if tape is not None:
            tape.append(Us)
        return U

    def step_adjoint(self, U0, dt, lam, Us=None):
        """lambda' -> lambda_U0 for one step; the stage states are recomputed from U0 unless
        given (Us, as stored by step(..., tape))."""
        if Us is None:
            Us, _ = self.stages(U0, dt, last_residual=False)
        lam_stage = [None] * self.n
        out = lam.clone()
        for s in reversed(range(self.n)):
            lr = lam * self.table[-1][s]
            for k in range(s + 1, self.n):
                c = self.table[k - 1][s]
                if c != 0.0:
                    lr.add_(lam_stage[k], alpha=c)
            lam_stage[s] = self.vjp(Us[s], dt, lr)
            out.add_(lam_stage[s])
        return out


@lru_cache(maxsize=None)
def _cost_table(nsteps, snaps):
    """cost[l][s]: fewest forward steps to reverse l steps with s free snapshots (the range's
    first state is held); split[l][s]: where to place the next snapshot."""
    inf = np.iinfo(np.int64).max // 4
    cost = np.zeros((nsteps + 1, snaps + 1), np.int64)
    split = np.zeros((nsteps + 1, snaps + 1), np.int64)
    ls = np.arange(nsteps + 1)
    cost[:, 0] = ls * (ls - 1) // 2
    for s in range(1, snaps + 1):
        for l in range(2, nsteps + 1):
            m = np.arange(1, l)
            c = m + cost[l - m, s - 1] + cost[m, s]
            j = int(np.argmin(c))
            cost[l, s] = c[j] if c[j] < inf else inf
            split[l, s] = m[j]
    return cost, split


def checkpoint_cost(nsteps, snaps):
    """Forward steps recomputed when reversing nsteps steps with `snaps` stored states."""
    return int(_cost_table(nsteps, snaps)[0][nsteps, snaps]) if nsteps > 0 else 0


def forward_steps(stepper, U0, dts):
    U = U0
    for dt in dts:
        U = stepper.step(U, dt)
    return U


def forward_steps_stored(stepper, U0, dts):
    """Forward steps that keep every stage state: (U_final, tape), tape[i] the stage states of
    step i.  n_stages x 5 x ncell_int doubles per step of device memory."""
    tape = []
    U = U0
    for dt in dts:
        U = stepper.step(U, dt, tape)
    return U, tape


def adjoint_steps_stored(stepper, dts, lam, tape):
    """dJ/dU0 from the stage states stored by forward_steps_stored: one reverse sweep, no
    recomputation."""
    for i in reversed(range(len(dts))):
        lam = stepper.step_adjoint(None, dts[i], lam, Us=tape[i])
    return lam


def plan_storage(nci, nstages, nsteps, budget_bytes=None):
    """Storage policy of the reverse sweep: "stages" when every stage state of the run fits in
    `budget_bytes` (default: half of the device's free memory), else the number of stored
    states (binomial checkpointing) that fit, at least 1."""
    state = 5 * nci * 8
    if budget_bytes is None:
        import torch
        free, _ = torch.cuda.mem_get_info()
        budget_bytes = free // 2
    if nsteps * nstages * state <= budget_bytes:
        return "stages"
    return int(max(1, min(nsteps, budget_bytes // state)))


def adjoint_steps(stepper, U0, dts, lam, snaps=20):
    """dJ/dU0 given lam = dJ/dU_final: the steps reversed from U0 with at most `snaps` states
    held besides U0, placed by the binomial schedule (stepper: step(U, dt) and
    step_adjoint(U, dt, lam))."""
    n = len(dts)
    if n == 0:
        return lam
    snaps = min(snaps, n)
    _, split = _cost_table(n, snaps)

    def run(U, a, b):
        for k in range(a, b):
            U = stepper.step(U, dts[k])
        return U

    def rev(a, b, Ua, s, lam):
        if b - a == 1:
            return stepper.step_adjoint(Ua, dts[a], lam)
        if s == 0:
            for i in reversed(range(a, b)):
                lam = stepper.step_adjoint(run(Ua, a, i), dts[i], lam)
            return lam
        m = a + int(split[b - a, s])
        lam = rev(m, b, run(Ua, a, m), s - 1, lam)
        return rev(a, m, Ua, s, lam)

    return rev(0, n, U0, snaps, lam)


def _make_function():
    import torch

    class RKSolve(torch.autograd.Function):
        """U_final = RKSolve.apply(U0, grid, method, dts, snaps): explicit steps at fixed dts,
        differentiable with respect to U0 (a CUDA float64 tensor [5, ncell_int]).  With snaps
        "stages" the forward pass keeps every stage state and the backward pass recomputes
        nothing; with a number it stores that many states and reverses by binomial
        checkpointing."""

        @staticmethod
        def forward(ctx, U0, grid, method, dts, snaps=None):
            st = Stepper(grid, method)
            dts = list(dts)
            if snaps is None:
                snaps = plan_storage(st.nci, st.n, len(dts))
            ctx.st, ctx.dts, ctx.snaps, ctx.tape = st, dts, snaps, None
            ctx.save_for_backward(U0)
            with torch.no_grad():
                if snaps == "stages":
                    U, ctx.tape = forward_steps_stored(st, U0.contiguous(), dts)
                    return U
                return forward_steps(st, U0.contiguous(), dts)

        @staticmethod
        def backward(ctx, lam):
            (U0,) = ctx.saved_tensors
            with torch.no_grad():
                if ctx.tape is not None:
                    g = adjoint_steps_stored(ctx.st, ctx.dts, lam.contiguous(), ctx.tape)
                    ctx.tape = None
                else:
                    g = adjoint_steps(ctx.st, U0.contiguous(), ctx.dts, lam.contiguous(), ctx.snaps)
            return g, None, None, None, None

    return RKSolve


_RKSolve = None


def rk_solve(U0, grid, method, dts, snaps=None):
    """Differentiable explicit solve (see RKSolve).  snaps: "stages" (keep every stage state),
    a number of stored states (binomial checkpointing), or None (the policy of plan_storage)."""
    global _RKSolve
    if _RKSolve is None:
        _RKSolve = _make_function()
    return _RKSolve.apply(U0, grid, method, list(dts), snaps)
