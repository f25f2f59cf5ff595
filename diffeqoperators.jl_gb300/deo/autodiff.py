"""Reverse-mode rules for the stencil apply and for SSP-RK3 method-of-lines
solves.  No reference counterpart (the reference's `adjoint(L)` returns L
itself, abstract_operator_functions.jl:130-135, which is not the transpose of
an N x (N+2) operator).

rrule(A, u) mirrors ChainRulesCore.rrule(*, A::GhostDerivativeOperator, u):
it returns y = A*u and a pullback ybar -> (NoTangent, NoTangent, A_l^T ybar),
where (A_l, A_b) = Array(A) is the affine map's linear part.  The pullback
runs libdeo's adjoint kernel (transposed stencil + transposed ghost fill).
"""
from __future__ import annotations

import math

from .operators import _dtype_code, julia_array, plan_for

NoTangent = None


def rrule(A, u):
    plan = plan_for(A.terms(), tuple(u.shape), _dtype_code(u))
    y = julia_array(tuple(u.shape), u.dtype, u.device)
    plan.apply(u, y)

    def pullback(ybar):
        ubar = julia_array(tuple(u.shape), u.dtype, u.device)
        plan.adjoint(ybar, ubar)
        return NoTangent, NoTangent, ubar

    return y, pullback


def _autograd_fn():
    import torch

    class _Apply(torch.autograd.Function):
        @staticmethod
        def forward(ctx, u, plan):
            ctx.plan = plan
            y = julia_array(tuple(u.shape), u.dtype, u.device)
            plan.apply(u.detach(), y)
            return y

        @staticmethod
        def backward(ctx, g):
            g = _jl(g)
            ub = julia_array(tuple(g.shape), g.dtype, g.device)
            ctx.plan.adjoint(g, ub)
            return ub, None

    return _Apply


_APPLY = None


def apply(A, u):
    """Differentiable y = A*u for torch autograd (backward = adjoint kernel)."""
    global _APPLY
    if _APPLY is None:
        _APPLY = _autograd_fn()
    plan = plan_for(A.terms(), tuple(u.shape), _dtype_code(u))
    return _APPLY.apply(u, plan)


# ---------------------------------------------------------------------------
# SSP-RK3 method-of-lines solves and their adjoint
# ---------------------------------------------------------------------------
def _stage_batches(plan, u, u1, u2, dt):
    """The three Shu-Osher stages as batched-stage launches (one instance)."""
    from .batch import StageBatch
    s1 = StageBatch([dict(plan=plan, c=u, out=u1, gamma=1.0, dt=dt)])
    s2 = StageBatch([dict(plan=plan, a=u, alpha=0.75, c=u1, out=u2, gamma=0.25, dt=dt)])
    s3 = StageBatch([dict(plan=plan, a=u, alpha=1.0 / 3.0, c=u2, out=u, gamma=2.0 / 3.0, dt=dt)])
    return s1, s2, s3


def ssprk3_solve(A, u0, dt: float, nsteps: int, use_graph: bool = True):
    """u(T) after `nsteps` SSP-RK3 steps of du/dt = A*u (A = L*Q terms); u0 is not modified."""
    plan = plan_for(A.terms(), tuple(u0.shape), _dtype_code(u0))
    u = u0.clone()
    u1 = julia_array(tuple(u0.shape), u0.dtype, u0.device)
    u2 = julia_array(tuple(u0.shape), u0.dtype, u0.device)
    stages = _stage_batches(plan, u, u1, u2, dt)
    for _ in range(nsteps):
        for s in stages:
            s.run(use_graph)
    return u


def _adjoint_stage_batches(plan, ub, g1, g2, dt):
    """Transposed stages of one SSP-RK3 step for a linear right-hand side
    F(u) = A_l u + A_b (given ubar of u_{n+1}, produce ubar of u_n in place):
        g2 = (2/3)(ub + dt A_l^T ub)
        g1 = (1/4)(g2 + dt A_l^T g2)
        ub = (1/3) ub + (3/4) g2 + (g1 + dt A_l^T g1)
    """
    from .batch import StageBatch
    a1 = StageBatch([dict(plan=plan, c=ub, out=g2, gamma=2.0 / 3.0, dt=dt, adjoint=True)])
    a2 = StageBatch([dict(plan=plan, c=g2, out=g1, gamma=0.25, dt=dt, adjoint=True)])
    a3 = StageBatch([dict(plan=plan, a=ub, alpha=1.0 / 3.0, b=g2, beta=0.75, c=g1, out=ub, gamma=1.0, dt=dt,
                          adjoint=True)])
    return a1, a2, a3


def ssprk3_grad_norm2(A, u0, dt: float, nsteps: int, checkpoint: str = "none", use_graph: bool = True):
    """(u(T), d||u(T)||^2 / du0) for the SSP-RK3 solve of du/dt = A*u.

    checkpoint = "none": the right-hand side is affine in u, so the transposed
    step needs no forward state; only u(T) is kept.
    checkpoint = "sqrtK": stores ceil(sqrt(K)) states during the forward sweep
    and recomputes each segment during the reverse sweep -- the schedule a
    state-dependent right-hand side needs; its gradient equals "none"'s bit
    for bit here, which the tests check.
    """
    import torch
    plan = plan_for(A.terms(), tuple(u0.shape), _dtype_code(u0))
    shape = tuple(u0.shape)
    u = u0.clone()
    u1 = julia_array(shape, u0.dtype, u0.device)
    u2 = julia_array(shape, u0.dtype, u0.device)
    fwd = _stage_batches(plan, u, u1, u2, dt)
    ckpts = {}
    seg = max(1, int(math.ceil(math.sqrt(max(nsteps, 1)))))
    for n in range(nsteps):
        if checkpoint == "sqrtK" and n % seg == 0:
            ckpts[n] = u.clone()
        for s in fwd:
            s.run(use_graph)
    uT = u.clone()
    ub = _jl(2.0 * uT)
    g1 = julia_array(shape, u0.dtype, u0.device)
    g2 = julia_array(shape, u0.dtype, u0.device)
    adj = _adjoint_stage_batches(plan, ub, g1, g2, dt)
    if checkpoint == "sqrtK":
        # reverse over segments: recompute the segment's states from its checkpoint
        starts = sorted(ckpts)
        for s0 in reversed(starts):
            s1 = min(s0 + seg, nsteps)
            states = [ckpts[s0].clone()]
            w = ckpts[s0].clone()
            wf = _stage_batches(plan, w, u1, u2, dt)
            for _ in range(s0, s1 - 1):
                for s in wf:
                    s.run(use_graph)
                states.append(w.clone())
            for _ in reversed(states):  # state-independent transposed step (affine RHS)
                for s in adj:
                    s.run(use_graph)
        del ckpts
    else:
        for _ in range(nsteps):
            for s in adj:
                s.run(use_graph)
    return uT, ub


def _jl(t):
    from .operators import fortran_strides, to_julia_layout
    return t if tuple(t.stride()) == fortran_strides(t.shape) else to_julia_layout(t)
