"""The adjoint gradient behind torch.autograd (the gradient-check harness).

The absorbed energy (or final current) of a short RK4 run is a function of the
sampled vector potential A(t_n) and of the ion potential on the grid.  Its
forward is mattohf_adjoint's objective and its backward the adjoint's
gradients; torch.autograd.gradcheck compares them with central differences of
the plain forward.  torch is used here only as the harness (needs a GB300).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class _Objective(torch.autograd.Function):
    """L(A, vion) with dL/dA and dL/dvion from the discrete adjoint."""

    @staticmethod
    def forward(fctx, A, vion, run):
        ctx, u0, dt, objective = run
        ctx.vion = vion.detach().cpu().numpy()
        ctx.set_orbitals(u0)
        L, gA, gv = ctx.adjoint(A.detach().cpu().numpy(), dt, objective, ckpt_every=3)
        fctx.save_for_backward(torch.from_numpy(np.asarray(gA)), torch.from_numpy(np.asarray(gv)))
        return torch.tensor(L, dtype=torch.float64)

    @staticmethod
    def backward(fctx, gout):
        gA, gv = fctx.saved_tensors
        return gout * gA, gout * gv, None


@pytest.mark.parametrize("objective", ["energy", "current"])
def test_adjoint_gradcheck(built_lib, objective):
    from mattohf_gb300 import Context, RunConfig
    cfg = RunConfig(acell=8.0, NG=32, NK=4, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    nt, dt = 6, 0.004
    rng = np.random.default_rng(7)
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u0 = ctx.get_orbitals()
        vion0 = ctx.vion
        A = torch.tensor(0.05 * np.sin(0.5 * np.arange(nt)) + 1e-3 * rng.standard_normal(nt),
                         dtype=torch.float64, requires_grad=True)
        vion = torch.tensor(vion0, dtype=torch.float64, requires_grad=True)
        run = (ctx, u0, dt, objective)
        f = lambda a, v: _Objective.apply(a, v, run)
        # the analytic gradient flows through torch.autograd
        L = f(A, vion)
        L.backward()
        gA, gv = A.grad.detach().clone(), vion.grad.detach().clone()
        assert torch.isfinite(gA).all() and torch.isfinite(gv).all()
        # central differences of the plain forward, against the adjoint
        scale = max(gA.abs().max().item(), gv.abs().max().item())
        assert torch.autograd.gradcheck(f, (A, vion), eps=1e-6, atol=1e-6 * scale + 1e-10, rtol=1e-4,
                                        raise_exception=True)
        ctx.vion = vion0
