"""Adjoint gradient on the GPU vs the oracle's discrete adjoint and vs finite differences."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cfg(**kw):
    from mattohf_gb300 import RunConfig
    base = dict(acell=8.0, NG=32, NK=4, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    base.update(kw)
    return RunConfig(**base)


SHAPES = {
    "ng32_nk4_nb2": {},
    "ng16_nk3_nb3": dict(NG=16, NK=3, NB=3, NBocc=3),
    "ng128_nk2_nb1": dict(NG=128, NK=2, NB=1, NBocc=1, acell=10.0),
}


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("objective", ["energy", "current"])
@pytest.mark.parametrize("ckpt", [0, 2])
@pytest.mark.parametrize("small", [0, 1])
def test_adjoint_matches_oracle(built_lib, shape, objective, ckpt, small):
    """Both the separate-launch path and the fused forward/reverse stages."""
    from mattohf_gb300 import Context, _capi
    from oracle import mattohf_oracle as O
    from conftest import to_oracle_config
    cfg = _cfg(**SHAPES[shape])
    S = O.make_system(to_oracle_config(cfg))
    u0 = O.gram_schmidt(S, O.init_wf(S))
    rng = np.random.default_rng(4)
    A = 0.05 * rng.standard_normal(5)
    dt = 0.004 * min(1.0, (64.0 / cfg.NG) ** 2)
    Lr, gr, gvr = O.rt_adjoint(S, u0, A, dt, objective)
    with Context(cfg) as ctx:
        ctx.set_option(_capi.OPT_SMALL_STAGES, small)
        ctx.set_orbitals(u0)
        L, g, gv = ctx.adjoint(A, dt, objective, ckpt_every=ckpt)
    assert abs(L - Lr) <= 1e-10 * max(1.0, abs(Lr))
    assert np.max(np.abs(g - gr)) <= 1e-9 * np.max(np.abs(gr))
    assert np.max(np.abs(gv - gvr)) <= 1e-9 * np.max(np.abs(gvr))


def test_adjoint_rejects_unoccupied_bands(built_lib):
    """The adjoint is defined for all bands occupied; NB > NBocc is an argument error."""
    from mattohf_gb300 import Context, MattohfError, _capi
    cfg = _cfg(NG=16, NK=3, NB=3, NBocc=1)
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        with pytest.raises(MattohfError) as ei:
            ctx.adjoint(np.zeros(4), 0.004, "energy")
    assert ei.value.status == _capi.ERR_ARG


def test_adjoint_finite_differences_gpu(built_lib):
    """Central differences (h = 1e-6) of the GPU objective on random samples agree to 1e-6."""
    from mattohf_gb300 import Context
    cfg = _cfg(NG=64, NK=4, NB=2, NBocc=2, acell=10.0)
    rng = np.random.default_rng(5)
    nt = 24
    A = 0.05 * np.sin(0.3 * np.arange(nt)) + 1e-3 * rng.standard_normal(nt)
    dt = 0.004
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u0 = ctx.get_orbitals()
        L, g, _ = ctx.adjoint(A, dt, "energy", ckpt_every=5)

        def obj(Ax):
            ctx.set_orbitals(u0)
            return ctx.adjoint(Ax, dt, "energy", ckpt_every=nt)[0]

        h = 1e-6
        for n in rng.choice(nt, size=6, replace=False):
            Ap, Am = A.copy(), A.copy()
            Ap[n] += h
            Am[n] -= h
            fd = (obj(Ap) - obj(Am)) / (2 * h)
            assert abs(g[n] - fd) <= 1e-6 * np.max(np.abs(g)) + 2e-10, (n, g[n], fd)


@pytest.mark.parametrize("NG,NK,NB", [(16, 3, 2), (32, 5, 1), (64, 4, 2), (128, 8, 2), (256, 3, 3)])
@pytest.mark.parametrize("objective", ["energy", "current"])
def test_fused_reverse_stages_match_separate_launches(built_lib, NG, NK, NB, objective):
    """The fused reverse stage (ordered exchange pairs, one launch per stage) gives
    the gradients of the separate-launch backward step (symmetric exchange) to
    round-off, for every team width of the transforms."""
    from mattohf_gb300 import Context, _capi
    cfg = _cfg(NG=NG, NK=NK, NB=NB, NBocc=NB, acell=9.0)
    rng = np.random.default_rng(6)
    nt = 7
    A = 0.05 * np.sin(0.4 * np.arange(nt)) + 1e-2 * rng.standard_normal(nt)
    dt = 2e-4          # RK4-stable up to NG = 256 at a = 9 (|E_max| dt < 1)
    out = {}
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u0 = ctx.get_orbitals()
        for small in (0, 1):
            for ckpt in (0, 3):
                ctx.set_option(_capi.OPT_SMALL_STAGES, small)
                ctx.set_orbitals(u0)
                out[small, ckpt] = ctx.adjoint(A, dt, objective, ckpt_every=ckpt)
    for ckpt in (0, 3):
        L0, g0, v0 = out[0, ckpt]
        L1, g1, v1 = out[1, ckpt]
        assert np.isfinite(L0) and np.all(np.isfinite(g0))
        assert abs(L1 - L0) <= 1e-12 * max(1.0, abs(L0))
        assert np.max(np.abs(g1 - g0)) <= 1e-11 * np.max(np.abs(g0))
        assert np.max(np.abs(v1 - v0)) <= 1e-11 * np.max(np.abs(v0))
    # the checkpoint modes of the fused path agree bitwise
    assert np.array_equal(out[1, 0][1], out[1, 3][1])
