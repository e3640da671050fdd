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


def fd_check(obj, A, g, samples, h_small=1e-6, h_large=1e-4):
    """Per-sample central differences of `obj` against the adjoint gradient g.

    h_large = 1e-4: truncation (h^2) and round-off stay far below 1e-7 of each
    sample, so that is the bound.  h_small = 1e-6: the quotient carries the
    round-off of two full propagations (about 1e-15 absolute in L, so ~1e-9 in
    the quotient), which exceeds 1e-6 of the smaller samples; its size is
    estimated per sample from the larger spread between the quotient at h
    and those at 1.25 h and 0.8 h (independent round-off, negligible
    truncation), and the bound is 1e-6 |fd| + 3 x that spread.  Returns the
    per-sample table."""
    rows = []
    for n in samples:
        q = {}
        for h in (h_large, h_small, 1.25 * h_small, 0.8 * h_small):
            Ap, Am = A.copy(), A.copy()
            Ap[n] += h
            Am[n] -= h
            q[h] = (obj(Ap) - obj(Am)) / (2 * h)
        spread = max(abs(q[h_small] - q[1.25 * h_small]), abs(q[h_small] - q[0.8 * h_small]))
        rows.append((int(n), g[n], q[h_large], q[h_small], spread))
    print("  n        g              fd(1e-4) rel     fd(1e-6) rel     round-off bound (rel)")
    for n, gn, fl, fs, sp in rows:
        print(f"  {n:5d}  {gn: .6e}  {abs(gn - fl) / abs(fl):.2e}         {abs(gn - fs) / abs(fs):.2e}"
              f"         {3 * sp / abs(fs):.2e}")
    for n, gn, fl, fs, sp in rows:
        assert abs(gn - fl) <= 1e-7 * abs(fl) + 1e-14, (n, gn, fl)
        assert abs(gn - fs) <= 1e-6 * abs(fs) + 3 * sp + 1e-14, (n, gn, fs, sp)
    return rows


@pytest.mark.parametrize("objective", ["energy", "current"])
def test_adjoint_finite_differences_gpu(built_lib, objective):
    """Central differences of the GPU objective on random samples, per sample."""
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
        L, g, _ = ctx.adjoint(A, dt, objective, ckpt_every=5)

        def obj(Ax):
            ctx.set_orbitals(u0)
            return ctx.adjoint(Ax, dt, objective, ckpt_every=nt)[0]

        fd_check(obj, A, g, rng.choice(nt, size=6, replace=False))


def test_adjoint_finite_differences_differentiation_shape(built_lib):
    """The differentiation workload's shape (a = 10, one ion of charge 2 at a/2,
    NG = 128, NK = 16, NB = NBocc = 2, dt = 2.5e-3, control = the A0 = 0.05,
    w = 0.057, T = 100 pulse plus N(0, 1e-3) noise, seed 2), truncated to 400
    steps: the absorbed-energy gradient against central differences on 12
    random samples, per sample (fd_check)."""
    from mattohf_gb300 import Context, RunConfig, aave_from_samples, define_afield
    nt = 400
    cfg = RunConfig.from_pulse(0.05, 0.057, 100.0, acell=10.0, NG=128, NK=16, NB=2, NBocc=2, Zeff=[2.0],
                               alpha=[1.0], Rion=[0.5], Kion=[1], dt=2.5e-3, NT=nt)
    rng = np.random.default_rng(2)
    A = define_afield(cfg)[1] + 1e-3 * rng.standard_normal(nt)
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        ctx.GS_calculation(5, 4)
        u0 = ctx.get_orbitals()
        E0 = ctx.observables(0.0)["Etot"]
        L, g, _ = ctx.adjoint(A, cfg.dt, "energy", ckpt_every=100)

        def obj(Ax):          # the plain forward: Etot(u_nt, A[nt-1]) - Etot(u_0, 0)
            ctx.set_orbitals(u0)
            E, _, _ = ctx.rk4_run(Ax, aave_from_samples(Ax), cfg.dt)
            return E[-1] - E0

        assert abs(obj(A) - L) <= 1e-12 * max(1.0, abs(L))
        fd_check(obj, A, g, rng.choice(nt, size=12, replace=False))


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


def test_ion_parameter_gradients(built_lib):
    """dL/d(Zeff, alpha) per species and dL/dRion per ion of the absorbed energy
    (the adjoint's dL/dvion carried through the ion potential and its max
    shift, src/Prep_periodic_ion_potential.f90:10-20) against the oracle's chain
    rule on the same dL/dvion (1e-12), and against central differences of the
    plain forward objective with the ion potential rebuilt for each perturbed
    parameter: h = 1e-5, bound 1e-6 relative plus three times the larger
    spread between the quotient at h and those at 1.25 h and 0.8 h (the
    quotient's own round-off and truncation; it matters for the small
    components, e.g. dL/dRion of the weaker ion)."""
    from mattohf_gb300 import Context, RunConfig, aave_from_samples
    from oracle import mattohf_oracle as O
    from conftest import to_oracle_config
    import dataclasses
    cfg = RunConfig(acell=10.0, NG=128, NK=8, NB=2, NBocc=2, Zeff=[1.5, 0.5], alpha=[1.0, 1.0],
                    Rion=[0.25, 0.75], Kion=[1, 2])
    nt, dt = 60, 2.5e-3
    rng = np.random.default_rng(12)
    A = 0.05 * np.sin(0.05 * np.arange(1, nt + 1)) + 1e-3 * rng.standard_normal(nt)
    ocfg = to_oracle_config(cfg)
    rx = np.arange(cfg.NG) / cfg.NG * cfg.acell
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u0 = ctx.get_orbitals()
        L, g, gv = ctx.adjoint(A, dt, "energy", ckpt_every=0)
        grad = ctx.ion_param_grad(gv)
        dZ, da, dR = O.ion_param_grad(ocfg, rx, gv)
        for k, ref in (("Zeff", dZ), ("alpha", da), ("Rion", dR)):
            assert np.max(np.abs(grad[k] - ref)) <= 1e-12 * np.max(np.abs(ref)), k
        vion0 = ctx.vion

        def obj(**kw):
            ctx.vion = O.ion_potential(dataclasses.replace(ocfg, **kw), rx)
            ctx.set_orbitals(u0)
            E0 = ctx.observables(0.0)["Etot"]
            E, _, _ = ctx.rk4_run(A, aave_from_samples(A), dt)
            return E[-1] - E0

        h0 = 1e-5
        rows = []
        for name in ("Zeff", "alpha", "Rion"):
            for i in range(len(getattr(cfg, name))):
                q = []
                for h in (h0, 1.25 * h0, 0.8 * h0):
                    p, m = list(getattr(cfg, name)), list(getattr(cfg, name))
                    p[i] += h
                    m[i] -= h
                    q.append((obj(**{name: p}) - obj(**{name: m})) / (2 * h))
                spread = max(abs(q[0] - q[1]), abs(q[0] - q[2]))
                rows.append((name, i, grad[name][i], q[0], spread))
        ctx.vion = vion0
    for name, i, gn, fd, sp in rows:
        print(f"  dL/d{name}[{i}] = {gn: .10e}   central difference {fd: .10e}   rel {abs(gn - fd) / abs(fd):.1e}"
              f"   spread bound (rel) {3 * sp / abs(fd):.1e}")
    for name, i, gn, fd, sp in rows:
        assert abs(gn - fd) <= 1e-6 * abs(fd) + 3 * sp, (name, i, gn, fd, sp)
