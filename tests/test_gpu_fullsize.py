"""Size-independent properties at the full workload shapes (needs a GB300).

The oracle is too slow at these sizes, so these tests check properties that
hold at any size:
  * h[u] is Hermitian: <v|h w> = conj(<w|h v>);
  * the symmetric exchange (w == u) equals the general pair kernel;
  * the double-float exchange agrees with FP64;
  * without a field, the RK4 loop conserves the electron number and the energy.
Shapes: NG=256, NK=64, NB=Nocc=4 (the exchange-dominated RT workload) and
NG=512, NK=128, NB=Nocc=8 (the largest single-run shape).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = {
    "ng256_nk64_nb4": dict(acell=10.0, NG=256, NK=64, NB=4, NBocc=4, Zeff=[1.5, 0.5], alpha=[1.0, 1.0],
                           Rion=[0.25, 0.75], Kion=[1, 2]),
    "ng512_nk128_nb8": dict(acell=12.0, NG=512, NK=128, NB=8, NBocc=8, Zeff=[1.0], alpha=[1.0],
                            Rion=[1 / 6, 0.5, 5 / 6], Kion=[1, 1, 1]),
}
_ctx = {}


def ctx_for(name):
    from mattohf_gb300 import Context, RunConfig
    if name not in _ctx:
        c = Context(RunConfig(**SHAPES[name]))
        c.Init_wf()
        c.Gram_Schmidt()
        _ctx[name] = c
    return _ctx[name]


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    yield
    for c in _ctx.values():
        c.close()
    _ctx.clear()


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("name", list(SHAPES))
def test_h_is_hermitian(name):
    ctx = ctx_for(name)
    u = ctx.get_orbitals()
    v = _rand((ctx.NK, 2, ctx.NG), 1)
    w = _rand((ctx.NK, 2, ctx.NG), 2)
    hv = ctx.ubkwbk_hwbk(u, v, 0.07)
    hw = ctx.ubkwbk_hwbk(u, w, 0.07)
    for k in (0, ctx.NK // 3, ctx.NK - 1):          # h is block-diagonal in k
        a = np.conj(v[k]) @ hw[k].T                   # <v_i|h w_j>
        b = np.conj(w[k]) @ hv[k].T                   # <w_j|h v_i>
        scale = np.linalg.norm(v[k]) * np.linalg.norm(hw[k])
        assert np.max(np.abs(a - b.T.conj())) <= 1e-12 * scale


@pytest.mark.parametrize("name", list(SHAPES))
def test_symmetric_exchange_equals_pair_kernel(name):
    from mattohf_gb300 import _capi
    ctx = ctx_for(name)
    u = ctx.get_orbitals() + 0.1 * _rand((ctx.NK, ctx.NB, ctx.NG), 3)   # non-trivial Nyquist content
    sym = ctx.ubkwbk_vFwbk(u, u)
    ctx.set_option(_capi.OPT_SYMMETRIC, 0)
    try:
        gen = ctx.ubkwbk_vFwbk(u, u)
    finally:
        ctx.set_option(_capi.OPT_SYMMETRIC, 1)
    assert np.max(np.abs(sym - gen)) <= 1e-12 * np.max(np.abs(gen))


@pytest.mark.parametrize("name", list(SHAPES))
def test_double_float_exchange_matches_fp64(name):
    from mattohf_gb300 import _capi
    ctx = ctx_for(name)
    u = ctx.get_orbitals()
    ref = ctx.ubkwbk_vFwbk(u, u)
    ctx.set_option(_capi.OPT_FOCK_DF64, 1)
    try:
        got = ctx.ubkwbk_vFwbk(u, u)
    finally:
        ctx.set_option(_capi.OPT_FOCK_DF64, 0)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_field_free_rk4_conserves_charge_and_energy():
    """From a few SCF iterations, no field.

    RK4 multiplies an eigenmode of energy e by R(-i e dt), |R| = 1 - (e dt)^6/72 + ...,
    so it conserves the norm only for e dt << 1.  Here the grid's highest
    kinetic energy is 0.5 (pi NG / a)^2 = 3.2e3 Ha.  At dt = 5e-5 (e dt <= 0.16)
    the charge must hold to 1e-10.  The energy drifts more (measured 7e-9
    relative over 40 steps): the damped grid-scale residue carries up to
    3.2e3 Ha per unit weight, so its bound is 1e-7.  At the workload's dt = 7e-4
    (e dt up to 2.3, still inside the RK4 stability interval 2 sqrt 2), the
    grid-scale residue of the SCF state is damped: the charge may only decrease,
    and by a bounded amount.
    """
    from mattohf_gb300 import Context, RunConfig
    with Context(RunConfig(**SHAPES["ng256_nk64_nb4"])) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        ctx.GS_calculation(5, 4)
        u0 = ctx.get_orbitals()
        E0 = ctx.observables(0.0)
        z = np.zeros(40)
        E, J, N = ctx.rk4_run(z, z, 5e-5)
        ctx.set_orbitals(u0)
        _, _, N7 = ctx.rk4_run(z, z, 7e-4)
    assert np.max(np.abs(N - E0["Nele"])) <= 1e-10 * E0["Nele"]
    assert np.max(np.abs(E - E0["Etot"])) <= 1e-7 * abs(E0["Etot"])
    assert np.all(np.diff(np.concatenate([[E0["Nele"]], N7])) <= 1e-13 * E0["Nele"])
    assert E0["Nele"] - N7[-1] <= 1e-5 * E0["Nele"]
