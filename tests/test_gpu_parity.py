"""CUDA path vs the oracle, through the C ABI (needs a GB300).

Tolerances (all complex128 / FP64):
  * tables, single operator applications: max|gpu-ref| <= 1e-12 * max|ref|
  * RK4 series over a few steps: relative 1e-10 (the parity bound for the RT series)
  * ground state: gauge-invariant quantities only (energies, Ritz values)
"""
from __future__ import annotations

import dataclasses
import json
import os

import numpy as np
import pytest

from conftest import to_oracle_config

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

TOL_OP = 1e-12
TOL_RT = 1e-10


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_cfg(**kw):
    from mattohf_gb300 import RunConfig
    base = dict(acell=10.0, NG=32, NK=4, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5],
                Kion=[1])
    base.update(kw)
    return RunConfig(**base)


CONFIGS = {
    "ng16_nk3_unocc": make_cfg(NG=16, NK=3, NB=3, NBocc=1, acell=8.0, Zeff=[1.5, 0.5],
                               alpha=[1.0, 0.7], Rion=[0.25, 0.75], Kion=[1, 2]),
    "ng32_nk4": make_cfg(),
    "ng64_nk8": make_cfg(NG=64, NK=8),
    "ng128_nk4_nb3": make_cfg(NG=128, NK=4, NB=3, NBocc=2),
    "ng256_nk2": make_cfg(NG=256, NK=2, NB=2, NBocc=2),
    "ng512_nk2": make_cfg(NG=512, NK=2, NB=2, NBocc=1),
    "ng32_nk1": make_cfg(NG=32, NK=1, NB=2, NBocc=2),        # single k-point: one kernel column
    "ng64_nk5_nb4": make_cfg(NG=64, NK=5, NB=4, NBocc=3, acell=7.0),
    # any functional but 'HF' drops the exchange term (src/Functions.f90:85-87, 204-207, 276-278)
    "ng64_nk4_no_exchange": make_cfg(NG=64, NK=4, NB=3, NBocc=2, functional="PZ"),
    "ng64_nk4_nb1": make_cfg(NG=64, NK=4, NB=1, NBocc=1),
}

_cache = {}


def ref_vF(S, u, w):
    """Exchange term of the oracle; without HF the library's exchange entry point returns zeros."""
    from oracle import mattohf_oracle as O
    return O.ubkwbk_vFwbk(S, u, w) if S.hf else np.zeros_like(w)


def setup(name):
    if name in _cache:
        return _cache[name]
    from mattohf_gb300 import Context
    from oracle import mattohf_oracle as O
    cfg = CONFIGS[name]
    ctx = Context(cfg)
    S = O.make_system(to_oracle_config(cfg))
    _cache[name] = (cfg, ctx, S)
    return _cache[name]


def rand_orbs(S, seed, nb=None):
    rng = np.random.default_rng(seed)
    shape = (S.NK, S.NB if nb is None else nb, S.NG)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    yield
    for _, ctx, _ in _cache.values():
        ctx.close()
    _cache.clear()


@pytest.mark.parametrize("name", list(CONFIGS))
def test_tables(name):
    cfg, ctx, S = setup(name)
    g = ctx.grids()
    assert np.array_equal(g["Gx"], S.Gx)
    assert np.array_equal(g["kx"], S.kx)
    assert np.array_equal(g["rx"], S.rx)
    assert rel(ctx.vion, S.vion) <= 1e-14
    vCG, vCq = ctx.coulomb()
    assert rel(vCG, S.vCG) <= TOL_OP
    if S.vCGkk is None:        # the reference builds vCGkk only for HF (src/Initialization.f90:116-141)
        return
    NK = S.NK
    for kr in range(NK):
        for kc in range(NK):
            assert rel(vCq[kr - kc + NK - 1], S.vCGkk[kr * NK + kc]) <= TOL_OP


@pytest.mark.parametrize("name", list(CONFIGS))
def test_hpsi(name):
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup(name)
    u = O.gram_schmidt(S, rand_orbs(S, 1))
    w = rand_orbs(S, 2)
    for A in (0.0, 0.3):
        ref = O.ubkwbk_hwbk(S, u, w, A)
        got = ctx.ubkwbk_hwbk(u, w, A)
        assert rel(got, ref) <= TOL_OP, (A, rel(got, ref))


@pytest.mark.parametrize("name", list(CONFIGS))
@pytest.mark.parametrize("sym", [1, 0])
def test_hpsi_self(name, sym):
    """h[u] u (w == u): symmetric occupied-pair exchange vs the oracle, and vs the plain kernel."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import _capi
    cfg, ctx, S = setup(name)
    u = O.gram_schmidt(S, rand_orbs(S, 11))
    ctx.set_option(_capi.OPT_SYMMETRIC, sym)
    try:
        got = ctx.ubkwbk_hwbk(u, u, 0.17)
        vf = ctx.ubkwbk_vFwbk(u, u)
    finally:
        ctx.set_option(_capi.OPT_SYMMETRIC, 1)
    assert rel(got, O.ubkwbk_hwbk(S, u, u, 0.17)) <= TOL_OP
    assert np.max(np.abs(vf - ref_vF(S, u, u))) <= TOL_OP * max(np.max(np.abs(ref_vF(S, u, u))), 1e-300)


@pytest.mark.parametrize("name", list(CONFIGS))
def test_hpsi_self_double_float(name):
    """Exchange transforms in double-float arithmetic stay within the operator tolerance."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import _capi
    cfg, ctx, S = setup(name)
    u = O.gram_schmidt(S, rand_orbs(S, 13))
    ctx.set_option(_capi.OPT_FOCK_DF64, 1)
    try:
        got = ctx.ubkwbk_hwbk(u, u, 0.07)
        vf = ctx.ubkwbk_vFwbk(u, u)
    finally:
        ctx.set_option(_capi.OPT_FOCK_DF64, 0)
    assert rel(got, O.ubkwbk_hwbk(S, u, u, 0.07)) <= TOL_OP
    assert np.max(np.abs(vf - ref_vF(S, u, u))) <= TOL_OP * max(np.max(np.abs(ref_vF(S, u, u))), 1e-300)


@pytest.mark.parametrize("name", ["ng32_nk4", "ng64_nk8"])
def test_rk4_run_double_float(name):
    """RK4 series with double-float exchange transforms vs the oracle (1e-10)."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import _capi, define_afield
    cfg, ctx, S = setup(name)
    cfg = dataclasses.replace(cfg, dt=0.004, NT=6, field_option="LP", omegac=1.55, Tpulse=0.1, E0=20.0)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    _, A, Aave, _ = define_afield(cfg)
    ctx.set_option(_capi.OPT_FOCK_DF64, 1)
    try:
        ctx.set_orbitals(u0)
        E, J, N = ctx.rk4_run(A, Aave, cfg.dt)
        uf = ctx.get_orbitals()
    finally:
        ctx.set_option(_capi.OPT_FOCK_DF64, 0)
    S.cfg = to_oracle_config(cfg)
    ref = O.rt_calculation(S, u0, nt=cfg.NT, A=A, Aave=Aave)
    assert rel(E, ref.Etot) <= TOL_RT
    assert np.max(np.abs(J - ref.Jtot)) <= TOL_RT * max(1.0, np.max(np.abs(ref.Jtot)))
    assert rel(uf, ref.ubk) <= TOL_RT


def test_sym_nyquist_correction():
    """Orbitals with a large Nyquist component: the symmetric kernel's Nyquist term matters."""
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup("ng32_nk4")
    u = rand_orbs(S, 12)
    u[..., 1::2] *= -1.0                    # push weight to the highest frequencies
    vf = ctx.ubkwbk_vFwbk(u, u)
    assert rel(vf, O.ubkwbk_vFwbk(S, u, u)) <= TOL_OP


@pytest.mark.parametrize("name", ["ng16_nk3_unocc", "ng64_nk8", "ng256_nk2"])
def test_fock_kinetic_density(name):
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup(name)
    u = rand_orbs(S, 3)
    w = rand_orbs(S, 4, nb=S.NB + 1)  # a Krylov-like block with another band count
    assert rel(ctx.ubkwbk_vFwbk(u, w), O.ubkwbk_vFwbk(S, u, w)) <= TOL_OP
    assert rel(ctx.ubk_tubk(w, -0.2), O.ubk_tubk(S, w, -0.2)) <= TOL_OP
    assert rel(ctx.ubk_dns(u), O.ubk_dns(S, u)) <= 1e-13
    assert rel(ctx.dns_vH_of(u), O.dns_vH(S, O.ubk_dns(S, u))) <= TOL_OP


@pytest.mark.parametrize("name", ["ng16_nk3_unocc", "ng32_nk4", "ng128_nk4_nb3"])
def test_observables(name):
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup(name)
    u = O.gram_schmidt(S, rand_orbs(S, 5))
    ctx.set_orbitals(u)
    for A in (0.0, 0.11):
        ob = ctx.observables(A)
        ec = O.ubk_Ecomps(S, u, A)
        for i, key in enumerate(("Ekin", "Eion", "EH", "Exc")):
            assert abs(ob[key] - ec[i]) <= 1e-12 * max(1.0, abs(ec[i])), key
        assert abs(ob["Etot"] - ec.sum()) <= 1e-12 * abs(ec.sum())
        assert abs(ob["Je"] - O.ubk_Je(S, u, A)) <= 1e-12
        assert abs(ob["Nele"] - 2.0 * S.NBocc) <= 1e-12


@pytest.mark.parametrize("name", ["ng32_nk4", "ng64_nk8", "ng16_nk3_unocc", "ng128_nk4_nb3", "ng256_nk2",
                                  "ng512_nk2", "ng64_nk4_nb1", "ng64_nk5_nb4"])
@pytest.mark.parametrize("small", [0, 1])
def test_rk4_run(name, small):
    """The RT loop vs the oracle, through the tiled path (small=0) and the fused
    one-launch-per-stage path (small=1)."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import define_afield, _capi
    cfg, ctx, S = setup(name)
    if small and cfg.NG > 256:
        pytest.skip("fused stages need NG <= 256")
    # RK4 is stable for |E_max| dt < 2.8 with E_max ~ (pi NG / a)^2 / 2: scale dt with the grid
    dt = 0.004 * min(1.0, (64.0 / cfg.NG) ** 2)
    cfg = dataclasses.replace(cfg, dt=dt, NT=5, field_option="LP", omegac=1.55, Tpulse=0.1, E0=20.0)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    _, A, Aave, _ = define_afield(cfg)
    ctx.set_orbitals(u0)
    ctx.set_option(_capi.OPT_SMALL_STAGES, small)
    try:
        E, J, N = ctx.rk4_run(A, Aave, cfg.dt)
    finally:
        ctx.set_option(_capi.OPT_SMALL_STAGES, 2)
    S.cfg = to_oracle_config(cfg)
    ref = O.rt_calculation(S, u0, nt=cfg.NT, A=A, Aave=Aave)
    assert rel(E, ref.Etot) <= TOL_RT
    assert rel(N, ref.Nele) <= TOL_RT
    assert np.max(np.abs(J - ref.Jtot)) <= TOL_RT * max(1.0, np.max(np.abs(ref.Jtot)))
    assert rel(ctx.get_orbitals(), ref.ubk) <= TOL_RT


def test_rk4_step_matches_run():
    """mattohf_rk4_step (host fields) == one step of mattohf_rk4_run (device fields):
    bitwise through the same tiled kernels, to rounding through the fused stages."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import _capi
    cfg, ctx, S = setup("ng32_nk4")
    u0 = O.gram_schmidt(S, O.init_wf(S))
    ctx.set_orbitals(u0)
    ctx.RT_RK4_ubk(0.01, 0.02, 0.005)
    a = ctx.get_orbitals()
    ctx.set_option(_capi.OPT_SMALL_STAGES, 0)
    try:
        ctx.set_orbitals(u0)
        ctx.rk4_run(np.array([0.02]), np.array([0.01]), 0.005)
        b = ctx.get_orbitals()
    finally:
        ctx.set_option(_capi.OPT_SMALL_STAGES, 2)
    assert np.array_equal(a, b)
    ctx.set_orbitals(u0)
    ctx.rk4_run(np.array([0.02]), np.array([0.01]), 0.005)
    assert rel(ctx.get_orbitals(), a) <= 1e-14
    ref = O.rk4_step(S, u0, 0.01, 0.02, 0.005)
    assert rel(a, ref) <= TOL_OP


@pytest.mark.parametrize("variant", ["TE", "TEPC", "TEPC2"])
def test_taylor_propagators(variant):
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup("ng16_nk3_unocc")
    u0 = O.gram_schmidt(S, O.init_wf(S))
    ctx.set_orbitals(u0)
    ctx.RT_TE_ubk(0.02, 0.004, variant)
    got = ctx.get_orbitals()
    ref = O.te_step(S, u0, 0.02, 0.004, variant)
    assert rel(got, ref) <= TOL_OP


@pytest.mark.parametrize("small", [0, 1])
def test_graph_equals_eager(small):
    """The graph-replayed RT loop (two eight-step graphs, then three one-step
    graphs) is bitwise identical to eager launches."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import _capi
    cfg, ctx, S = setup("ng64_nk8")
    ctx.set_option(_capi.OPT_SMALL_STAGES, small)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    A = np.linspace(0.0, 0.05, 19)
    Aave = np.concatenate([[A[0] / 2], 0.5 * (A[1:] + A[:-1])])
    ctx.set_orbitals(u0)
    r1 = ctx.rk4_run(A, Aave, 0.005)
    u1 = ctx.get_orbitals()
    ctx.set_option(_capi.OPT_GRAPH, 0)
    ctx.set_orbitals(u0)
    r2 = ctx.rk4_run(A, Aave, 0.005)
    u2 = ctx.get_orbitals()
    ctx.set_option(_capi.OPT_GRAPH, 1)
    ctx.set_option(_capi.OPT_SMALL_STAGES, 2)
    assert np.array_equal(u1, u2)
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("small", [0, 1])
def test_nonfinite_detected(small):
    """An unstable dt overflows; the run returns ERR_NONFINITE naming the step."""
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import MattohfError, _capi
    cfg, ctx, S = setup("ng64_nk8")
    u0 = O.gram_schmidt(S, O.init_wf(S))
    ctx.set_orbitals(u0)
    nt = 600
    A = np.zeros(nt)
    ctx.set_option(_capi.OPT_SMALL_STAGES, small)
    try:
        with pytest.raises(MattohfError) as ei:
            ctx.rk4_run(A, A, 0.5)   # eps_max*dt ~ 100 >> 2.83
    finally:
        ctx.set_option(_capi.OPT_SMALL_STAGES, 2)
    assert ei.value.status == _capi.ERR_NONFINITE
    assert "step" in str(ei.value)


def gs_errors(got, ref, S, dns):
    """Gauge-invariant deviations of a GPU ground state from the oracle's: Etot of
    every iteration (relative per iteration), final Ritz values and
    eigen-residuals (the reference's sum of abs, not abs^2, F:353; max-norm
    relative), Je of every iteration (absolute) and the final density."""
    from oracle import mattohf_oracle as O
    return {"Etot": float(np.max(np.abs(got["Etot"] - ref.Etot) / np.abs(ref.Etot))),
            "epsbk": rel(got["epsbk"], ref.epsbk),
            "epserrorbk": rel(got["epserrorbk"], ref.epserrorbk),
            "Je": float(np.max(np.abs(got["Je"] - ref.Je))),
            "density": rel(dns, O.ubk_dns(S, ref.ubk))}


def check_gs(label, errs, bound):
    print(f"{label}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v <= bound[k], (label, k, v, bound[k])


@pytest.mark.parametrize("name,ncg", [("ng32_nk4", 4), ("ng16_nk3_unocc", 2), ("ng16_nk3_unocc", 3),
                                      ("ng64_nk4_nb1", 5)])  # Krylov dimension 8, 6, 9 and 5
def test_gs_gauge_invariants(name, ncg):
    """SCF iterations against the oracle.  A Krylov block amplifies rounding in
    the h-applies, so each case's bounds sit 100x above what a relative 1e-13
    perturbation of every h-apply does to the oracle (measured on these cases:
    Etot <= 2.3e-13, epsbk <= 1.1e-12, epserrorbk <= 1.4e-11, Je <= 1.8e-13,
    density <= 2.1e-12).  Odd Krylov dimensions are included."""
    from oracle import mattohf_oracle as O
    cfg, ctx, S = setup(name)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    nscf = 4
    S.cfg = dataclasses.replace(S.cfg, NCG=ncg)
    ref = O.gs_calculation(S, u0, nscf=nscf)
    ctx.set_orbitals(u0)
    got = ctx.GS_calculation(nscf, ncg)
    errs = gs_errors(got, ref, S, ctx.ubk_dns(ctx.get_orbitals()))
    check_gs(f"GS {name} ncg={ncg}", errs,
             {"Etot": 1e-11, "epsbk": 1e-10, "epserrorbk": 1e-9, "Je": 1e-11, "density": 1e-10})


def test_gs_wide_krylov_block():
    """Krylov dimension 48 (NB=24, NCG=2): the eigensolver's and the staged
    Gram-Schmidt's shared memory exceed 48 KB.  A relative 1e-13 perturbation
    of every h-apply moves the oracle by Etot 4.5e-12, epsbk 7.7e-11,
    epserrorbk 8.2e-9, Je 3.2e-11 and the density 1.4e-9; the bounds sit 10x
    above (Etot and Je 100x)."""
    from mattohf_gb300 import Context
    from oracle import mattohf_oracle as O
    cfg = make_cfg(NG=128, NK=1, NB=24, NBocc=24)
    S = O.make_system(to_oracle_config(cfg))
    nscf, ncg = 3, 2
    S.cfg = dataclasses.replace(S.cfg, NCG=ncg)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    ref = O.gs_calculation(S, u0, nscf=nscf)
    with Context(cfg) as ctx:
        ctx.set_orbitals(u0)
        got = ctx.GS_calculation(nscf, ncg)
        errs = gs_errors(got, ref, S, ctx.ubk_dns(ctx.get_orbitals()))
    check_gs("GS wide block", errs, {"Etot": 1e-9, "epsbk": 1e-9, "epserrorbk": 1e-7, "Je": 1e-9,
                                     "density": 1e-8})


def test_gs_krylov_block_in_global_memory():
    """Krylov dimension 48 at NG=256 (NB=24, NCG=2): the block of a k-point is
    48*256*16 B = 192 KB, above the 160 KB shared-memory staging limit, so the
    Krylov Gram-Schmidt (classical, applied twice) runs on global memory.  A
    relative 1e-13 perturbation of every h-apply moves the oracle by Etot
    2.5e-10, epsbk 8.6e-10, epserrorbk 6.7e-8, Je 7.3e-11 and the density
    5.0e-9; the bounds sit 10x above that, except for Je.  At one k-point
    (kx = 0) with real Gaussian orbitals the current vanishes by symmetry but
    for the unpaired Nyquist component G = -NG/2 bx (src/Initialization.f90:97-102),
    so Je (about 2.5e-6 here) measures the orbitals' highest-frequency content,
    where the Krylov block [u, hu] holds its largest and the GPU's transforms
    and orthonormalisation round differently from the oracle's (measured
    5.9e-9).  Its bound is 2e-8 absolute."""
    from mattohf_gb300 import Context
    from oracle import mattohf_oracle as O
    cfg = make_cfg(NG=256, NK=1, NB=24, NBocc=24)
    S = O.make_system(to_oracle_config(cfg), vCk=O.k_vCk_fast)
    nscf, ncg = 3, 2
    S.cfg = dataclasses.replace(S.cfg, NCG=ncg)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    ref = O.gs_calculation(S, u0, nscf=nscf)
    with Context(cfg) as ctx:
        vCG, vCq = ctx.coulomb()
        assert rel(vCG, S.vCG) <= TOL_OP and rel(vCq[0], S.vCGkk[0]) <= TOL_OP
        ctx.set_orbitals(u0)
        got = ctx.GS_calculation(nscf, ncg)
        errs = gs_errors(got, ref, S, ctx.ubk_dns(ctx.get_orbitals()))
    check_gs("GS block in global memory", errs, {"Etot": 3e-9, "epsbk": 1e-8, "epserrorbk": 1e-6, "Je": 2e-8,
                                                  "density": 5e-8})


@pytest.mark.parametrize("ng,nb", [(64, 5), (512, 24)])
def test_gram_schmidt_staged_and_global(ng, nb):
    """Gram-Schmidt with the k-point's columns held in shared memory (NB*NG*16 B
    up to 160 KB) and in global memory (above it), against the oracle."""
    from mattohf_gb300 import Context
    from oracle import mattohf_oracle as O
    cfg = make_cfg(NG=ng, NK=2, NB=nb, NBocc=1)
    S = O.make_system(to_oracle_config(cfg))
    u = O.init_wf(S)
    rng = np.random.default_rng(11)
    u = u + 0.3 * (rng.standard_normal(u.shape) + 1j * rng.standard_normal(u.shape)) * np.max(np.abs(u))
    ref = O.gram_schmidt(S, u)
    with Context(cfg) as ctx:
        ctx.set_orbitals(u)
        ctx.Gram_Schmidt()
        got = ctx.get_orbitals()
    assert rel(got, ref) <= 1e-11


@pytest.mark.parametrize("case", ["hf_ng32_nk4", "hf_ng16_nk3_unocc"])
def test_golden(case):
    """GPU path against the committed oracle fixtures."""
    from mattohf_gb300 import Context, RunConfig
    g = np.load(os.path.join(GOLD, case + ".npz"))
    with open(os.path.join(GOLD, case + ".json")) as fh:
        d = json.load(fh)
    cfg = RunConfig(**{f.name: d[f.name] for f in dataclasses.fields(RunConfig)})
    with Context(cfg) as ctx:
        A = float(g["A"])
        assert rel(ctx.ubkwbk_hwbk(g["u"], g["w"], A), g["hw"]) <= TOL_OP
        assert rel(ctx.ubkwbk_vFwbk(g["u"], g["w"]), g["vF"]) <= TOL_OP
        ctx.set_orbitals(g["u"])
        ob = ctx.observables(A)
        assert abs(ob["Etot"] - g["Ecomps"].sum()) <= 1e-12 * abs(g["Ecomps"].sum())
        from mattohf_gb300 import aave_from_samples
        A_t = g["rt_A"]
        E, J, N = ctx.rk4_run(A_t, aave_from_samples(A_t), cfg.dt)
        assert rel(E, g["rt_Etot"]) <= TOL_RT
        assert np.max(np.abs(J - g["rt_Jtot"])) <= TOL_RT
        assert rel(ctx.get_orbitals(), g["rt_u"]) <= TOL_RT


def test_context_usable_after_errors():
    """Invalid calls return ERR_ARG with a message and leave the context usable; so
    does a non-finite run once the orbitals are reset."""
    import ctypes as C
    from oracle import mattohf_oracle as O
    from mattohf_gb300 import MattohfError, _capi
    cfg, ctx, S = setup("ng32_nk4")
    u0 = O.gram_schmidt(S, O.init_wf(S))
    lib = ctx.lib
    assert lib.mattohf_set_option(ctx.h, 99, 1) == _capi.ERR_ARG
    assert b"unknown option" in lib.mattohf_last_error(ctx.h)
    assert lib.mattohf_set_option(ctx.h, _capi.OPT_SMALL_STAGES, 5) == _capi.ERR_ARG
    D = C.POINTER(C.c_double)
    buf = np.zeros(8)
    assert lib.mattohf_rk4_run(ctx.h, -1, C.c_double(0.01), buf.ctypes.data_as(D), buf.ctypes.data_as(D),
                               None, None, None) == _capi.ERR_ARG
    ctx.set_orbitals(u0)
    with pytest.raises(MattohfError) as ei:
        ctx.rk4_run(np.zeros(300), np.zeros(300), 0.5)
    assert ei.value.status == _capi.ERR_NONFINITE
    ctx.set_orbitals(u0)
    A = np.array([0.01, 0.02])
    Aave = np.array([0.005, 0.015])
    E, J, N = ctx.rk4_run(A, Aave, 0.004)
    S.cfg = to_oracle_config(dataclasses.replace(cfg, dt=0.004))
    ref = O.rt_calculation(S, u0, nt=2, A=A, Aave=Aave)
    assert rel(E, ref.Etot) <= TOL_RT
    assert rel(ctx.get_orbitals(), ref.ubk) <= TOL_RT


@pytest.mark.parametrize("small", [0, 1])
def test_long_golden_run(small):
    """The full 2000-step run of the CPU-runnable shape (stable dt) against the oracle's
    committed series, through the tiled path and through the fused stages.  The
    relative error of each result (Etot, Je, Nele, the dipole, the final orbitals)
    is printed and stays within the 1e-10 bound.  Je crosses zero, so its error is
    relative to max |Je| (at least 1); the dipole is -int Je dt from the initial
    current by the trapezoid rule, pinned only through Je."""
    from mattohf_gb300 import Context, RunConfig, aave_from_samples, dipole_from_current, _capi
    from oracle import mattohf_oracle as O
    g = np.load(os.path.join(GOLD, "rt2000_ng64_nk8.npz"))
    with open(os.path.join(GOLD, "rt2000_ng64_nk8.json")) as fh:
        d = json.load(fh)
    cfg = RunConfig(**{f.name: d[f.name] for f in dataclasses.fields(RunConfig)})
    A = g["rt_A"]
    with Context(cfg) as ctx:
        ctx.set_option(_capi.OPT_SMALL_STAGES, small)
        ctx.set_orbitals(g["u0"])
        J0 = ctx.observables(0.0)["Je"]
        E, J, N = ctx.rk4_run(A, aave_from_samples(A), cfg.dt)
        u = ctx.get_orbitals()
    S = O.make_system(to_oracle_config(cfg))
    J0r = O.ubk_Je(S, g["u0"], 0.0)
    P = dipole_from_current(J, J0, cfg.dt)
    Pr = O.dipole_from_current(None, g["rt_Jtot"], J0r, cfg.dt)
    err = {"Etot": rel(E, g["rt_Etot"]),
           "Je": np.max(np.abs(J - g["rt_Jtot"])) / max(1.0, np.max(np.abs(g["rt_Jtot"]))),
           "Nele": rel(N, g["rt_Nele"]),
           "dipole": rel(P, Pr),
           "orbitals": rel(u, g["rt_u"])}
    print("golden 2000-step run, small=%d: " % small + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for k, v in err.items():
        assert v <= TOL_RT, (k, v)


@pytest.mark.parametrize("NG,NK,NB", [(64, 8, 2), (128, 16, 2), (256, 8, 4)])
def test_autotune_restores_state_and_keeps_results(NG, NK, NB):
    """The autotuner times its candidates on the context's own orbitals, restores
    them bitwise, and the tuned launch shapes give the same run (1e-12)."""
    from mattohf_gb300 import Context, RunConfig, _capi
    cfg = RunConfig(acell=10.0, NG=NG, NK=NK, NB=NB, NBocc=NB, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    A = 0.02 * np.sin(0.3 * np.arange(1, 9))
    Aave = np.concatenate([0.5 * A[:1], 0.5 * (A[1:] + A[:-1])])
    dt = 2e-4
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u0 = ctx.get_orbitals()
        E0, J0, N0 = ctx.rk4_run(A, Aave, dt)
        u_end0 = ctx.get_orbitals()
        ctx.set_orbitals(u0)
        res = ctx.autotune(steps=8)
        assert np.array_equal(ctx.get_orbitals(), u0)
        assert res["sym_tile"] >= 1 and res["sym_tile"] & (res["sym_tile"] - 1) == 0
        assert res["exchange_us"] > 0 and res["tiled_step_us"] > 0
        if res["small_ctas"]:
            assert res["fused_step_us"] > 0
        E, J, N = ctx.rk4_run(A, Aave, dt)
        assert rel(E, E0) <= 1e-12 and rel(N, N0) <= 1e-12
        assert np.max(np.abs(J - J0)) <= 1e-12 * max(1.0, np.max(np.abs(J0)))
        # every CTAs-per-column setting of the fused stages gives the same run,
        # including grids far beyond one wave (the stage field is read by each
        # column's first CTA while other columns finish)
        for P in (1, 2, 3, 4, 5, 6, 8, 12, 24):
            ctx.set_option(_capi.OPT_SMALL_STAGES, 1)
            ctx.set_option(_capi.OPT_SMALL_CTAS, P)
            ctx.set_orbitals(u0)
            E, J, N = ctx.rk4_run(A, Aave, dt)
            assert rel(E, E0) <= 1e-12 and rel(N, N0) <= 1e-12, P
            assert np.max(np.abs(J - J0)) <= 1e-12 * max(1.0, np.max(np.abs(J0))), P
            assert rel(ctx.get_orbitals(), u_end0) <= 1e-12, P
