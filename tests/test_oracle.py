"""Oracle self-checks on CPU: golden fixtures, physics known answers, the C port.

The reference ships no tests or golden vectors (parity unpinned), so the
oracle is pinned by known answers of the physics it restates.
"""
from __future__ import annotations

import dataclasses
import json
import math
import os

import numpy as np
import pytest

from oracle import mattohf_oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def small(**kw):
    base = dict(acell=10.0, NG=32, NK=4, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    base.update(kw)
    return O.Config(**base)


def rand(S, seed, nb=None):
    rng = np.random.default_rng(seed)
    sh = (S.NK, S.NB if nb is None else nb, S.NG)
    return rng.standard_normal(sh) + 1j * rng.standard_normal(sh)


@pytest.mark.parametrize("case", ["hf_ng32_nk4", "hf_ng16_nk3_unocc"])
def test_oracle_reproduces_golden(case):
    g = np.load(os.path.join(GOLD, case + ".npz"))
    with open(os.path.join(GOLD, case + ".json")) as fh:
        cfg = O.Config(**json.load(fh))
    S = O.make_system(cfg)
    np.testing.assert_allclose(S.vCGkk, g["vCGkk"], rtol=0, atol=1e-14 * np.abs(g["vCGkk"]).max())
    hw = O.ubkwbk_hwbk(S, g["u"], g["w"], float(g["A"]))
    assert np.max(np.abs(hw - g["hw"])) <= 1e-13 * np.max(np.abs(g["hw"]))
    rt = O.rt_calculation(S, g["u"], nt=cfg.NT)
    assert np.max(np.abs(rt.Etot - g["rt_Etot"])) <= 1e-12 * np.max(np.abs(g["rt_Etot"]))


def test_free_particle_eigenvalues():
    """No ions, no e-e: h = 1/2 (G+k+A)^2, plane waves are eigenvectors."""
    cfg = small(functional="none", Zeff=[0.0])
    S = O.make_system(cfg)
    S.vCG[:] = 0.0
    u = np.zeros((S.NK, S.NB, S.NG), dtype=np.complex128)
    for ik in range(S.NK):
        for ib, g in enumerate([0, 3]):
            u[ik, ib] = np.exp(1j * S.Gx[g] * S.rx)
    A = 0.07
    h = O.ubkwbk_hwbk(S, u, u, A)
    for ik in range(S.NK):
        for ib, g in enumerate([0, 3]):
            lam = 0.5 * (S.Gx[g] + S.kx[ik] + A) ** 2
            assert np.max(np.abs(h[ik, ib] - lam * u[ik, ib])) < 1e-12


def test_hermiticity():
    S = O.make_system(small())
    u = O.gram_schmidt(S, rand(S, 1))
    a, b = rand(S, 2), rand(S, 3)
    ha, hb = O.ubkwbk_hwbk(S, u, a, 0.2), O.ubkwbk_hwbk(S, u, b, 0.2)
    assert abs(np.vdot(a, hb) - np.conj(np.vdot(b, ha))) < 1e-11 * abs(np.vdot(a, hb))


def test_particle_number():
    S = O.make_system(small(NB=3, NBocc=2))
    u = O.gram_schmidt(S, rand(S, 4))
    assert abs(O.ubk_dns(S, u).sum() * S.dvcell - 2 * S.NBocc) < 1e-12


def test_soft_coulomb_transform_limit():
    """2 int_0^L cos(qx)/sqrt(x^2+1) dx -> 2 K0(|q|) as L = NK*a grows."""
    from scipy.special import k0
    L = 64 * 10.0
    for q in (0.5, 1.3, 2.7):
        v = O.k_vCk_fast(q, 10.0, 64, 64)[0]
        # the truncated tail of int cos(qx)/x oscillates with amplitude ~ 1/(q L)
        assert abs(v - 2.0 * k0(q)) < 1.5 / (q * L)


def test_k_vck_orders_agree():
    ks = np.array([0.0, 0.3, 1.7, 5.5])
    a = O.k_vCk(ks, 7.0, 16, 3)
    b = O.k_vCk_fast(ks, 7.0, 16, 3)
    assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(a))


def test_gauge_uniform_A_is_k_shift():
    """A uniform A enters the kinetic term as k -> k + A; the Fock term depends on k-k' only."""
    S = O.make_system(small())
    u = rand(S, 5)
    A = 0.031
    t1 = O.ubk_tubk(S, u, A)
    S2 = O.make_system(small())
    S2.kx = S.kx + A
    t2 = O.ubk_tubk(S2, u, 0.0)
    assert np.max(np.abs(t1 - t2)) < 1e-12 * np.max(np.abs(t1))


def test_rk4_fourth_order():
    """Global error of RK4 scales as dt^4 at stable dt."""
    cfg = small(NG=16, NK=2, acell=6.0)
    S = O.make_system(cfg)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    T = 0.04

    def run(n):
        u = u0.copy()
        dt = T / n
        for _ in range(n):
            u = O.rk4_step(S, u, 0.01, 0.01, dt)
        return u

    ref = run(64)
    e1 = np.max(np.abs(run(4) - ref))
    e2 = np.max(np.abs(run(8) - ref))
    assert 10.0 < e1 / e2 < 24.0   # ~16 for a 4th-order method


def test_energy_conserved_without_field():
    cfg = small(NG=16, NK=2, acell=6.0, dt=0.002, NT=20, field_option="LR", dAc=0.0)
    S = O.make_system(cfg)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    rt = O.rt_calculation(S, u0)
    assert np.max(np.abs(rt.Etot - rt.Etot0)) < 1e-7 * abs(rt.Etot0)


def test_current_is_minus_dipole_rate():
    """Je is the time derivative of -P; the dipole extension integrates it."""
    t = np.linspace(0, 1, 11)
    J = np.sin(t)
    P = O.dipole_from_current(t, J[1:], J[0], t[1] - t[0])
    assert abs(P[-1] - (-(1 - math.cos(1.0)))) < 1e-2


def test_c_port_matches_numpy_oracle():
    from oracle import build_cref
    import ctypes as C
    lib = build_cref.load()
    cfg = small(NG=32, NK=4, NB=3, NBocc=2)
    S = O.make_system(cfg)
    D = C.POINTER(C.c_double)
    h = lib.cref_create(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, cfg.acell, 1,
                        S.vion.ctypes.data_as(D), None, None)
    try:
        vCG = np.empty(cfg.NG)
        vCq = np.empty((2 * cfg.NK - 1, cfg.NG))
        lib.cref_get_tables(h, vCG.ctypes.data_as(D), vCq.ctypes.data_as(D))
        assert np.max(np.abs(vCG - S.vCG)) < 1e-13
        u = O.gram_schmidt(S, rand(S, 6))
        w = rand(S, 7)
        hw = np.empty_like(w)
        lib.cref_hpsi(h, u.view(np.float64).ctypes.data_as(D), w.view(np.float64).ctypes.data_as(D),
                      cfg.NB, C.c_double(0.2), hw.view(np.float64).ctypes.data_as(D))
        ref = O.ubkwbk_hwbk(S, u, w, 0.2)
        assert np.max(np.abs(hw - ref)) < 1e-12 * np.max(np.abs(ref))
        nt = 3
        A = np.array([0.01, 0.02, 0.03])
        Aave = np.array([0.005, 0.015, 0.025])
        uu = u.copy()
        E, J, N = np.empty(nt), np.empty(nt), np.empty(nt)
        lib.cref_rk4_run(h, uu.view(np.float64).ctypes.data_as(D), nt, C.c_double(0.004),
                         A.ctypes.data_as(D), Aave.ctypes.data_as(D), E.ctypes.data_as(D),
                         J.ctypes.data_as(D), N.ctypes.data_as(D))
        cfg2 = dataclasses.replace(cfg, dt=0.004)
        S.cfg = cfg2
        rt = O.rt_calculation(S, u, nt=nt, A=A, Aave=Aave)
        assert np.max(np.abs(E - rt.Etot)) < 1e-11 * np.max(np.abs(rt.Etot))
        assert np.max(np.abs(J - rt.Jtot)) < 1e-11
        assert np.max(np.abs(uu - rt.ubk)) < 1e-11
    finally:
        lib.cref_destroy(h)


def test_c_port_matches_numpy_oracle_medium():
    """The C restatement against the numpy oracle at NG=128, NK=16, NB=NBocc=4
    (4096 exchange pairs per apply, two ions): h[u] w, h[u] u, the observables
    and 3 RK4 steps.  With the small-size check above and the GPU parity tests
    at the benchmarked shapes (which compare the GPU with the C restatement)
    this closes the chain GPU -> C restatement -> numpy oracle.  The C
    restatement builds the Coulomb tables; the numpy oracle takes them over."""
    from oracle import build_cref
    import ctypes as C
    lib = build_cref.load()
    cfg = small(NG=128, NK=16, NB=4, NBocc=4, acell=10.0, Zeff=[1.5, 0.5], alpha=[1.0, 1.0],
                Rion=[0.25, 0.75], Kion=[1, 2], dt=2e-3)
    S = O.make_system(cfg, vCk=lambda k, *a: np.zeros(np.shape(k)))
    D = C.POINTER(C.c_double)
    h = lib.cref_create(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, cfg.acell, 1, S.vion.ctypes.data_as(D), None, None)
    try:
        NK = cfg.NK
        vCG = np.empty(cfg.NG)
        vCq = np.empty((2 * NK - 1, cfg.NG))
        lib.cref_get_tables(h, vCG.ctypes.data_as(D), vCq.ctypes.data_as(D))
        # spot-check the C tables against the oracle's sequential trapezoid sum
        q = np.array([S.Gx[3] + S.kx[5] - S.kx[2], S.Gx[64] + S.kx[0] - S.kx[15]])
        ref_q = O.k_vCk(q, cfg.acell, cfg.NG, NK)
        assert abs(vCq[5 - 2 + NK - 1, 3] - ref_q[0]) <= 1e-13 * np.max(np.abs(vCq))
        assert abs(vCq[0 - 15 + NK - 1, 64] - ref_q[1]) <= 1e-13 * np.max(np.abs(vCq))
        idx = (np.arange(NK)[:, None] - np.arange(NK)[None, :] + NK - 1).reshape(-1)
        S.vCGkk = vCq[idx]
        S.vCG = vCG
        u = O.gram_schmidt(S, rand(S, 16))
        w = rand(S, 17)
        for ww, A in ((w, 0.07), (u, -0.05)):
            hw = np.empty_like(ww)
            lib.cref_hpsi(h, u.view(np.float64).ctypes.data_as(D), ww.view(np.float64).ctypes.data_as(D),
                          cfg.NB, C.c_double(A), hw.view(np.float64).ctypes.data_as(D))
            ref = O.ubkwbk_hwbk(S, u, ww, A)
            assert np.max(np.abs(hw - ref)) <= 1e-12 * np.max(np.abs(ref))
        e, j, n = C.c_double(), C.c_double(), C.c_double()
        lib.cref_observables(h, u.view(np.float64).ctypes.data_as(D), C.c_double(0.03), C.byref(e), C.byref(j),
                             C.byref(n))
        assert abs(e.value - O.ubk_Etot(S, u, 0.03)) <= 1e-12 * abs(e.value)
        assert abs(j.value - O.ubk_Je(S, u, 0.03)) <= 1e-12
        nt = 3
        A = np.array([0.02, 0.05, 0.04])
        Aave = np.concatenate([[0.5 * A[0]], 0.5 * (A[1:] + A[:-1])])
        uu = u.copy()
        E, J, N = np.empty(nt), np.empty(nt), np.empty(nt)
        lib.cref_rk4_run(h, uu.view(np.float64).ctypes.data_as(D), nt, C.c_double(cfg.dt),
                         A.ctypes.data_as(D), Aave.ctypes.data_as(D), E.ctypes.data_as(D),
                         J.ctypes.data_as(D), N.ctypes.data_as(D))
        rt = O.rt_calculation(S, u, nt=nt, A=A, Aave=Aave)
        assert np.max(np.abs(E - rt.Etot)) <= 1e-11 * np.max(np.abs(rt.Etot))
        assert np.max(np.abs(J - rt.Jtot)) <= 1e-11
        assert np.max(np.abs(N - rt.Nele)) <= 1e-11 * np.max(np.abs(rt.Nele))
        assert np.max(np.abs(uu - rt.ubk)) <= 1e-11 * np.max(np.abs(rt.ubk))
    finally:
        lib.cref_destroy(h)


@pytest.mark.parametrize("objective", ["energy", "current"])
@pytest.mark.parametrize("NG,NK", [(16, 2), (32, 3)])
def test_oracle_adjoint_matches_finite_differences(objective, NG, NK):
    """Discrete RK4 adjoint of the oracle vs central differences, per sample.

    h = 1e-4: the truncation error (h^2) and the round-off of the quotient
    (1e-16 |L| / h) both stay below 1e-9 relative here, so the bound is 1e-7
    relative to each sample's own difference quotient.  Both exchange terms
    that involve the Nyquist index (the transposed pair operator of the RK4
    adjoint and the exchange-energy gradient) were off by about 5e-6 in this
    per-sample form before they carried the Nyquist correction."""
    cfg = small(NG=NG, NK=NK, NB=2, NBocc=2, acell=6.0 if NG == 16 else 10.0)
    S = O.make_system(cfg)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    rng = np.random.default_rng(3)
    A = 0.05 * rng.standard_normal(4)
    dt = 0.01
    L, g, gv = O.rt_adjoint(S, u0, A, dt, objective)
    h = 1e-4
    for n in range(A.size):
        Ap, Am = A.copy(), A.copy()
        Ap[n] += h
        Am[n] -= h
        fd = (O.rt_adjoint(S, u0, Ap, dt, objective)[0] - O.rt_adjoint(S, u0, Am, dt, objective)[0]) / (2 * h)
        assert abs(g[n] - fd) <= 1e-7 * abs(fd) + 1e-14, (n, g[n], fd)
    h = 1e-6
    # ion potential on the grid
    for x in (0, 5):
        vp = S.vion.copy()
        S.vion = vp.copy(); S.vion[x] += h
        Lp = O.rt_adjoint(S, u0, A, dt, objective)[0]
        S.vion = vp.copy(); S.vion[x] -= h
        Lm = O.rt_adjoint(S, u0, A, dt, objective)[0]
        S.vion = vp
        fd = (Lp - Lm) / (2 * h)
        assert abs(gv[x] - fd) <= 1e-5 * np.max(np.abs(gv)) + 1e-9  # FD round-off ~ 1e-16*|E|/h


def test_ion_param_grad_matches_finite_differences():
    """The chain rule from dL/dvion to (Zeff, alpha, Rion) through the ion
    potential and its max shift (src/Prep_periodic_ion_potential.f90:10-20),
    on a linear functional L = sum g vion, against central differences."""
    cfg = small(NG=64, NK=3, Zeff=[1.5, 0.5], alpha=[1.0, 0.7], Rion=[0.25, 0.7, 0.8], Kion=[1, 2, 2])
    rx = np.arange(cfg.NG) / cfg.NG * cfg.acell
    g = np.random.default_rng(8).standard_normal(cfg.NG)
    dZ, da, dR = O.ion_param_grad(cfg, rx, g)
    h = 1e-6

    def L(**kw):
        return float(np.sum(g * O.ion_potential(dataclasses.replace(cfg, **kw), rx)))

    for s in range(2):
        for name, grad in (("Zeff", dZ), ("alpha", da)):
            p, m = list(getattr(cfg, name)), list(getattr(cfg, name))
            p[s] += h
            m[s] -= h
            fd = (L(**{name: p}) - L(**{name: m})) / (2 * h)
            assert abs(grad[s] - fd) <= 1e-7 * abs(fd) + 1e-9, (name, s, grad[s], fd)
    for i in range(3):
        p, m = list(cfg.Rion), list(cfg.Rion)
        p[i] += h
        m[i] -= h
        fd = (L(Rion=p) - L(Rion=m)) / (2 * h)
        assert abs(dR[i] - fd) <= 1e-7 * abs(fd) + 1e-9, (i, dR[i], fd)


def test_c_port_matches_long_golden_run():
    """The C restatement over the full 2000-step run of the CPU-runnable shape
    reproduces the oracle's committed series (tests/golden/rt2000_ng64_nk8)."""
    import json
    import os
    import ctypes as C
    from oracle import build_cref
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    g = np.load(os.path.join(here, "rt2000_ng64_nk8.npz"))
    with open(os.path.join(here, "rt2000_ng64_nk8.json")) as fh:
        cfg = O.Config(**json.load(fh))
    S = O.make_system(cfg)
    lib = build_cref.load()
    D = C.POINTER(C.c_double)
    h = lib.cref_create(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, cfg.acell, 1, S.vion.ctypes.data_as(D), None, None)
    try:
        A = np.ascontiguousarray(g["rt_A"])
        Aave = np.concatenate([[0.5 * A[0]], 0.5 * (A[1:] + A[:-1])])
        u = np.ascontiguousarray(g["u0"]).copy()
        nt = A.size
        E, J, N = np.empty(nt), np.empty(nt), np.empty(nt)
        lib.cref_rk4_run(h, u.view(np.float64).ctypes.data_as(D), nt, C.c_double(cfg.dt), A.ctypes.data_as(D),
                         Aave.ctypes.data_as(D), E.ctypes.data_as(D), J.ctypes.data_as(D), N.ctypes.data_as(D))
    finally:
        lib.cref_destroy(h)
    assert np.max(np.abs(E - g["rt_Etot"])) <= 1e-10 * np.max(np.abs(g["rt_Etot"]))
    assert np.max(np.abs(J - g["rt_Jtot"])) <= 1e-10 * max(1.0, np.max(np.abs(g["rt_Jtot"])))
    assert np.max(np.abs(N - g["rt_Nele"])) <= 1e-10 * np.max(np.abs(g["rt_Nele"]))
    assert np.max(np.abs(u - g["rt_u"])) <= 1e-10 * np.max(np.abs(g["rt_u"]))


def test_dipole_helper_matches_oracle_quadrature():
    """The product's dipole (P = -int J dt, trapezoid from J(0)) is the oracle's
    quadrature, bitwise, on the golden 2000-step current."""
    import json
    import os
    from mattohf_gb300 import dipole_from_current
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    g = np.load(os.path.join(here, "rt2000_ng64_nk8.npz"))
    with open(os.path.join(here, "rt2000_ng64_nk8.json")) as fh:
        cfg = O.Config(**json.load(fh))
    S = O.make_system(cfg)
    J0 = O.ubk_Je(S, g["u0"], 0.0)
    P = dipole_from_current(g["rt_Jtot"], J0, cfg.dt)
    assert np.array_equal(P, O.dipole_from_current(None, g["rt_Jtot"], J0, cfg.dt))
    assert P.shape == g["rt_Jtot"].shape and np.all(np.isfinite(P))


def test_oracle_edit_descriptors():
    """The oracle's Ew.d / Ew.dEe / Fw.d restatement (oracle/mattohf_program.py)
    on values whose Fortran output the standard fixes, and against the
    drivers' own formatter on random values (two independent writers)."""
    from oracle.mattohf_program import ew, fw, band_record
    from mattohf_gb300.driver import fortran_e, fortran_f
    assert ew(1.0) == "  0.100000000000E+01"
    assert ew(-0.00123456789012345) == " -0.123456789012E-02"
    assert ew(0.0) == "  0.000000000000E+00"
    assert ew(1.5e123) == "  0.150000000000+124"          # a 3-digit exponent drops the E
    assert ew(1.7976931348623157e308) == "  0.179769313486+309"
    assert ew(2.5, e=3) == " 0.250000000000E+001"
    assert fw(-1.2345) == " -1.23450000"
    assert fw(1.7976931348623157e308) == "*" * 12
    assert fw(float("inf")) == "    Infinity" and fw(float("-inf")) == "   -Infinity"
    # '(i5,3e20.12,4x,1e20.12,4x,1000e20.12)': kx, the residual and band 1 share the first group
    rec = band_record(3, 0.5, 0.25, [1.0, 2.0, 3.0])
    assert rec == "    3" + ew(0.5) + ew(0.25) + ew(1.0) + "    " + ew(2.0) + "    " + ew(3.0)
    assert band_record(1, 0.5, 0.25, [1.0]) == "    1" + ew(0.5) + ew(0.25) + ew(1.0)
    rng = np.random.default_rng(4)
    for x in np.concatenate([rng.standard_normal(200) * 10.0 ** rng.integers(-30, 30, 200), [0.0, -0.0]]):
        assert ew(x) == fortran_e(x), x
        assert ew(x, e=3) == fortran_e(x, e=3), x
        if abs(x) < 1e3:
            assert fw(x) == fortran_f(x), x
