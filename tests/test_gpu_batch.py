"""Batched ensemble vs the same runs advanced one at a time (needs a GB300)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cfgs():
    from mattohf_gb300 import RunConfig
    out = []
    rng = np.random.default_rng(1)
    for nk, nb in [(2, 1), (4, 2), (8, 3), (4, 4), (2, 2)]:
        a = float(rng.uniform(8.0, 14.0))
        out.append(RunConfig(acell=a, NG=64, NK=nk, NB=nb, NBocc=nb, Zeff=[2.0], alpha=[1.0],
                             Rion=[0.5], Kion=[1]))
    return out


def test_batch_matches_single_runs(built_lib):
    from mattohf_gb300 import Batch, Context
    cfgs = _cfgs()
    nt = 4
    rng = np.random.default_rng(2)
    A = 0.02 * rng.standard_normal((len(cfgs), nt))
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    dts = np.array([0.004, 0.003, 0.002, 0.004, 0.005])
    with Batch(cfgs) as b:
        u0 = []
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
            u0.append(b[r].get_orbitals())
        E, J, N = b.rk4_run(A, Aave, dts)
        ub = [b[r].get_orbitals() for r in range(len(cfgs))]
    for r, cfg in enumerate(cfgs):
        with Context(cfg) as c:
            c.set_orbitals(u0[r])
            e, j, n = c.rk4_run(A[r], Aave[r], dts[r])
            us = c.get_orbitals()
        # same kernels; the single run may pick a smaller exchange tile (a
        # different but fixed summation order), so agreement is to rounding
        assert np.max(np.abs(e - E[r])) <= 1e-13 * np.max(np.abs(e)), r
        assert np.max(np.abs(j - J[r])) <= 1e-13 * max(1.0, np.max(np.abs(j))), r
        assert np.max(np.abs(n - N[r])) <= 1e-13 * np.max(np.abs(n)), r
        assert np.max(np.abs(us - ub[r])) <= 1e-12 * np.max(np.abs(us)), r


def test_batch_against_oracle(built_lib):
    """One member of a mixed batch against the oracle's RT loop."""
    from mattohf_gb300 import Batch
    from oracle import mattohf_oracle as O
    from conftest import to_oracle_config
    cfgs = _cfgs()
    nt = 3
    A = np.tile(np.array([0.01, 0.02, 0.015]), (len(cfgs), 1))
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    with Batch(cfgs) as b:
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
        u2 = b[2].get_orbitals()
        E, J, N = b.rk4_run(A, Aave, 0.003)
    import dataclasses
    S = O.make_system(to_oracle_config(dataclasses.replace(cfgs[2], dt=0.003)))
    ref = O.rt_calculation(S, u2, nt=nt, A=A[2], Aave=Aave[2])
    assert np.max(np.abs(E[2] - ref.Etot)) <= 1e-10 * np.max(np.abs(ref.Etot))
    assert np.max(np.abs(J[2] - ref.Jtot)) <= 1e-10


def test_batch_double_float_matches_single_runs(built_lib):
    """Batched double-float exchange vs the same runs advanced one at a time in double-float,
    and vs the FP64 batch within the 1e-10 real-time tolerance."""
    from mattohf_gb300 import Batch, Context, _capi
    cfgs = _cfgs()
    nt = 4
    rng = np.random.default_rng(3)
    A = 0.02 * rng.standard_normal((len(cfgs), nt))
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    dts = np.array([0.004, 0.003, 0.002, 0.004, 0.005])
    with Batch(cfgs) as b:
        u0 = []
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
            u0.append(b[r].get_orbitals())
        E64, J64, _ = b.rk4_run(A, Aave, dts)
        for r in range(len(cfgs)):
            b[r].set_orbitals(u0[r])
        b.set_option(_capi.OPT_FOCK_DF64, 1)
        E, J, N = b.rk4_run(A, Aave, dts)
        ub = [b[r].get_orbitals() for r in range(len(cfgs))]
    assert np.max(np.abs(E - E64)) <= 1e-10 * np.max(np.abs(E64))
    assert np.max(np.abs(J - J64)) <= 1e-10 * max(1.0, np.max(np.abs(J64)))
    for r, cfg in enumerate(cfgs):
        with Context(cfg) as c:
            c.set_option(_capi.OPT_FOCK_DF64, 1)
            c.set_orbitals(u0[r])
            e, j, n = c.rk4_run(A[r], Aave[r], dts[r])
            us = c.get_orbitals()
        assert np.max(np.abs(e - E[r])) <= 1e-12 * np.max(np.abs(e)), r
        assert np.max(np.abs(j - J[r])) <= 1e-12 * max(1.0, np.max(np.abs(j))), r
        assert np.max(np.abs(n - N[r])) <= 1e-12 * np.max(np.abs(n)), r
        assert np.max(np.abs(us - ub[r])) <= 1e-11 * np.max(np.abs(us)), r


def test_batch_autotune_restores_state_and_keeps_results(built_lib):
    """The batch autotuner restores every run's orbitals bitwise; every tile it
    may pick (and the tuned one) gives the ensemble's results to rounding."""
    from mattohf_gb300 import Batch, _capi
    cfgs = _cfgs()
    nt = 4
    rng = np.random.default_rng(3)
    A = 0.02 * rng.standard_normal((len(cfgs), nt))
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    dts = np.array([0.004, 0.003, 0.002, 0.004, 0.005])
    with Batch(cfgs) as b:
        u0 = []
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
            u0.append(b[r].get_orbitals())
        E0, J0, N0 = b.rk4_run(A, Aave, dts)
        for r in range(len(cfgs)):
            b[r].set_orbitals(u0[r])
        res = b.autotune(steps=3)
        assert res["sym_tile"] >= 1 and res["step_us"] > 0
        for r in range(len(cfgs)):
            assert np.array_equal(b[r].get_orbitals(), u0[r]), r
        E, J, N = b.rk4_run(A, Aave, dts)
        assert np.max(np.abs(E - E0)) <= 1e-13 * np.max(np.abs(E0))
        assert np.max(np.abs(N - N0)) <= 1e-13 * np.max(np.abs(N0))
        for tile in (1, 2, 4):
            b.set_option(_capi.OPT_SYM_TILE, tile)
            for r in range(len(cfgs)):
                b[r].set_orbitals(u0[r])
            E, J, N = b.rk4_run(A, Aave, dts)
            assert np.max(np.abs(E - E0)) <= 1e-13 * np.max(np.abs(E0)), tile
            assert np.max(np.abs(J - J0)) <= 1e-13 * max(1.0, np.max(np.abs(J0))), tile


@pytest.mark.parametrize("ckpt", [0, 3])
def test_batch_adjoint_matches_single_runs(built_lib, ckpt):
    """mattohf_batch_adjoint gives every member the gradients of mattohf_adjoint
    run on that member alone (1e-11), for uneven members, both objectives'
    energy form and an explicit and a fitted checkpoint interval."""
    from mattohf_gb300 import Batch, RunConfig
    cfgs = [RunConfig(acell=a, NG=64, NK=k, NB=b, NBocc=b, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
            for a, k, b in [(10.0, 4, 2), (8.0, 6, 1), (12.0, 3, 3)]]
    nt = 10
    rng = np.random.default_rng(21)
    A = 0.05 * np.sin(0.2 * np.arange(1, nt + 1))[None, :] + 1e-3 * rng.standard_normal((len(cfgs), nt))
    dts = np.array([2e-3, 1.5e-3, 2.5e-3])
    with Batch(cfgs) as b:
        u0 = []
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
            u0.append(b[r].get_orbitals())
        L, g, gv = b.adjoint(A, dts, "energy", ckpt_every=ckpt)
        for r in range(len(cfgs)):
            b[r].set_orbitals(u0[r])
            Lr, gr, gvr = b[r].adjoint(A[r], dts[r], "energy", ckpt_every=ckpt)
            assert abs(L[r] - Lr) <= 1e-11 * max(1.0, abs(Lr))
            assert np.max(np.abs(g[r] - gr)) <= 1e-11 * np.max(np.abs(gr))
            assert np.max(np.abs(gv[r] - gvr)) <= 1e-11 * np.max(np.abs(gvr))
        assert b.last_run_ms() > 0


def test_batch_at_ng512_matches_single_runs(built_lib):
    """A batch at the largest grid (its symmetric-exchange CTAs use more than
    48 KB of dynamic shared memory) against each member run alone."""
    from mattohf_gb300 import Batch, Context, RunConfig
    cfgs = [RunConfig(acell=12.0, NG=512, NK=k, NB=b, NBocc=b, Zeff=[1.0], alpha=[1.0], Rion=[1 / 6, 0.5, 5 / 6],
                      Kion=[1, 1, 1]) for k, b in [(2, 2), (3, 1)]]
    nt = 3
    A = 0.01 * np.arange(1, nt + 1)[None, :] * np.array([[1.0], [-0.5]])
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    dt = 2.5e-4
    with Batch(cfgs) as b:
        u0 = []
        for r in range(len(cfgs)):
            b[r].Init_wf()
            b[r].Gram_Schmidt()
            u0.append(b[r].get_orbitals())
        E, J, N = b.rk4_run(A, Aave, dt)
        ub = [b[r].get_orbitals() for r in range(len(cfgs))]
    for r, cfg in enumerate(cfgs):
        with Context(cfg) as c:
            c.set_orbitals(u0[r])
            e, j, n = c.rk4_run(A[r], Aave[r], dt)
            assert np.max(np.abs(E[r] - e)) <= 1e-12 * np.max(np.abs(e))
            assert np.max(np.abs(ub[r] - c.get_orbitals())) <= 1e-12 * np.max(np.abs(ub[r]))
