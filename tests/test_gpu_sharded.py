"""The k-slice entry points and a run split by output k-point (needs a GB300).

Two ranks share one GPU here: each is its own process with its own context,
the all-gather goes through host memory (gloo), and no kernel waits on
another rank's kernel.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from conftest import to_oracle_config

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cfg(**kw):
    from mattohf_gb300 import RunConfig
    base = dict(acell=9.0, NG=64, NK=5, NB=3, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    base.update(kw)
    return RunConfig(**base)


def _fields(nt=4):
    A = 0.02 * np.sin(0.7 * np.arange(1, nt + 1))
    Aave = np.concatenate([0.5 * A[:1], 0.5 * (A[1:] + A[:-1])])
    return A, Aave


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("NG,NK", [(64, 5), (128, 4), (256, 3)])
def test_hpsi_kslice_rows_match_full_apply(built_lib, NG, NK):
    from mattohf_gb300 import Context
    from mattohf_gb300.sharded import DeviceBackend
    cfg = _cfg(NG=NG, NK=NK)
    rng = np.random.default_rng(7)
    u = rng.standard_normal((NK, 3, NG)) + 1j * rng.standard_normal((NK, 3, NG))
    w = rng.standard_normal((NK, 2, NG)) + 1j * rng.standard_normal((NK, 2, NG))
    A = 0.13
    be = DeviceBackend(cfg)
    try:
        ctx = be.ctx
        full = {0: ctx.ubkwbk_hwbk(u, w, A), 1: ctx.ubkwbk_vFwbk(u, w), 2: ctx.ubk_tubk(w, A)}
        uocc = torch.from_numpy(np.ascontiguousarray(u[:, :2])).cuda()
        for k0, nkl in [(0, NK), (0, 1), (NK - 1, 1), (1, NK - 1)]:
            ws = torch.from_numpy(np.ascontiguousarray(w[k0:k0 + nkl])).cuda()
            for term in (0, 1, 2):
                got = be.hpsi_kslice(uocc, k0, ws, A, term).cpu().numpy()
                assert _rel(got, full[term][k0:k0 + nkl]) <= 1e-12, (k0, nkl, term)
    finally:
        be.close()


def test_observables_kslice_sum_to_whole(built_lib):
    from mattohf_gb300.sharded import DeviceBackend
    cfg = _cfg()
    be = DeviceBackend(cfg)
    try:
        ctx = be.ctx
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        u = ctx.get_orbitals()
        A = 0.05
        obs = ctx.observables(A)
        uocc = torch.from_numpy(np.ascontiguousarray(u[:, :cfg.NBocc])).cuda()
        tot = np.zeros(3)
        for k0, nkl in [(0, 2), (2, 3)]:
            p, s = be.observables_kslice(uocc, k0, torch.from_numpy(np.ascontiguousarray(u[k0:k0 + nkl])).cuda(), A)
            tot += p
        assert abs(s[0] - obs["Nele"]) <= 1e-12 * abs(obs["Nele"])
        assert abs(tot[0] + s[1] + s[2] + tot[2] - obs["Etot"]) <= 1e-12 * abs(obs["Etot"])
        assert abs(tot[1] - obs["Je"]) <= 1e-12 * max(1.0, abs(obs["Je"]))
    finally:
        be.close()


def test_sharded_single_rank_matches_rk4_run(built_lib):
    from mattohf_gb300 import Context
    from mattohf_gb300.sharded import DeviceBackend, ShardedRun
    cfg = _cfg()
    A, Aave = _fields()
    dt = 0.004
    with Context(cfg) as c:
        c.Init_wf()
        c.Gram_Schmidt()
        u0 = c.get_orbitals()
        E0, J0, N0 = c.rk4_run(A, Aave, dt)
        uf = c.get_orbitals()
    be = DeviceBackend(cfg)
    try:
        run = ShardedRun(cfg, be)
        run.set_orbitals(u0)
        E, J, N = run.rk4_run(A, Aave, dt)
        assert _rel(E, E0) <= 1e-12
        assert np.max(np.abs(J - J0)) <= 1e-12 * max(1.0, np.max(np.abs(J0)))
        assert _rel(N, N0) <= 1e-12
        assert _rel(run.get_orbitals(), uf) <= 1e-11
    finally:
        be.close()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, u0, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    from mattohf_gb300.sharded import DeviceBackend, ShardedRun
    dist.init_process_group("gloo", rank=rank, world_size=world)
    be = DeviceBackend(_cfg())
    try:
        run = ShardedRun(_cfg(), be)
        run.set_orbitals(u0)
        A, Aave = _fields()
        E, J, N = run.rk4_run(A, Aave, 0.004)
        q.put((rank, E, J, N, run.get_orbitals()))
    finally:
        be.close()
        dist.destroy_process_group()


def test_two_ranks_on_one_gpu_match_single_context_and_oracle(built_lib):
    import dataclasses
    import torch.multiprocessing as mp
    from mattohf_gb300 import Context
    from oracle import mattohf_oracle as O
    cfg = _cfg()
    A, Aave = _fields()
    with Context(cfg) as c:
        c.Init_wf()
        c.Gram_Schmidt()
        u0 = c.get_orbitals()
        E0, J0, N0 = c.rk4_run(A, Aave, 0.004)
    S = O.make_system(to_oracle_config(dataclasses.replace(cfg, dt=0.004)))
    ref = O.rt_calculation(S, u0, nt=A.size, A=A, Aave=Aave)
    mctx = mp.get_context("spawn")
    q = mctx.Queue()
    port = _free_port()
    procs = [mctx.Process(target=_worker, args=(r, 2, port, u0, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(2)]
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for _, E, J, N, u in res:
        assert _rel(E, E0) <= 1e-12
        assert np.max(np.abs(J - J0)) <= 1e-12 * max(1.0, np.max(np.abs(J0)))
        assert _rel(N, N0) <= 1e-12
        assert _rel(E, ref.Etot) <= 1e-10
        assert np.max(np.abs(J - ref.Jtot)) <= 1e-10 * max(1.0, np.max(np.abs(ref.Jtot)))
        assert _rel(u, ref.ubk) <= 1e-10
