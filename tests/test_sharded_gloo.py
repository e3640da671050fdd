"""A run split by output k-point over CPU ranks (gloo), against the oracle.

The per-rank compute here is a stand-in built on the oracle (CPU, test
infrastructure).  Under test is the product's host logic in
mattohf_gb300/sharded.py: the k-point partition, the per-apply all-gather of
the occupied orbitals, the RK4 stage fields and the cross-rank reduction of
the observables.  The GPU compute behind the same calls is tested in
tests/test_gpu_sharded.py.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from conftest import to_oracle_config

torch = pytest.importorskip("torch")

NT = 3
DT = 0.004


def _cfg():
    from mattohf_gb300 import RunConfig
    # NK = 5 splits unevenly; one unoccupied band exercises the NBocc gather
    return RunConfig(acell=9.0, NG=32, NK=5, NB=3, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])


def _fields():
    A = np.array([0.01, 0.025, 0.02])
    Aave = np.concatenate([0.5 * A[:1], 0.5 * (A[1:] + A[:-1])])
    return A, Aave


class OracleSliceBackend:
    """The two k-slice calls of the C ABI, restated on the oracle (CPU tensors)."""

    def __init__(self, S):
        self.S = S
        self.device = torch.device("cpu")

    def _pad(self, uocc):
        S = self.S
        u = np.zeros((S.NK, S.NB, S.NG), dtype=np.complex128)
        u[:, :S.NBocc] = uocc.numpy()
        return u

    def _rows(self, k0, v):
        S = self.S
        w = np.zeros((S.NK, v.shape[1], S.NG), dtype=np.complex128)
        w[k0:k0 + v.shape[0]] = v.numpy()
        return w

    def hpsi_kslice(self, uocc, k0, w, A, term=0):
        from oracle import mattohf_oracle as O
        u, wf = self._pad(uocc), self._rows(k0, w)
        h = {0: lambda: O.ubkwbk_hwbk(self.S, u, wf, A), 1: lambda: O.ubkwbk_vFwbk(self.S, u, wf),
             2: lambda: O.ubk_tubk(self.S, wf, A)}[term]()
        return torch.from_numpy(h[k0:k0 + w.shape[0]].copy())

    def observables_kslice(self, uocc, k0, uloc, A):
        from oracle import mattohf_oracle as O
        S = self.S
        u, us = self._pad(uocc), self._rows(k0, uloc)
        dns = O.ubk_dns(S, u)
        vF = O.ubkwbk_vFwbk(S, u, us)
        ex = 0.0
        for ik in range(k0, k0 + uloc.shape[0]):
            for ib in range(S.NBocc):
                ex += S.occbk[ik, ib] * np.sum(np.conj(us[ik, ib]) * vF[ik, ib]).real * S.dvcell
        partial = np.array([O.ubk_Ekin(S, us, A), O.ubk_Je(S, us, A), 0.5 * ex if S.hf else 0.0])
        scal = np.array([np.sum(dns) * S.dvcell, O.dns_Eion(S, dns), O.dns_EH(S, dns)])
        return partial, scal


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    from oracle import mattohf_oracle as O
    from mattohf_gb300.sharded import ShardedRun
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg = _cfg()
        S = O.make_system(to_oracle_config(cfg))
        u0 = O.gram_schmidt(S, O.init_wf(S))
        run = ShardedRun(cfg, OracleSliceBackend(S))
        run.set_orbitals(u0)
        A, Aave = _fields()
        E, J, N = run.rk4_run(A, Aave, DT)
        u = run.get_orbitals()
        q.put((rank, run.k0, run.nkl, E, J, N, u))
    finally:
        dist.destroy_process_group()


def _reference():
    from oracle import mattohf_oracle as O
    import dataclasses
    cfg = dataclasses.replace(_cfg(), dt=DT)
    S = O.make_system(to_oracle_config(cfg))
    u0 = O.gram_schmidt(S, O.init_wf(S))
    A, Aave = _fields()
    return O.rt_calculation(S, u0, nt=NT, A=A, Aave=Aave)


def test_k_partition_covers_every_k_point_once():
    from mattohf_gb300.sharded import k_partition
    for NK in (1, 2, 5, 8, 64, 127):
        for world in range(1, min(NK, 9) + 1):
            parts = [k_partition(NK, world, r) for r in range(world)]
            assert parts[0][0] == 0
            for (a0, n0), (a1, _) in zip(parts, parts[1:]):
                assert a0 + n0 == a1
            assert sum(n for _, n in parts) == NK
            assert max(n for _, n in parts) - min(n for _, n in parts) <= 1


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_rk4_matches_oracle(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in range(world)), key=lambda t: t[0])
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    ref = _reference()
    expect = {2: [(0, 3), (3, 2)], 3: [(0, 2), (2, 2), (4, 1)]}[world]
    assert [(r[1], r[2]) for r in res] == expect
    for _, _, _, E, J, N, u in res:
        assert np.max(np.abs(E - ref.Etot)) <= 1e-12 * np.max(np.abs(ref.Etot))
        assert np.max(np.abs(J - ref.Jtot)) <= 1e-12 * max(1.0, np.max(np.abs(ref.Jtot)))
        assert np.max(np.abs(N - ref.Nele)) <= 1e-12 * np.max(np.abs(ref.Nele))
        assert np.max(np.abs(u - ref.ubk)) <= 1e-12 * np.max(np.abs(ref.ubk))


def test_sharded_single_rank_matches_oracle():
    from oracle import mattohf_oracle as O
    from mattohf_gb300.sharded import ShardedRun
    cfg = _cfg()
    S = O.make_system(to_oracle_config(cfg))
    run = ShardedRun(cfg, OracleSliceBackend(S))
    assert (run.k0, run.nkl, run.world) == (0, 5, 1)
    run.set_orbitals(O.gram_schmidt(S, O.init_wf(S)))
    A, Aave = _fields()
    E, J, N = run.rk4_run(A, Aave, DT)
    ref = _reference()
    assert np.max(np.abs(E - ref.Etot)) <= 1e-12 * np.max(np.abs(ref.Etot))
    assert np.max(np.abs(J - ref.Jtot)) <= 1e-12 * max(1.0, np.max(np.abs(ref.Jtot)))
