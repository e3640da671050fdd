"""One real-time run split over ranks by output k-point.

The reference distributes its exchange over MPI ranks by ranges of (k, k')
pairs (the NKK split, src/Initialization.f90:64-76, used by the pair loop at
src/Functions.f90:247) and all-reduces the whole NG x NB x NK result inside
every h-apply (src/Functions.f90:258).  Here each rank owns whole output
k-points [k0, k0 + nkl) of the state.  Per h-apply the ranks all-gather the
occupied orbitals (NK x NBocc x NG complex128, the only exchange step), then
each rank applies the full h to its own rows with no reduction of the result.
The density, the Hartree potential and the density scalars are recomputed on
every rank from the gathered orbitals.  Observables take one all-reduce of
three scalars (the slices' Ekin, Je and Ex contributions).

Compute goes through a backend with two calls, ``hpsi_kslice`` and
``observables_kslice``; :class:`DeviceBackend` is the C ABI
(``mattohf_hpsi_kslice_device`` / ``mattohf_observables_kslice_device``) on
this process's GPU.  Communication is ``torch.distributed``: NCCL on device
tensors, or gloo through host copies.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np
import torch
import torch.distributed as dist

from . import _capi
from .api import Context, MattohfError
from .inputs import RunConfig


def k_partition(NK: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous balanced split of the k-points: (first k-point, count)."""
    base, rem = divmod(NK, world)
    nkl = base + (1 if rank < rem else 0)
    k0 = rank * base + min(rank, rem)
    return k0, nkl


class DeviceBackend:
    """The k-slice entry points of the C ABI on one GPU (complex128 device tensors)."""

    def __init__(self, cfg: RunConfig, device: int = 0):
        self.ctx = Context(cfg, device=device)
        self.lib = self.ctx.lib
        self.device = torch.device("cuda", device)

    def close(self):
        self.ctx.close()

    def _sync_torch(self):
        torch.cuda.current_stream(self.device).synchronize()

    def hpsi_kslice(self, uocc: torch.Tensor, k0: int, w: torch.Tensor, A: float, term: int = 0) -> torch.Tensor:
        uocc, w = uocc.contiguous(), w.contiguous()
        out = torch.empty_like(w)
        self._sync_torch()
        self.ctx._check(self.lib.mattohf_hpsi_kslice_device(
            self.ctx.h, C.c_void_p(uocc.data_ptr()), k0, w.shape[0], C.c_void_p(w.data_ptr()), w.shape[1],
            float(A), term, C.c_void_p(out.data_ptr())))
        self.ctx._check(self.lib.mattohf_synchronize(self.ctx.h))
        return out

    def observables_kslice(self, uocc: torch.Tensor, k0: int, u: torch.Tensor, A: float):
        uocc, u = uocc.contiguous(), u.contiguous()
        partial, scal = np.empty(3), np.empty(3)
        self._sync_torch()
        D = C.POINTER(C.c_double)
        self.ctx._check(self.lib.mattohf_observables_kslice_device(
            self.ctx.h, C.c_void_p(uocc.data_ptr()), k0, u.shape[0], C.c_void_p(u.data_ptr()), float(A),
            partial.ctypes.data_as(D), scal.ctypes.data_as(D)))
        return partial, scal


class ShardedRun:
    """A run whose state is split by k-point over the ranks of ``group``.

    ``backend`` provides the per-rank compute on tensors of ``backend.device``.
    Without an initialised process group the run has one rank.
    """

    def __init__(self, cfg: RunConfig, backend, group=None):
        self.cfg = cfg
        self.backend = backend
        self.group = group
        self.dist = dist.is_available() and dist.is_initialized()
        self.rank = dist.get_rank(group) if self.dist else 0
        self.world = dist.get_world_size(group) if self.dist else 1
        self.NG, self.NK, self.NB, self.NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
        if self.NK < self.world:
            raise ValueError(f"NK={self.NK} k-points cannot be split over {self.world} ranks")
        self.k0, self.nkl = k_partition(self.NK, self.world, self.rank)
        self.parts = [k_partition(self.NK, self.world, r) for r in range(self.world)]
        self.kmax = max(n for _, n in self.parts)
        self.device = backend.device
        # NCCL gathers device tensors; every other backend goes through host memory
        self.comm_device = self.device
        if self.dist and dist.get_backend(group) != "nccl":
            self.comm_device = torch.device("cpu")
        self.u = torch.zeros((self.nkl, self.NB, self.NG), dtype=torch.complex128, device=self.device)

    # -- state --------------------------------------------------------------
    def set_orbitals(self, ubk):
        """Keep this rank's k-points of the full (NK, NB, NG) state."""
        ubk = np.ascontiguousarray(ubk, dtype=np.complex128)
        if ubk.shape != (self.NK, self.NB, self.NG):
            raise ValueError(f"expected shape {(self.NK, self.NB, self.NG)}, got {ubk.shape}")
        self.u = torch.from_numpy(ubk[self.k0:self.k0 + self.nkl].copy()).to(self.device)

    def _gather_k(self, v: torch.Tensor) -> torch.Tensor:
        """All k-point slices of v (nkl, nb, NG) concatenated in k order."""
        if self.world == 1:
            return v.contiguous()
        nb = v.shape[1]
        pad = torch.zeros((self.kmax, nb, self.NG), dtype=v.dtype, device=self.comm_device)
        pad[:self.nkl] = v.to(self.comm_device)
        bufs = [torch.empty_like(pad) for _ in range(self.world)]
        dist.all_gather(bufs, pad, group=self.group)
        full = torch.cat([bufs[r][:n] for r, (_, n) in enumerate(self.parts)], dim=0)
        return full.to(self.device).contiguous()

    def gather_occupied(self, v: torch.Tensor) -> torch.Tensor:
        """Occupied orbitals of every k-point, (NK, NBocc, NG): the per-apply exchange step."""
        return self._gather_k(v[:, :self.NBocc])

    def get_orbitals(self) -> np.ndarray:
        """The full (NK, NB, NG) state, on every rank."""
        return self._gather_k(self.u).cpu().numpy()

    # -- operators ----------------------------------------------------------
    def hpsi(self, v: torch.Tensor, A: float) -> torch.Tensor:
        """h[v](A) v on this rank's k-points (ubkwbk_hwbk with w = u, F:187-209)."""
        return self.backend.hpsi_kslice(self.gather_occupied(v), self.k0, v, A, 0)

    def rk4_step(self, Aave: float, A: float, dt: float):
        """RT_RK4_ubk (src/RT_calculation.f90:154-173): stage fields A(it-1), Aave, Aave, A(it)."""
        Am = 2.0 * Aave - A
        u = self.u
        k1 = -1j * self.hpsi(u, Am)
        k2 = -1j * self.hpsi(u + (0.5 * dt) * k1, Aave)
        k3 = -1j * self.hpsi(u + (0.5 * dt) * k2, Aave)
        k4 = -1j * self.hpsi(u + dt * k3, A)
        s = k1 + 2.0 * k2
        s = s + 2.0 * k3
        s = s + k4
        self.u = u + s * (dt / 6.0)

    def observables(self, A: float):
        """(Etot, Je, Nele) of the whole state (F:74-91, F:289-318, RT:43-47)."""
        partial, scal = self.backend.observables_kslice(self.gather_occupied(self.u), self.k0, self.u, A)
        if self.world > 1:
            t = torch.tensor(partial, dtype=torch.float64, device=self.comm_device)
            dist.all_reduce(t, group=self.group)
            partial = t.cpu().numpy()
        Etot = partial[0] + scal[1] + scal[2] + partial[2]
        return float(Etot), float(partial[1]), float(scal[0])

    def rk4_run(self, A, Aave, dt: float):
        """The RT loop (RT:38-60): RK4 step, then Etot, Je, Nele of every step."""
        A = np.asarray(A, dtype=np.float64)
        Aave = np.asarray(Aave, dtype=np.float64)
        nt = A.size
        E, J, N = np.empty(nt), np.empty(nt), np.empty(nt)
        for it in range(nt):
            self.rk4_step(float(Aave[it]), float(A[it]), dt)
            E[it], J[it], N[it] = self.observables(float(A[it]))
            if not (np.isfinite(E[it]) and np.isfinite(J[it]) and np.isfinite(N[it])):
                raise MattohfError(_capi.ERR_NONFINITE, f"non-finite observables at step {it}")
        return E, J, N
