"""Host-side mirror of the reference's hot-path interface over the C ABI.

Names follow the reference's Fortran procedures (src/Functions.f90,
src/RT_calculation.f90, src/GS_calculation.f90); arrays are numpy complex128
with shape (NK, NB, NG) — the bytes of Fortran ``ubk(1:NG,1:NB,1:NK)``.
Every call goes through ``libmattohf.so``; errors raise ``MattohfError``
carrying the library's status code and message.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import _capi
from .inputs import RunConfig

_D = C.POINTER(C.c_double)


class MattohfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mattohf status {status}: {msg}")
        self.status = status


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(_D)


def _c128(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class Context:
    """One device-resident run (``mattohf_ctx``)."""

    def __init__(self, cfg: RunConfig, device: int = 0):
        self.lib = _capi.load()
        self.cfg = cfg
        self.NG, self.NK, self.NB, self.NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
        z = np.ascontiguousarray(cfg.Zeff, dtype=np.float64)
        al = np.ascontiguousarray(cfg.alpha, dtype=np.float64)
        R = np.ascontiguousarray(cfg.Rion, dtype=np.float64)
        K = np.ascontiguousarray(cfg.Kion, dtype=np.int32)
        self._keep = (z, al, R, K)
        c = _capi.mattohf_config()
        c.NG, c.NK, c.NB, c.NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
        c.acell = cfg.acell
        c.functional_hf = 1 if cfg.functional.strip() == "HF" else 0
        c.device = device
        c.nspecies = z.size
        c.Zeff = _dp(z)
        c.alpha = _dp(al)
        c.nion = R.size
        c.Rion = _dp(R)
        c.Kion = K.ctypes.data_as(C.POINTER(C.c_int))
        h = C.c_void_p()
        st = self.lib.mattohf_create(C.byref(c), C.byref(h))
        if st != _capi.OK:
            raise MattohfError(st, self.lib.mattohf_status_string(st).decode())
        self.h = h

    # -- plumbing -----------------------------------------------------------
    def _check(self, st: int):
        if st != _capi.OK:
            raise MattohfError(st, self.lib.mattohf_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.mattohf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_option(self, opt: int, value: int):
        self._check(self.lib.mattohf_set_option(self.h, opt, int(value)))

    @property
    def shape(self):
        return (self.NK, self.NB, self.NG)

    # -- tables -------------------------------------------------------------
    def grids(self) -> Dict[str, np.ndarray]:
        rx, Gx, kx, cell = np.empty(self.NG), np.empty(self.NG), np.empty(self.NK), np.empty(3)
        self._check(self.lib.mattohf_get_grids(self.h, _dp(rx), _dp(Gx), _dp(kx), _dp(cell)))
        return {"rx": rx, "Gx": Gx, "kx": kx, "vcell": cell[0], "dvcell": cell[1], "bx": cell[2]}

    def coulomb(self):
        vCG = np.empty(self.NG)
        vCq = np.empty((2 * self.NK - 1, self.NG))
        self._check(self.lib.mattohf_get_coulomb(self.h, _dp(vCG), _dp(vCq)))
        return vCG, vCq

    def vck(self, q) -> np.ndarray:
        """k_vCk(q) of this cell (src/Functions.f90:33-52) at arbitrary arguments."""
        q = np.ascontiguousarray(q, dtype=np.float64).ravel()
        out = np.empty_like(q)
        self._check(self.lib.mattohf_vck(self.h, _dp(q), q.size, _dp(out)))
        return out

    @property
    def vion(self) -> np.ndarray:
        v = np.empty(self.NG)
        self._check(self.lib.mattohf_get_vion(self.h, _dp(v)))
        return v

    @vion.setter
    def vion(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._check(self.lib.mattohf_set_vion(self.h, _dp(v)))

    # -- state --------------------------------------------------------------
    def set_orbitals(self, ubk):
        u = _c128(ubk, self.shape)
        self._check(self.lib.mattohf_set_orbitals(self.h, _dp(u.view(np.float64))))

    def get_orbitals(self) -> np.ndarray:
        u = np.empty(self.shape, dtype=np.complex128)
        self._check(self.lib.mattohf_get_orbitals(self.h, _dp(u.view(np.float64))))
        return u

    ubk = property(get_orbitals, set_orbitals)

    def Init_wf(self):
        self._check(self.lib.mattohf_init_wf(self.h))

    def Gram_Schmidt(self):
        self._check(self.lib.mattohf_gram_schmidt(self.h))

    # -- operator kernels (src/Functions.f90) -----------------------------------
    def ubkwbk_hwbk(self, ubk, wbk, A: float) -> np.ndarray:
        """h[ubk](A) wbk; passing the same array twice applies h[u] u (symmetric exchange)."""
        u = _c128(ubk, self.shape)
        w = u if wbk is ubk else np.ascontiguousarray(wbk, dtype=np.complex128)
        nbw = w.shape[1]
        _c128(w, (self.NK, nbw, self.NG))
        out = np.empty_like(w)
        self._check(self.lib.mattohf_hpsi(self.h, _dp(u.view(np.float64)), _dp(w.view(np.float64)),
                                          nbw, float(A), _dp(out.view(np.float64))))
        return out

    def ubkwbk_vFwbk(self, ubk, wbk) -> np.ndarray:
        u = _c128(ubk, self.shape)
        w = u if wbk is ubk else np.ascontiguousarray(wbk, dtype=np.complex128)
        nbw = w.shape[1]
        out = np.empty_like(w)
        self._check(self.lib.mattohf_fock(self.h, _dp(u.view(np.float64)), _dp(w.view(np.float64)),
                                          nbw, _dp(out.view(np.float64))))
        return out

    def ubk_tubk(self, wbk, A: float) -> np.ndarray:
        w = np.ascontiguousarray(wbk, dtype=np.complex128)
        out = np.empty_like(w)
        self._check(self.lib.mattohf_kinetic(self.h, _dp(w.view(np.float64)), w.shape[1], float(A),
                                             _dp(out.view(np.float64))))
        return out

    def ubk_dns(self, ubk) -> np.ndarray:
        u = _c128(ubk, self.shape)
        d = np.empty(self.NG)
        self._check(self.lib.mattohf_density(self.h, _dp(u.view(np.float64)), _dp(d), None))
        return d

    def dns_vH_of(self, ubk) -> np.ndarray:
        """Hartree potential of the density of ``ubk`` (dns_vH(ubk_dns(ubk)))."""
        u = _c128(ubk, self.shape)
        vH = np.empty(self.NG)
        self._check(self.lib.mattohf_density(self.h, _dp(u.view(np.float64)), None, _dp(vH)))
        return vH

    def observables(self, A: float = 0.0) -> Dict[str, float]:
        """Ecomps/Etot (F:74-91, F:265-286), Je (F:289-318), Nele of the device orbitals."""
        ec = np.empty(4)
        et, je, ne = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.mattohf_observables(self.h, float(A), _dp(ec), C.byref(et), C.byref(je),
                                                 C.byref(ne)))
        return {"Etot": et.value, "Ekin": ec[0], "Eion": ec[1], "EH": ec[2], "Exc": ec[3],
                "Je": je.value, "Nele": ne.value}

    def ubk_epsbk(self):
        eps = np.empty((self.NK, self.NB))
        err = np.empty((self.NK, self.NB))
        self._check(self.lib.mattohf_eps(self.h, _dp(eps), _dp(err)))
        return eps, err

    # -- propagation (src/RT_calculation.f90) ------------------------------------
    def RT_RK4_ubk(self, Aave: float, A: float, dt: float):
        self._check(self.lib.mattohf_rk4_step(self.h, float(Aave), float(A), float(dt)))

    def RT_TE_ubk(self, Aave: float, dt: float, variant: str = "TE"):
        """Taylor / predictor-corrector propagators (RT:72-151): 'TE', 'TEPC' or 'TEPC2'."""
        v = {"TE": 0, "TEPC": 1, "TEPC2": 2}[variant]
        self._check(self.lib.mattohf_te_step(self.h, v, float(Aave), float(dt)))

    def rk4_run(self, A, Aave, dt: float):
        """nt RK4 steps with per-step (Etot, Je, Nele) at A[it] (RT:38-60)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        Aave = np.ascontiguousarray(Aave, dtype=np.float64)
        nt = A.size
        E, J, N = np.empty(nt), np.empty(nt), np.empty(nt)
        st = self.lib.mattohf_rk4_run(self.h, nt, float(dt), _dp(A), _dp(Aave), _dp(E), _dp(J), _dp(N))
        self._check(st)
        return E, J, N

    def autotune(self, steps: int = 20) -> dict:
        """Time the tunable launch shapes on the current orbitals and keep the
        fastest (exchange tile, fused-stage CTAs per column, fused vs tiled
        stepping); the orbitals are restored.  Returns the choices and times."""
        out = (C.c_int * 3)()
        us = (C.c_double * 3)()
        self._check(self.lib.mattohf_autotune(self.h, int(steps), out, us))
        return {"sym_tile": out[0], "small_ctas": out[1], "small_stages": bool(out[2]),
                "exchange_us": us[0], "tiled_step_us": us[1], "fused_step_us": us[2]}

    def last_run_timing(self):
        r, f = C.c_double(), C.c_double()
        n = C.c_int()
        self._check(self.lib.mattohf_last_run_timing(self.h, C.byref(r), C.byref(f), C.byref(n)))
        return r.value, f.value, n.value

    # -- adjoint gradient (extension) -------------------------------------------
    def adjoint(self, A, dt: float, objective: str = "energy", ckpt_every: int = 0):
        """(L, dL/dA[n], dL/dvion[x]) of the absorbed energy or final current.

        Propagates the device orbitals nt = len(A) RK4 steps (they end at u_nt).
        """
        A = np.ascontiguousarray(A, dtype=np.float64)
        obj = {"energy": 0, "current": 1}[objective]
        L = C.c_double()
        g = np.empty(A.size)
        gv = np.empty(self.NG)
        self._check(self.lib.mattohf_adjoint(self.h, obj, A.size, float(dt), _dp(A), int(ckpt_every),
                                             C.byref(L), _dp(g), _dp(gv)))
        return L.value, g, gv

    def ion_param_grad(self, dLdvion) -> Dict[str, np.ndarray]:
        """Chain rule from dL/dvion on the grid to the ion-potential parameters
        (src/Prep_periodic_ion_potential.f90:10-20): dL/dZeff and dL/dalpha per
        species, dL/dRion per ion (reduced position)."""
        g = np.ascontiguousarray(dLdvion, dtype=np.float64)
        if g.shape != (self.NG,):
            raise ValueError(f"expected shape ({self.NG},), got {g.shape}")
        ns, ni = len(self.cfg.Zeff), len(self.cfg.Rion)
        dZ, da, dR = np.empty(ns), np.empty(ns), np.empty(ni)
        self._check(self.lib.mattohf_ion_param_grad(self.h, _dp(g), _dp(dZ), _dp(da), _dp(dR)))
        return {"Zeff": dZ, "alpha": da, "Rion": dR}

    def adjoint_timing(self):
        f, t = C.c_double(), C.c_double()
        self._check(self.lib.mattohf_adjoint_timing(self.h, C.byref(f), C.byref(t)))
        return f.value, t.value

    # -- ground state (src/GS_calculation.f90) -----------------------------------
    def GS_calculation(self, nscf: int, ncg: int) -> Dict[str, np.ndarray]:
        Et = np.empty(nscf + 1)
        Je = np.empty(max(nscf, 1))
        dd = np.empty(max(nscf, 1))
        eps = np.empty((self.NK, self.NB))
        err = np.empty((self.NK, self.NB))
        self._check(self.lib.mattohf_gs_run(self.h, int(nscf), int(ncg), _dp(Et), _dp(Je), _dp(dd),
                                             _dp(eps), _dp(err)))
        return {"Etot": Et, "Je": Je[:nscf], "dnsdiff": dd[:nscf], "epsbk": eps, "epserrorbk": err}

    def synchronize(self):
        self._check(self.lib.mattohf_synchronize(self.h))


class _Member(Context):
    """A run owned by a Batch: an ordinary context that the batch destroys."""

    def __init__(self, lib, handle, cfg):  # noqa: D401 - no mattohf_create here
        self.lib = lib
        self.cfg = cfg
        self.NG, self.NK, self.NB, self.NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
        self.h = C.c_void_p(handle)
        self._owned = False

    def close(self):
        self.h = None  # destroyed with the batch


class Batch:
    """Many independent runs advanced together (``mattohf_batch``).

    All runs share NG and have NB == NBocc; NK, acell, ions, dt and the
    vector potential differ per run.  ``batch[r]`` is run r's context.
    """

    def __init__(self, cfgs, device: int = 0):
        self.lib = _capi.load()
        self.cfgs = list(cfgs)
        keep = []
        arr = (_capi.mattohf_config * len(self.cfgs))()
        for c, cfg in zip(arr, self.cfgs):
            z = np.ascontiguousarray(cfg.Zeff, dtype=np.float64)
            al = np.ascontiguousarray(cfg.alpha, dtype=np.float64)
            R = np.ascontiguousarray(cfg.Rion, dtype=np.float64)
            K = np.ascontiguousarray(cfg.Kion, dtype=np.int32)
            keep.append((z, al, R, K))
            c.NG, c.NK, c.NB, c.NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
            c.acell = cfg.acell
            c.functional_hf = 1 if cfg.functional.strip() == "HF" else 0
            c.device = device
            c.nspecies, c.Zeff, c.alpha = z.size, _dp(z), _dp(al)
            c.nion, c.Rion, c.Kion = R.size, _dp(R), K.ctypes.data_as(C.POINTER(C.c_int))
        h = C.c_void_p()
        st = self.lib.mattohf_batch_create(len(self.cfgs), arr, C.byref(h))
        if st != _capi.OK:
            raise MattohfError(st, self.lib.mattohf_status_string(st).decode())
        self.h = h
        self.members = [_Member(self.lib, self.lib.mattohf_batch_run(h, r), cfg)
                        for r, cfg in enumerate(self.cfgs)]

    def __len__(self):
        return len(self.members)

    def __getitem__(self, r) -> Context:
        return self.members[r]

    def _check(self, st):
        if st != _capi.OK:
            raise MattohfError(st, self.lib.mattohf_batch_last_error(self.h).decode())

    def autotune(self, steps: int = 10) -> dict:
        """Time every exchange tile over ensemble steps on the runs' current
        orbitals (restored afterwards) and keep the fastest."""
        tile = C.c_int()
        us = C.c_double()
        self._check(self.lib.mattohf_batch_autotune(self.h, int(steps), C.byref(tile), C.byref(us)))
        return {"sym_tile": tile.value, "step_us": us.value}

    def rk4_run(self, A, Aave, dt):
        """A, Aave: (nruns, nt); dt: scalar or (nruns,).  Returns (Etot, Je, Nele), each (nruns, nt)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        Aave = np.ascontiguousarray(Aave, dtype=np.float64)
        R, nt = A.shape
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (R,)))
        E, J, N = np.empty((R, nt)), np.empty((R, nt)), np.empty((R, nt))
        self._check(self.lib.mattohf_batch_rk4_run(self.h, nt, _dp(dts), _dp(A), _dp(Aave), _dp(E), _dp(J),
                                                    _dp(N)))
        return E, J, N

    def last_run_ms(self) -> float:
        ms = C.c_double()
        self._check(self.lib.mattohf_batch_last_run_ms(self.h, C.byref(ms)))
        return ms.value

    def adjoint(self, A, dt, objective: str = "energy", ckpt_every: int = 0):
        """Every member's (L, dL/dA[n], dL/dvion[x]) from its current orbitals
        (mattohf_batch_adjoint).  A: (nruns, nt); dt: scalar or (nruns,).
        Returns L (nruns,), dLdA (nruns, nt), dLdvion (nruns, NG)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        R, nt = A.shape
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (R,)))
        obj = {"energy": 0, "current": 1}[objective]
        L, g, gv = np.empty(R), np.empty((R, nt)), np.empty((R, self.cfgs[0].NG))
        self._check(self.lib.mattohf_batch_adjoint(self.h, obj, nt, _dp(dts), _dp(A), int(ckpt_every), _dp(L),
                                                    _dp(g), _dp(gv)))
        return L, g, gv

    def set_option(self, opt: int, value: int):
        self._check(self.lib.mattohf_batch_set_option(self.h, opt, int(value)))

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.lib.mattohf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
