"""Run configuration, ``input.dat`` parser and vector-potential construction.

Mirrors the reference's keyword input (``Read_input``, src/mATTOHF.f90:198-272),
its defaults (src/Global_variables.f90:7-26) and ``Define_Afield``
(src/RT_calculation.f90:175-244), on the host.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

# src/Constants.f90:5-18
PI = 4.0 * math.atan(1.0)
HARTREE = 27.2116
ATOMTIME = 0.02419
ATOMFIELD = 514.2
ATOMFLUENCE = 3.509e16 * ATOMTIME * 1.0e-15


@dataclasses.dataclass
class RunConfig:
    """The reference's global inputs (GV:7-26 defaults) for one run."""
    acell: float = 10.0
    NG: int = 64
    NK: int = 8
    NB: int = 2
    NBocc: int = 2
    Zeff: List[float] = dataclasses.field(default_factory=lambda: [2.0])
    alpha: List[float] = dataclasses.field(default_factory=lambda: [1.0])
    Rion: List[float] = dataclasses.field(default_factory=lambda: [0.5])
    Kion: List[int] = dataclasses.field(default_factory=lambda: [1])
    functional: str = "HF"
    sys_name: str = ""
    Nscf: int = 100
    NCG: int = 5
    NT: int = 2000
    dt: float = 0.5
    Nomega: int = 4000
    omegaM: float = 4.0
    field_option: str = "LP"
    dAc: float = float(np.float32(0.0001))  # single-precision default literal (GV:19)
    omegac: float = 1.55     # eV
    Tpulse: float = 16.0     # fs
    phiCEP: float = 0.5      # units of 2 pi
    nenvelope: int = 4
    E0: float = 1.0          # V/nm

    @staticmethod
    def from_pulse(A0: float, w: float, T: float, **kw) -> "RunConfig":
        """Map A(t) = A0 sin^2(pi t/T) sin(w t) [a.u.] onto the reference's LP inputs.

        nenvelope=2; omegac = w*Hartree [eV]; Tpulse = T*Atomtime [fs];
        E0 = A0*w*Atomfield [V/nm]; phiCEP = w*T/(4 pi) mod 1 so that
        sin(w(t - T/2) + 2 pi phiCEP) = sin(w t).
        """
        cfg = RunConfig(**kw)
        cfg.field_option = "LP"
        cfg.nenvelope = 2
        cfg.omegac = w * HARTREE
        cfg.Tpulse = T * ATOMTIME
        cfg.E0 = A0 * w * ATOMFIELD
        cfg.phiCEP = math.fmod(w * T / (4.0 * PI), 1.0)
        return cfg


def _token(line: str) -> Optional[str]:
    s = line.strip()
    if not s:
        return None
    if s[0] in "'\"":
        end = s.find(s[0], 1)
        return s[1:end] if end > 0 else s[1:]
    for i, ch in enumerate(s):
        if ch in " \t,/":
            return s[:i]
    return s


def _items(lines, pos, n):
    out = []
    while len(out) < n:
        if pos >= len(lines):
            raise EOFError("input ended inside a read")
        rec = lines[pos].strip()
        pos += 1
        if not rec:
            continue
        for t in rec.replace(",", " ").split():
            if t == "/":
                break
            out.append(t.strip("'\""))
            if len(out) == n:
                break
    return out, pos


def _real(t: str) -> float:
    return float(t.replace("d", "e").replace("D", "e"))


def read_input(path: str) -> RunConfig:
    """Keyword file reader with the reference's list-directed semantics.

    Each key's value is read from the following record(s); unknown records
    are skipped, so only the first value after a key counts.  ``functional``
    has no case in the reference reader and keeps its default.
    """
    cfg = RunConfig()
    with open(path) as fh:
        lines = fh.read().splitlines()
    ints = {"NB", "NBocc", "NG", "NK", "Nscf", "NCG", "NT", "Nomega", "nenvelope"}
    reals = {"acell", "dt", "omegaM", "dAc", "omegac", "Tpulse", "phiCEP", "E0"}
    pos = 0
    while pos < len(lines):
        key = _token(lines[pos])
        pos += 1
        if key is None:
            continue
        if key in ints:
            (v,), pos = _items(lines, pos, 1)
            setattr(cfg, key, int(v))
        elif key in reals:
            (v,), pos = _items(lines, pos, 1)
            setattr(cfg, key, _real(v))
        elif key in ("sys_name", "field_option"):
            while pos < len(lines) and _token(lines[pos]) is None:
                pos += 1
            v = _token(lines[pos]) or ""
            pos += 1
            setattr(cfg, key, v[:2] if key == "field_option" else v)
        elif key in ("dir_name", "DFT_option", "TD_option", "Band_option"):
            _, pos = _items(lines, pos, 1)
        elif key == "atoms":
            (ns,), pos = _items(lines, pos, 1)
            z, pos = _items(lines, pos, int(ns))
            a, pos = _items(lines, pos, int(ns))
            (ni,), pos = _items(lines, pos, 1)
            R, K = [], []
            for _ in range(int(ni)):
                (r, k), pos = _items(lines, pos, 2)
                R.append(_real(r))
                K.append(int(k))
            cfg.Zeff = [_real(x) for x in z]
            cfg.alpha = [_real(x) for x in a]
            cfg.Rion, cfg.Kion = R, K
    return cfg


def _powi(x: float, m: int) -> float:
    """x**m for integer m by square-and-multiply (how x**n is evaluated in Fortran)."""
    n = abs(m)
    y = x if n % 2 else 1.0
    n >>= 1
    while n:
        x = x * x
        if n % 2:
            y = y * x
        n >>= 1
    return 1.0 / y if m < 0 else y


def define_afield(cfg: RunConfig, nt: Optional[int] = None):
    """(time, A, Aave, E) of ``Define_Afield`` (src/RT_calculation.f90:175-244)."""
    NT = cfg.NT if nt is None else nt
    dt = cfg.dt
    time = dt * np.arange(NT, dtype=np.float64)
    A = np.zeros(NT)
    if cfg.field_option == "LR":
        A[:] = cfg.dAc
    elif cfg.field_option == "LP":
        omegac = cfg.omegac / HARTREE
        Tpulse = cfg.Tpulse / ATOMTIME
        E0 = cfg.E0 / ATOMFIELD
        Aamp = E0 / omegac
        NTpulse = int(min(Tpulse / dt, float(NT)))
        for it in range(NTpulse):
            t = time[it]
            A[it] = Aamp * math.sin(omegac * (t - 0.5 * Tpulse) + 2.0 * PI * cfg.phiCEP) \
                * _powi(math.sin(PI * t / Tpulse), cfg.nenvelope)
    else:
        raise ValueError("field_option must be 'LR' or 'LP'")
    Aave = np.empty(NT)
    E = np.empty(NT)
    if NT:
        Aave[0] = 0.5 * (A[0] + 0.0)
        Aave[1:] = 0.5 * (A[1:] + A[:-1])
        E[0] = -(A[0] - 0.0) / dt
        E[1:] = -(A[1:] - A[:-1]) / dt
    return time, A, Aave, E


def aave_from_samples(A: np.ndarray) -> np.ndarray:
    """Aave(it) = (A(it)+A(it-1))/2 with A(0)=0 (RT:227-230), for a tabulated A."""
    A = np.asarray(A, dtype=np.float64)
    Aave = np.empty_like(A)
    if A.size:
        Aave[0] = 0.5 * (A[0] + 0.0)
        Aave[1:] = 0.5 * (A[1:] + A[:-1])
    return Aave


def dipole_from_current(J: np.ndarray, J0: float, dt: float) -> np.ndarray:
    """Dipole P(t_i) = -int_0^{t_i} J dt' by the trapezoid rule on the RT time
    grid t_i = (i+1) dt, with J(0) = J0 (the current of the initial state).

    An extension: the reference writes Etot, Nele, Jtot, E and A
    (src/RT_calculation.f90:52-53) and no dipole, so P is pinned only through J.
    """
    J = np.asarray(J, dtype=np.float64)
    P = np.empty_like(J)
    acc = 0.0
    prev = float(J0)
    for i in range(J.size):
        acc -= 0.5 * dt * (prev + J[i])
        P[i] = acc
        prev = J[i]
    return P
