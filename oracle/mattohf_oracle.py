"""CPU restatement of mATTOHF's hot path — TEST INFRASTRUCTURE ONLY.

This module is the oracle that the CUDA path is checked against.  Only the
test-suite, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import it, and only as the checker; the product path in
``mattohf_gb300`` never routes through it.

parity unpinned: the reference (Fortran 90 + MPI + FFTW3 + LAPACK) ships no
tests, golden vectors or fixtures, and it cannot be compiled here (no Fortran
compiler, no FFTW, no system LAPACK).  The restatement is therefore pinned by
physics known-answer tests instead (free-particle eigenvalues, the 2*K0(|q|)
limit of the soft-Coulomb transform, Hermiticity, particle number, gauge
covariance, RK4 order) which live in ``tests/test_oracle.py``.

Third-party arithmetic the reference links but does not vendor:
  * FFTW3 (unpinned OS build, ``src/make.inc:7``): ``dfftw_plan_dft_1d`` with
    FFTW_FORWARD (sign -1) / FFTW_BACKWARD (sign +1), both unnormalised
    (``src/Initialization.f90:271-272``).  Restated with ``numpy.fft`` using
    the same conventions (``fft`` / ``ifft(norm="forward")``).
  * LAPACK ZGESVD('O','N') (``src/GS_calculation.f90:162``) and
    ZHEEV('V','U') (``src/GS_calculation.f90:183,226``), unpinned.  Restated
    with ``scipy.linalg.lapack`` (the same LAPACK routines, from scipy's
    bundled OpenBLAS).

Layout: the reference stores ``ubk(1:NG,1:NB,1:NK)`` column-major; numpy
arrays here have shape ``(NK, NB, NG)`` C-order, i.e. the same bytes.
Loop orders that set floating-point rounding (density ig->ik->ib, Fock
kk->ibr->ibc accumulation) follow the reference.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

# ---------------------------------------------------------------------------
# Constants (src/Constants.f90:5-18)
# ---------------------------------------------------------------------------
PI = 4.0 * math.atan(1.0)
TPI = 2.0 * PI
FPI = 4.0 * PI
HARTREE = 27.2116          # eV
ATOMTIME = 0.02419         # fs
ATOMFIELD = 514.2          # V/nm
HALFEPSC = 3.509e16        # W/cm^2
ATOMFLUENCE = HALFEPSC * ATOMTIME * 1.0e-15


def _f32(x: float) -> float:
    """Value of a default-kind (single precision) Fortran literal."""
    return float(np.float32(x))


# ---------------------------------------------------------------------------
# Configuration (src/Global_variables.f90:7-26 defaults; parser mATTOHF.f90:198-272)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Config:
    acell: float = 10.0
    NG: int = 64
    NK: int = 8
    NB: int = 2
    NBocc: int = 2
    # atoms block (src/mATTOHF.f90:229-240): per-species charge and softening,
    # per-ion reduced position and 1-based species index
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
    dAc: float = _f32(0.0001)  # default literal is single precision (GV:19)
    omegac: float = 1.55       # eV
    Tpulse: float = 16.0       # fs
    phiCEP: float = 0.5        # units of 2*pi
    nenvelope: int = 4
    E0: float = 1.0            # V/nm

    @property
    def nion(self) -> int:
        return len(self.Rion)


def _fortran_token(line: str) -> Optional[str]:
    """First list-directed item of a record (quotes stripped), or None if blank."""
    s = line.strip()
    if not s:
        return None
    if s[0] in "'\"":
        q = s[0]
        end = s.find(q, 1)
        return s[1:end] if end > 0 else s[1:]
    for i, ch in enumerate(s):
        if ch in " \t,/":
            return s[:i]
    return s


def _fortran_items(lines, pos, n):
    """Read n list-directed items starting at record pos; returns (items, next pos).

    A list-directed READ consumes whole records and skips blank ones; items
    beyond n on the last record are discarded (src/mATTOHF.f90:208-267).
    """
    items = []
    while len(items) < n:
        if pos >= len(lines):
            raise EOFError("input ended inside a read")
        rec = lines[pos].strip()
        pos += 1
        if not rec:
            continue
        toks = rec.replace(",", " ").split()
        for t in toks:
            if t == "/":
                break
            items.append(t)
            if len(items) == n:
                break
    return items, pos


def _freal(t: str) -> float:
    return float(t.replace("d", "e").replace("D", "e"))


def _flogical(t: str) -> bool:
    t = t.strip(".").lower()
    return t.startswith("t")


def read_input(path: str) -> Config:
    """Keyword parser restated from ``Read_input`` (src/mATTOHF.f90:198-272).

    Unknown keys are skipped, so only the first value after each key is used;
    the ``functional`` key is not parsed (there is no case for it) and keeps its
    default 'HF'.
    """
    cfg = Config()
    with open(path) as fh:
        lines = fh.read().splitlines()
    pos = 0
    ints = {"NB", "NBocc", "NG", "NK", "Nscf", "NCG", "NT", "Nomega", "nenvelope"}
    reals = {"acell", "dt", "omegaM", "dAc", "omegac", "Tpulse", "phiCEP", "E0"}
    strs = {"sys_name": "sys_name", "field_option": "field_option"}
    while pos < len(lines):
        key = _fortran_token(lines[pos])
        pos += 1
        if key is None:
            continue
        if key in ints:
            (v,), pos = _fortran_items(lines, pos, 1)
            setattr(cfg, key, int(v))
        elif key in reals:
            (v,), pos = _fortran_items(lines, pos, 1)
            setattr(cfg, key, _freal(v))
        elif key in strs:
            while pos < len(lines) and _fortran_token(lines[pos]) is None:
                pos += 1
            v = _fortran_token(lines[pos]) or ""
            pos += 1
            if key == "field_option":
                v = v[:2]  # character(2)
            setattr(cfg, strs[key], v)
        elif key in ("dir_name", "DFT_option", "TD_option"):
            (_,), pos = _fortran_items(lines, pos, 1)
        elif key == "Band_option":
            (_,), pos = _fortran_items(lines, pos, 1)
        elif key == "atoms":
            (ns,), pos = _fortran_items(lines, pos, 1)
            ns = int(ns)
            z, pos = _fortran_items(lines, pos, ns)
            a, pos = _fortran_items(lines, pos, ns)
            (ni,), pos = _fortran_items(lines, pos, 1)
            ni = int(ni)
            R, K = [], []
            for _ in range(ni):
                (r, k), pos = _fortran_items(lines, pos, 2)
                R.append(_freal(r))
                K.append(int(k))
            cfg.Zeff = [_freal(x) for x in z]
            cfg.alpha = [_freal(x) for x in a]
            cfg.Rion, cfg.Kion = R, K
    return cfg


# ---------------------------------------------------------------------------
# FFT conventions (FFTW, unnormalised both ways)
# ---------------------------------------------------------------------------
def fftf(x, axis=-1):
    return np.fft.fft(x, axis=axis)


def fftb(x, axis=-1):
    return np.fft.ifft(x, axis=axis, norm="forward")


# ---------------------------------------------------------------------------
# Grids, tables, occupations (src/Initialization.f90:46-186)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class System:
    cfg: Config
    vcell: float
    dvcell: float
    bx: float
    rx: np.ndarray
    Gx: np.ndarray
    kx: np.ndarray
    occbk: np.ndarray      # (NK, NB)
    vCG: np.ndarray        # (NG,)
    vCGkk: Optional[np.ndarray]  # (NK*NK, NG), ikk = ikr*NK + ikc (0-based)
    vion: Optional[np.ndarray] = None

    @property
    def NG(self):
        return self.cfg.NG

    @property
    def NK(self):
        return self.cfg.NK

    @property
    def NB(self):
        return self.cfg.NB

    @property
    def NBocc(self):
        return self.cfg.NBocc

    @property
    def hf(self):
        return self.cfg.functional.strip() == "HF"


def k_vCk_count(acell: float, NG: int, NK: int) -> tuple:
    """dx and the trip count of ``Do While ((ix*dx) < (NK*acell))`` (F:42-48)."""
    dx = acell / float(NG) / 20.0
    lim = float(NK) * acell
    n = int(lim / dx) - 2
    n = max(n, 0)
    while float(n) * dx < lim:
        n += 1
    while n > 0 and float(n - 1) * dx >= lim:
        n -= 1
    return dx, n


def k_vCk(k, acell: float, NG: int, NK: int) -> np.ndarray:
    """Trapezoid transform of the soft-Coulomb kernel (src/Functions.f90:33-52).

    vCk(k) = 2*dx*sum_{ix=0}^{n-1} 0.5*(f(ix*dx)+f((ix+1)*dx)),
    f(x) = cos(k*x)/sqrt(x**2+1), summed in ix order like the Fortran loop.
    Vectorised over k; the ix summation is sequential (cumulative) per k.
    """
    k = np.atleast_1d(np.asarray(k, dtype=np.float64))
    dx, n = k_vCk_count(acell, NG, NK)
    x = np.arange(n + 1, dtype=np.float64) * dx
    den = np.sqrt(x * x + 1.0)
    out = np.empty(k.shape, dtype=np.float64)
    flat_k = k.reshape(-1)
    flat_o = out.reshape(-1)
    chunk = max(1, (1 << 22) // (n + 1))
    for s in range(0, flat_k.size, chunk):
        kk = flat_k[s:s + chunk, None]
        f = np.cos(kk * x[None, :]) / den[None, :]
        terms = 0.5 * (f[:, :-1] + f[:, 1:])
        # sequential left-to-right accumulation (the Fortran loop order)
        acc = np.zeros(kk.shape[0])
        for i in range(terms.shape[1]):
            acc = acc + terms[:, i]
        flat_o[s:s + chunk] = 2.0 * acc * dx
    return out


def k_vCk_fast(k, acell: float, NG: int, NK: int) -> np.ndarray:
    """Same sum as :func:`k_vCk` with numpy pairwise summation (for large sizes).

    Differs from the sequential order only by summation rounding.
    """
    k = np.atleast_1d(np.asarray(k, dtype=np.float64))
    dx, n = k_vCk_count(acell, NG, NK)
    x = np.arange(n + 1, dtype=np.float64) * dx
    den = np.sqrt(x * x + 1.0)
    out = np.empty(k.size)
    flat_k = k.reshape(-1)
    chunk = max(1, (1 << 22) // (n + 1))
    for s in range(0, flat_k.size, chunk):
        kk = flat_k[s:s + chunk, None]
        f = np.cos(kk * x[None, :]) / den[None, :]
        out[s:s + chunk] = 2.0 * (0.5 * (f[:, :-1] + f[:, 1:])).sum(axis=1) * dx
    return out.reshape(k.shape)


def make_grids(cfg: Config):
    """Cell, real-space grid, FFT-ordered G and Monkhorst-Pack k (I:46-49, 93-112)."""
    NG, NK = cfg.NG, cfg.NK
    ax = cfg.acell
    vcell = abs(cfg.acell)
    bx = TPI / ax
    dvcell = vcell / float(NG)
    rx = np.arange(NG, dtype=np.float64) / float(NG) * cfg.acell
    i1 = np.arange(1, NG + 1)
    Gx = np.where(i1 <= NG // 2, (i1 - 1) * bx, (i1 - 1 - NG) * bx).astype(np.float64)
    i = np.arange(1, NK + 1, dtype=np.float64)
    kx = (-0.5 + (2.0 * i - 1.0) / float(2 * NK)) * bx
    return vcell, dvcell, bx, rx, Gx, kx


def make_system(cfg: Config, vCk=k_vCk, with_vion=True) -> System:
    """Initialization (src/Initialization.f90:46-186) + ion potential."""
    vcell, dvcell, bx, rx, Gx, kx = make_grids(cfg)
    NG, NK, NB, NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
    vCGkk = None
    if cfg.functional.strip() == "HF":
        # vCGkk(ig,ikk) = k_vCk(Gx(ig)+kx(ikr)-kx(ikc)) (I:130-137); ikk = (ikr-1)*NK+ikc
        # only 2*NK-1 distinct k-differences exist; evaluate on the exact
        # floating-point argument of each (ikr, ikc) pair.
        args = (Gx[None, None, :] + kx[:, None, None]) - kx[None, :, None]
        vCGkk = vCk(args.reshape(NK * NK, NG), cfg.acell, NG, NK)
    vCG = vCk(Gx, cfg.acell, NG, NK)          # I:143-145
    vCG[0] = 0.0                               # I:146
    occbk = np.zeros((NK, NB))
    occbk[:, :NBocc] = 2.0 / float(NK)         # I:179-186
    sysm = System(cfg, vcell, dvcell, bx, rx, Gx, kx, occbk, vCG, vCGkk)
    if with_vion:
        sysm.vion = ion_potential(cfg, rx)
    return sysm


def ion_potential(cfg: Config, rx: np.ndarray) -> np.ndarray:
    """Periodic soft-Coulomb ion potential (src/Prep_periodic_ion_potential.f90:10-20)."""
    ax = cfg.acell
    NK = cfg.NK
    vion = np.zeros_like(rx)
    for ii in range(cfg.nion):
        sp = cfg.Kion[ii] - 1
        Za = float(cfg.Zeff[sp])
        al = float(cfg.alpha[sp])
        for icell in range(-4 * NK, 4 * NK + 1):
            dist = np.abs(rx - ax * cfg.Rion[ii] - ax * icell)
            vion = vion - Za / np.sqrt(dist * dist + al * al)
    return vion - vion.max()


def ion_param_grad(cfg: Config, rx: np.ndarray, g: np.ndarray):
    """dL/d(Zeff, alpha per species; Rion per ion) from dL/dvion = g on the grid,
    by the chain rule through :func:`ion_potential`.  The max shift
     contributes -(sum g) dvraw(x*)/dp at the grid point x* of the
    maximum (the first one at a tie).  Extension: the reference has no
    gradients."""
    ax, NK = cfg.acell, cfg.NK
    vraw = np.zeros_like(rx)
    for ii in range(cfg.nion):
        sp = cfg.Kion[ii] - 1
        for icell in range(-4 * NK, 4 * NK + 1):
            dist = np.abs(rx - ax * cfg.Rion[ii] - ax * icell)
            vraw = vraw - float(cfg.Zeff[sp]) / np.sqrt(dist * dist + float(cfg.alpha[sp]) ** 2)
    w = np.asarray(g, dtype=np.float64).copy()
    w[int(np.argmax(vraw))] -= np.sum(g)
    dZ = np.zeros(len(cfg.Zeff))
    da = np.zeros(len(cfg.alpha))
    dR = np.zeros(cfg.nion)
    for ii in range(cfg.nion):
        sp = cfg.Kion[ii] - 1
        Za, al = float(cfg.Zeff[sp]), float(cfg.alpha[sp])
        for icell in range(-4 * NK, 4 * NK + 1):
            d = rx - ax * cfg.Rion[ii] - ax * icell
            r = 1.0 / np.sqrt(d * d + al * al)
            dZ[sp] += np.sum(w * -r)
            da[sp] += np.sum(w * Za * al * r ** 3)
            dR[ii] += np.sum(w * -ax * Za * d * r ** 3)
    return dZ, da, dR


# ---------------------------------------------------------------------------
# Initial guess and orthonormalisation (src/mATTOHF.f90:134-196)
# ---------------------------------------------------------------------------
def quickrnd(iseed: int):
    """LCG of ``quickrnd`` (M:186-196): iseed = mod(106*iseed+1283, 6075)."""
    iseed = (iseed * 106 + 1283) % 6075
    return iseed, float(iseed) / 6075.0


def init_wf(sysm: System) -> np.ndarray:
    """Real Gaussians at LCG-random centres (``Init_wf``, M:159-184)."""
    cfg = sysm.cfg
    u = np.empty((cfg.NK, cfg.NB, cfg.NG), dtype=np.complex128)
    iseed = 123
    for ik in range(cfg.NK):
        for ib in range(cfg.NB):
            iseed, rnd = quickrnd(iseed)
            rxc = rnd * cfg.acell
            r2 = (sysm.rx - rxc) ** 2
            u[ik, ib] = np.exp(-0.5 * r2)
    return u


def init_wf_normal(sysm: System, seed: int) -> np.ndarray:
    """Seeded complex-normal guess (extension: not in the reference)."""
    cfg = sysm.cfg
    rng = np.random.default_rng(seed)
    re = rng.standard_normal((cfg.NK, cfg.NB, cfg.NG))
    im = rng.standard_normal((cfg.NK, cfg.NB, cfg.NG))
    return re + 1j * im


def gram_schmidt(sysm: System, ubk: np.ndarray) -> np.ndarray:
    """Modified Gram-Schmidt per k with weight vcell/NG (``Gram_Schmidt``, M:134-157)."""
    u = ubk.copy()
    w = sysm.vcell / float(sysm.NG)
    for ik in range(sysm.NK):
        for ib in range(sysm.NB):
            for ibt in range(ib):
                zov = np.sum(np.conj(u[ik, ibt]) * u[ik, ib]) * w
                u[ik, ib] = u[ik, ib] - u[ik, ibt] * zov
            s = np.sum(np.abs(u[ik, ib]) ** 2) * w
            u[ik, ib] = u[ik, ib] / math.sqrt(s)
    return u


# ---------------------------------------------------------------------------
# Operator kernels (src/Functions.f90)
# ---------------------------------------------------------------------------
def ubk_dns(sysm: System, ubk: np.ndarray) -> np.ndarray:
    """rho(ig) = sum_{ik,ib} occbk*|u|^2 in ig->ik->ib order (F:55-71)."""
    NK, NB = sysm.NK, sysm.NB
    dns = np.zeros(sysm.NG)
    for ik in range(NK):
        for ib in range(NB):
            z = ubk[ik, ib]
            dns = dns + sysm.occbk[ik, ib] * (z.real * z.real + z.imag * z.imag)
    return dns


def dns_vH(sysm: System, dns: np.ndarray) -> np.ndarray:
    """Hartree potential vH = Re IFFT(vCG*FFT(rho))/NG (F:147-162)."""
    w2 = fftf(dns.astype(np.complex128))
    w2 = sysm.vCG * w2
    return fftb(w2).real / float(sysm.NG)


def ubk_tubk(sysm: System, ubk: np.ndarray, A: float) -> np.ndarray:
    """Kinetic operator 0.5*(G+k+A)^2 applied per column (F:212-234)."""
    kAx = sysm.kx + A                                        # (NK,)
    kA2 = kAx ** 2
    Gx = sysm.Gx
    mult = 0.5 * (Gx[None, :] ** 2 + 2.0 * Gx[None, :] * kAx[:, None] + kA2[:, None])
    work = fftf(ubk)
    work = mult[:, None, :] * work / float(sysm.NG)
    return fftb(work)


def ubkwbk_vFwbk(sysm: System, ubk: np.ndarray, wbk: np.ndarray) -> np.ndarray:
    """Fock exchange on wbk with the occupied orbitals of ubk (F:237-261).

    For ikk=(ikr,ikc), ibr<nbw, ibc<NBocc (in that loop order):
      pairrho = wbk(:,ibr,ikr)*conj(ubk(:,ibc,ikc))/NK; FFT;
      *= -vCGkk(:,ikk)/NG; IFFT; vFwbk(:,ibr,ikr) += VF*ubk(:,ibc,ikc).
    ``wbk`` may have any number of bands (the Krylov blocks use NB).
    """
    NK, NG, NBocc = sysm.NK, sysm.NG, sysm.NBocc
    nbw = wbk.shape[1]
    out = np.zeros_like(wbk)
    for ikr in range(NK):
        # all pair densities of this ikr at once: (NK, nbw, NBocc, NG)
        pr = wbk[ikr][None, :, None, :] * np.conj(ubk[:, None, :NBocc, :]) / float(NK)
        pg = fftf(pr)
        v = sysm.vCGkk[ikr * NK:(ikr + 1) * NK]             # (NK, NG)
        pg = -v[:, None, None, :] * pg / float(NG)
        VF = fftb(pg)
        acc = np.zeros((nbw, NG), dtype=np.complex128)
        for ikc in range(NK):
            for ibc in range(NBocc):
                acc = acc + VF[ikc, :, ibc, :] * ubk[ikc, ibc][None, :]
        out[ikr] = acc
    return out


def ubkwbk_hwbk(sysm: System, ubk: np.ndarray, wbk: np.ndarray, A: float) -> np.ndarray:
    """h[u] w = T_A w + (vH[rho(u)]+vion) w + VF[u] w (F:187-209)."""
    h = ubk_tubk(sysm, wbk, A)
    vH = dns_vH(sysm, ubk_dns(sysm, ubk))
    h = h + (vH + sysm.vion)[None, None, :] * wbk
    if sysm.hf:
        h = h + ubkwbk_vFwbk(sysm, ubk, wbk)
    return h


def ubk_Ekin(sysm: System, ubk: np.ndarray, A: float) -> float:
    """Kinetic energy (F:94-119)."""
    t = ubk_tubk(sysm, ubk, A)
    e = 0.0
    for ik in range(sysm.NK):
        for ib in range(sysm.NB):
            e += sysm.occbk[ik, ib] * np.sum(np.conj(ubk[ik, ib]) * t[ik, ib]) * sysm.dvcell
    return float(np.real(e))


def dns_Eion(sysm: System, dns) -> float:
    """Ion energy (F:122-131)."""
    return float(np.sum(sysm.vion * dns) * sysm.dvcell)


def dns_EH(sysm: System, dns) -> float:
    """Hartree energy 0.5*sum(vH*rho)*dvcell (F:134-144)."""
    return float(0.5 * np.sum(dns_vH(sysm, dns) * dns) * sysm.dvcell)


def ubk_Ex(sysm: System, ubk: np.ndarray) -> float:
    """Exchange energy 0.5*sum_occ occ<u|VF u>*dvcell (F:165-183)."""
    vF = ubkwbk_vFwbk(sysm, ubk, ubk)
    ex = 0.0
    for ik in range(sysm.NK):
        for ib in range(sysm.NBocc):
            ex += sysm.occbk[ik, ib] * np.sum(np.conj(ubk[ik, ib]) * vF[ik, ib]) * sysm.dvcell
    return float(np.real(0.5 * ex))


def ubk_Ecomps(sysm: System, ubk: np.ndarray, A: float):
    """(Ekin, Eion, EH, Exc) (F:265-286); Etot = their sum (F:74-91)."""
    dns = ubk_dns(sysm, ubk)
    Ekin = ubk_Ekin(sysm, ubk, A)
    Eion = dns_Eion(sysm, dns)
    EH = dns_EH(sysm, dns)
    Exc = ubk_Ex(sysm, ubk) if sysm.hf else 0.0
    return np.array([Ekin, Eion, EH, Exc])


def ubk_Etot(sysm: System, ubk: np.ndarray, A: float) -> float:
    c = ubk_Ecomps(sysm, ubk, A)
    return float(c[0] + c[1] + c[2] + c[3])


def ubk_Je(sysm: System, ubk: np.ndarray, A: float) -> float:
    """Current Je = -Re sum occ <u|(G+k+A) u> dvcell/vcell (F:289-318)."""
    J = 0.0 + 0.0j
    for ik in range(sysm.NK):
        GkAx = sysm.Gx + sysm.kx[ik] + A
        for ib in range(sysm.NB):
            w1 = fftf(ubk[ik, ib]) / float(sysm.NG)
            w2 = fftb(GkAx * w1)
            J += sysm.occbk[ik, ib] * np.sum(np.conj(ubk[ik, ib]) * w2)
    return float(-np.real(J * sysm.dvcell / sysm.vcell))


def ubk_epsbk(sysm: System, ubk: np.ndarray) -> np.ndarray:
    """Ritz values Re<u|h u>*dvcell at A=0 (F:321-337); shape (NK, NB)."""
    h = ubkwbk_hwbk(sysm, ubk, ubk, 0.0)
    return np.real(np.sum(np.conj(ubk) * h, axis=2)) * sysm.dvcell


def ubk_epserrorbk(sysm: System, ubk: np.ndarray) -> np.ndarray:
    """Residual sqrt(sum |h u - eps u| * dvcell) — abs, not abs^2 (F:340-358)."""
    h = ubkwbk_hwbk(sysm, ubk, ubk, 0.0)
    eps = np.real(np.sum(np.conj(ubk) * h, axis=2)) * sysm.dvcell
    r = h - eps[:, :, None] * ubk
    return np.sqrt(np.sum(np.abs(r), axis=2) * sysm.dvcell)


# ---------------------------------------------------------------------------
# Real-time propagation (src/RT_calculation.f90)
# ---------------------------------------------------------------------------
def powi(x: float, m: int) -> float:
    """Integer power by square-and-multiply, as gfortran evaluates x**n."""
    n = abs(m)
    y = x if n % 2 else 1.0
    n >>= 1
    while n:
        x = x * x
        if n % 2:
            y = y * x
        n >>= 1
    return 1.0 / y if m < 0 else y


def define_afield(cfg: Config):
    """time, A, Aave, E, E2 of ``Define_Afield`` (RT:175-244)."""
    NT, dt = cfg.NT, cfg.dt
    time = dt * np.arange(NT, dtype=np.float64)              # RT:186-188
    A = np.zeros(NT)
    Am1 = 0.0
    if cfg.field_option == "LR":
        A[:] = cfg.dAc                                       # RT:203
    elif cfg.field_option == "LP":
        omegac = cfg.omegac / HARTREE                        # RT:209-211
        Tpulse = cfg.Tpulse / ATOMTIME
        E0 = cfg.E0 / ATOMFIELD
        Aamp = E0 / omegac
        NTpulse = int(min(Tpulse / dt, float(NT)))            # RT:215
        for it in range(NTpulse):
            t = time[it]
            A[it] = Aamp * math.sin(omegac * (t - 0.5 * Tpulse) + 2.0 * PI * cfg.phiCEP) \
                * powi(math.sin(PI * t / Tpulse), cfg.nenvelope)
    else:
        raise ValueError("# Error stop: substituted field_option  is not acceptable.")
    Aave = np.empty(NT)
    Aave[0] = 0.5 * (A[0] + Am1)
    Aave[1:] = 0.5 * (A[1:] + A[:-1])
    E = np.empty(NT)
    E[0] = -(A[0] - Am1) / dt
    E[1:] = -(A[1:] - A[:-1]) / dt
    E2 = E ** 2
    return time, A, Aave, E, E2


def rk4_step(sysm: System, ubk: np.ndarray, Aave: float, A: float, dt: float) -> np.ndarray:
    """Classical RK4 with stage fields A(it-1), Aave, Aave, A(it) (RT:154-173)."""
    Am = 2.0 * Aave - A
    h = lambda u, a: ubkwbk_hwbk(sysm, u, u, a)
    k1 = -1j * h(ubk, Am)
    u2 = ubk + (0.5 * dt) * k1
    k2 = -1j * h(u2, Aave)
    u3 = ubk + (0.5 * dt) * k2
    k3 = -1j * h(u3, Aave)
    u4 = ubk + dt * k3
    k4 = -1j * h(u4, A)
    return ubk + (k1 + 2.0 * k2 + 2.0 * k3 + k4) * dt / 6.0


def _te(sysm: System, u: np.ndarray, base: np.ndarray, Aave: float, dt: float, norder: int = 4):
    """u + sum_n (-i dt h[base])^n u / n! term by term (RT:83-89)."""
    w = u.copy()
    out = u.copy()
    for iorder in range(1, norder + 1):
        w = -(1j * dt) * ubkwbk_hwbk(sysm, base, w, Aave) / float(iorder)
        out = out + w
    return out


def te_step(sysm: System, ubk: np.ndarray, Aave: float, dt: float, variant: str = "TE"):
    """Alternative propagators RT_TE_ubk / RT_TEPC_ubk / RT_TEPC2_ubk (RT:72-151)."""
    u0 = ubk.copy()
    if variant == "TE":
        return _te(sysm, ubk, u0, Aave, dt)
    u1 = _te(sysm, ubk, u0, Aave, dt)
    if variant == "TEPC":
        w = ubk.copy()
        out = ubk.copy()
        for iorder in range(1, 5):
            w = -(1j * dt * 0.5) * (ubkwbk_hwbk(sysm, u0, w, Aave) + ubkwbk_hwbk(sysm, u1, w, Aave)) / float(iorder)
            out = out + w
        return out
    if variant == "TEPC2":
        return _te(sysm, ubk, 0.5 * (u0 + u1), Aave, dt)
    raise ValueError(variant)


@dataclasses.dataclass
class RTResult:
    time: np.ndarray
    Etot: np.ndarray
    Nele: np.ndarray
    Jtot: np.ndarray
    E: np.ndarray
    A: np.ndarray
    Etot0: float
    Nele0: float
    Jtot0: float
    ubk: np.ndarray
    dipole: Optional[np.ndarray] = None


def dipole_from_current(time, J, J0, dt):
    """Dipole P(t) = -int_0^t J dt' (trapezoid, J(0)=J0) — extension, not in the reference."""
    P = np.empty_like(J)
    acc = 0.0
    prev = J0
    for i in range(J.size):
        acc -= 0.5 * dt * (prev + J[i])
        P[i] = acc
        prev = J[i]
    return P


def rt_calculation(sysm: System, ubk: np.ndarray, nt: Optional[int] = None,
                   A: Optional[np.ndarray] = None, Aave: Optional[np.ndarray] = None) -> RTResult:
    """Real-time loop (RT:27-60): RK4 then rho, Nele, Etot, Jtot per step."""
    cfg = sysm.cfg
    time, A_, Aave_, E, _ = define_afield(cfg)
    if A is None:
        A, Aave = A_, Aave_
    nt = cfg.NT if nt is None else nt
    u = ubk.copy()
    dns = ubk_dns(sysm, u)
    Nele0 = float(np.sum(dns) * sysm.dvcell)
    Etot0 = ubk_Etot(sysm, u, 0.0)
    J0 = ubk_Je(sysm, u, 0.0)
    Et, Ne, Jt = np.empty(nt), np.empty(nt), np.empty(nt)
    for it in range(nt):
        u = rk4_step(sysm, u, Aave[it], A[it], cfg.dt)
        dns = ubk_dns(sysm, u)
        Ne[it] = np.sum(dns) * sysm.dvcell
        Et[it] = ubk_Etot(sysm, u, A[it])
        Jt[it] = ubk_Je(sysm, u, A[it])
    res = RTResult(time[:nt], Et, Ne, Jt, E[:nt], np.asarray(A)[:nt], Etot0, Nele0, J0, u)
    res.dipole = dipole_from_current(res.time, Jt, J0, cfg.dt)
    return res


# ---------------------------------------------------------------------------
# Ground state (src/GS_calculation.f90)
# ---------------------------------------------------------------------------
def _zheev(a):
    from scipy.linalg import lapack
    w, v, info = lapack.zheev(a, compute_v=1, lower=0)
    if info != 0:
        raise RuntimeError(f"zheev info={info}")
    return w, v


def cgs2_block(blk: np.ndarray, weight: float) -> np.ndarray:
    """Orthonormal basis of the rows of ``blk`` (m, NG) by classical
    Gram-Schmidt applied twice per column, in column order, with the inner
    product weight * <a|b>.  Not the reference's method: it is the
    orthonormalisation the GPU path uses in place of ZGESVD('O') (GS:161-166),
    restated here so the two choices can be compared on the same inputs."""
    q = blk.copy()
    for j in range(q.shape[0]):
        c = q[j]
        for _ in range(2 if j > 0 else 0):
            z = weight * (np.conj(q[:j]) @ c)
            c = c - z @ q[:j]
        q[j] = c / math.sqrt(weight * float(np.real(np.vdot(c, c))))
    return q


def ks_ubk2_svd(sysm: System, ubk: np.ndarray, A0: float = 0.0, ortho: str = "svd") -> np.ndarray:
    """Block-Krylov Rayleigh-Ritz (``KS_ubk2_SVD``, GS:124-194).

    ``ortho="svd"`` is the reference's ZGESVD('O') basis; ``ortho="cgs2"``
    swaps in :func:`cgs2_block` (the GPU path's choice) for comparisons."""
    from scipy.linalg import lapack
    NK, NB, NG, NCG = sysm.NK, sysm.NB, sysm.NG, sysm.cfg.NCG
    m = NB * NCG
    work = np.empty((NK, m, NG), dtype=np.complex128)
    work[:, :NB] = ubk
    for iCG in range(1, NCG):                                   # GS:155-158
        work[:, NB * iCG:NB * (iCG + 1)] = ubkwbk_hwbk(
            sysm, ubk, work[:, NB * (iCG - 1):NB * iCG], A0)
    for ik in range(NK):                                        # GS:161-166
        if ortho == "cgs2":
            work[ik] = cgs2_block(work[ik], sysm.dvcell)
            continue
        a = np.asfortranarray(work[ik].T)                       # (NG, m)
        u_, s_, vt_, info = lapack.zgesvd(a, compute_uv=1, full_matrices=0)
        if info != 0:
            raise RuntimeError(f"zgesvd info={info}")
        blk = u_[:, :m].T.copy()                                # left singular vectors
        s = np.sum(np.abs(blk[0]) ** 2) * sysm.dvcell
        work[ik] = blk / math.sqrt(s)
    hwork = np.empty_like(work)
    for iCG in range(NCG):                                      # GS:169-171
        sl = slice(NB * iCG, NB * (iCG + 1))
        hwork[:, sl] = ubkwbk_hwbk(sysm, ubk, work[:, sl], A0)
    out = ubk.copy()
    for ik in range(NK):                                        # GS:173-191
        whw = np.conj(work[ik]) @ hwork[ik].T * sysm.dvcell     # whw[i,j] = <w_i|h w_j>
        H = np.tril(whw, -1)
        H = H + np.conj(H.T)
        H[np.diag_indices(m)] = np.real(np.diag(whw))
        _, coef = _zheev(H)
        out[ik] = (coef[:, :NB].T @ work[ik])
    return out


def subspace_diag(sysm: System, ubk: np.ndarray, A0: float = 0.0) -> np.ndarray:
    """NB x NB Rayleigh-Ritz per k (``Subspace_diag``, GS:197-237)."""
    NB = sysm.NB
    h = ubkwbk_hwbk(sysm, ubk, ubk, A0)
    out = np.empty_like(ubk)
    for ik in range(sysm.NK):
        M = np.conj(ubk[ik]) @ h[ik].T * sysm.dvcell
        H = np.tril(M, -1)
        H = H + np.conj(H.T)
        H[np.diag_indices(NB)] = np.real(np.diag(M))
        _, coef = _zheev(H)
        out[ik] = coef.T @ ubk[ik]
    return out


@dataclasses.dataclass
class GSResult:
    ubk: np.ndarray
    Etot: np.ndarray          # Etotscf(0:Nscf)
    Je: np.ndarray            # per iteration
    epsbk: np.ndarray         # final (NK, NB)
    epserrorbk: np.ndarray    # final (NK, NB)
    dnsdiff: np.ndarray       # sum|dnsscf(iter+1)-dnsscf(iter)|/NG per iteration
    Ecomps: np.ndarray
    eps_hist: Optional[list] = None     # epsbk of every iteration (the GSinfo columns)
    err_hist: Optional[list] = None     # epserrorbk of every iteration


def gs_calculation(sysm: System, ubk: np.ndarray, nscf: Optional[int] = None, ortho: str = "svd") -> GSResult:
    """SCF loop (``GS_calculation``, GS:26-60); ``ortho`` as in :func:`ks_ubk2_svd`."""
    nscf = sysm.cfg.Nscf if nscf is None else nscf
    u = ubk.copy()
    dnsmix = 0.5
    dprev = ubk_dns(sysm, u)
    Et = np.empty(nscf + 1)
    Et[0] = ubk_Etot(sysm, u, 0.0)
    Je = np.empty(nscf)
    dd = np.empty(nscf)
    eps = err = None
    eh, rh = [], []
    for it in range(nscf):
        u = gram_schmidt(sysm, u)
        u = ks_ubk2_svd(sysm, u, 0.0, ortho)
        u = gram_schmidt(sysm, u)
        u = subspace_diag(sysm, u, 0.0)
        Et[it + 1] = ubk_Etot(sysm, u, 0.0)
        Je[it] = ubk_Je(sysm, u, 0.0)
        eps = ubk_epsbk(sysm, u)
        err = ubk_epserrorbk(sysm, u)
        eh.append(eps)
        rh.append(err)
        dnew = dnsmix * ubk_dns(sysm, u) + (1.0 - dnsmix) * dprev   # GS:44 (never fed back)
        dd[it] = np.sum(np.abs(dnew - dprev)) / float(sysm.NG)
        dprev = dnew
    return GSResult(u, Et, Je, eps, err, dd, ubk_Ecomps(sysm, u, 0.0), eh, rh)


# ---------------------------------------------------------------------------
# Spectral post-processing (RT:246-351)
# ---------------------------------------------------------------------------
def fourier_tr(cfg: Config, time, Jtot, Jtotm1, E, A):
    """Polynomial-filtered DFT of J, E, A and (LR) sigma/eps (``FourierTr``, RT:246-303)."""
    NT = time.size
    filt = 1.0 - 3.0 * (time / time[NT - 1]) ** 2 + 2.0 * (time / time[NT - 1]) ** 3
    omega = np.arange(1, cfg.Nomega + 1, dtype=np.float64) / float(cfg.Nomega) * cfg.omegaM
    Jtemp = filt * (Jtot - Jtotm1)
    eiwt = np.exp(1j * omega[:, None] * time[None, :])
    JF = (eiwt * Jtemp[None, :]).sum(axis=1) * cfg.dt
    EF = (eiwt * (filt * E)[None, :]).sum(axis=1) * cfg.dt
    AF = (eiwt * (filt * A)[None, :]).sum(axis=1) * cfg.dt
    sigma = eps = None
    if cfg.field_option == "LR":
        sigma = -JF / cfg.dAc
        eps = FPI * 1j * sigma / omega
    return omega, JF, EF, AF, sigma, eps


def window_fourier_tr(cfg: Config, time, Jtot, Jtotm1, E, A):
    """Envelope-windowed DFT (``WindowFourierTr``, RT:305-351); None for LR."""
    if cfg.field_option == "LR":
        return None
    NT = time.size
    Tpulse = cfg.Tpulse / ATOMTIME
    NTpulse = int(min(Tpulse / cfg.dt, float(NT)))
    filt = np.zeros(NT)
    for it in range(NTpulse):
        filt[it] = powi(math.sin(PI * time[it] / Tpulse), cfg.nenvelope)
    omega = np.arange(1, cfg.Nomega + 1, dtype=np.float64) / float(cfg.Nomega) * cfg.omegaM
    Jtemp = filt * (Jtot - Jtotm1)
    eiwt = np.exp(1j * omega[:, None] * time[None, :])
    JF = (eiwt * Jtemp[None, :]).sum(axis=1) * cfg.dt
    EF = (eiwt * (filt * E)[None, :]).sum(axis=1) * cfg.dt
    AF = (eiwt * (filt * A)[None, :]).sum(axis=1) * cfg.dt
    return omega, JF, EF, AF


# ---------------------------------------------------------------------------
# Adjoint of the RK4 real-time loop (extension: no counterpart in the reference)
# ---------------------------------------------------------------------------
# Real inner product <a, b>_R = Re sum conj(a) b over all orbital entries.
# f(v, a) = -i h[v](a) v is the RK4 right-hand side (RT:166-169).  The
# adjoint needs J_f(v)^T mu for that real inner product.

def _pair_potential(S: System, ki: int, kj: int, rho: np.ndarray) -> np.ndarray:
    """Phi_ij[rho] = IFFT(-vCGkk(:,ki,kj)/NG * FFT(rho/NK)) as in F:250-253."""
    v = S.vCGkk[ki * S.NK + kj]
    g = fftf(rho / float(S.NK))
    return fftb(-v * g / float(S.NG))


def _pair_potential_reflected(S: System, ki: int, kj: int, rho: np.ndarray) -> np.ndarray:
    """Phi~_ji[rho]: the pair convolution with multiplier m_ji(-G), where m_ji(G)
    = -vCGkk(G, kj, ki)/(NG NK) is Phi_ji's.  Because v is even this equals
    Phi_ij (multiplier m_ij(G)) at every G except the self-aliased Nyquist index
    NG/2 (Gx = -NG/2 bx, src/Initialization.f90:97-102), where -G is G itself and
    the multiplier stays m_ji.  It is the operator that the transpose of the
    map dv_j -> Phi_ij[v_i conj(dv_j)] brings in."""
    v = S.vCGkk[ki * S.NK + kj].copy()
    v[S.NG // 2] = S.vCGkk[kj * S.NK + ki][S.NG // 2]
    g = fftf(rho / float(S.NK))
    return fftb(-v * g / float(S.NG))


def velocity(S: System, u: np.ndarray, A: float) -> np.ndarray:
    """P_A u = IFFT((G+k+A) FFT(u)/NG) per column (the operator inside ubk_Je, F:306-310)."""
    GkA = S.Gx[None, :] + S.kx[:, None] + A            # (NK, NG)
    return fftb(GkA[:, None, :] * fftf(u) / float(S.NG))


def hf_vjp(S: System, v: np.ndarray, mu: np.ndarray, A: float) -> np.ndarray:
    """J^T mu of f(v) = -i h[v](A) v (all bands occupied, NB == NBocc)."""
    assert S.NB == S.NBocc
    NK, NB = S.NK, S.NB
    # kinetic + local + exchange operator at fixed v: (-i h)^T = i h
    out = 1j * ubkwbk_hwbk(S, v, mu, A)
    # Hartree: delta vH from delta rho = 2 occ Re(conj(v) dv)
    sig = np.sum(np.imag(np.conj(mu) * v), axis=(0, 1))
    psi = dns_vH(S, sig)
    out += 2.0 * S.occbk[:, :, None] * psi[None, None, :] * v
    if S.hf:
        # exchange operator's dependence on v:
        #   out_i += i sum_j conj(phi_ji) mu_j,  phi_ji = Phi_ji[v_j conj(v_i)]
        #   out_i += -i sum_j v_j Phi~_ji[v_i conj(mu_j)]   (the transpose of
        #            dv_j -> Phi_ij[v_i conj(dv_j)]; Phi~_ji differs from Phi_ij
        #            only at the Nyquist index)
        for ki in range(NK):
            for bi in range(NB):
                acc = np.zeros(S.NG, dtype=np.complex128)
                for kj in range(NK):
                    for bj in range(NB):
                        phi_ji = _pair_potential(S, kj, ki, v[kj, bj] * np.conj(v[ki, bi]))
                        acc += 1j * np.conj(phi_ji) * mu[kj, bj]
                        acc += -1j * v[kj, bj] * _pair_potential_reflected(S, ki, kj,
                                                                           v[ki, bi] * np.conj(mu[kj, bj]))
                out[ki, bi] += acc
    return out


def _field_grad(S: System, lam_k: np.ndarray, v: np.ndarray, a: float) -> float:
    """<lam_k, d f/d a>_R with d f / d a = -i P_a v."""
    return float(np.real(np.sum(np.conj(lam_k) * (-1j) * velocity(S, v, a))))


def objective_grad_u(S: System, u: np.ndarray, A: float, objective: str) -> np.ndarray:
    """Gradient g of the objective w.r.t. u (dL = <g, du>_R).

    Energy: 2 occ dvcell h[u] u, plus a Nyquist term of the exchange energy.
    Ex = 1/2 occ dvcell sum_ij <p_ij, Phi_ij p_ij> with p_ij = u_i conj(u_j)
    (F:165-183); varying the conj(u_j) factor brings in conj(Phi_ij[p_ij]),
    which is Phi_ji[p_ji] except at the self-aliased Nyquist index, so
      g_i += occ dvcell sum_j (m_ji - m_ij)(N/2) Nyq(p_ij) (-1)^x u_j,
    with m_ij = -vCGkk(:, ki, kj)/(NG NK) and Nyq(p) = sum_x (-1)^x p(x)."""
    if objective == "energy":
        g = 2.0 * S.occbk[:, :, None] * S.dvcell * ubkwbk_hwbk(S, u, u, A)
        if S.hf:
            NK, NG, NBo = S.NK, S.NG, S.NBocc
            sg = (-1.0) ** np.arange(NG)
            occ = 2.0 / float(NK)
            m = -S.vCGkk[:, NG // 2].reshape(NK, NK) / float(NG * NK)   # m[ki, kj] at N/2
            nyq = np.einsum("ibx,jcx,x->ibjc", u[:, :NBo], np.conj(u[:, :NBo]), sg)
            d = (m.T - m)[:, None, :, None]                             # m_ji - m_ij
            corr = np.einsum("ibjc,jcx->ibx", d * nyq, u[:, :NBo]) * sg
            g[:, :NBo] += occ * S.dvcell * corr
        return g
    if objective == "current":
        return -2.0 * S.occbk[:, :, None] * (S.dvcell / S.vcell) * velocity(S, u, A)
    raise ValueError(objective)


def objective_value(S: System, u: np.ndarray, A: float, objective: str, u0: np.ndarray) -> float:
    if objective == "energy":
        return ubk_Etot(S, u, A) - ubk_Etot(S, u0, 0.0)
    return ubk_Je(S, u, A)


def objective_dA(S: System, u: np.ndarray, A: float, objective: str) -> float:
    """Explicit derivative of the objective w.r.t. the final field sample."""
    if objective == "energy":
        return -ubk_Je(S, u, A) * S.vcell
    return -float(np.sum(ubk_dns(S, u)) * S.dvcell) / S.vcell


def rt_adjoint(S: System, u0: np.ndarray, A: np.ndarray, dt: float, objective: str = "energy"):
    """Objective, its gradient w.r.t. every field sample A[n] and w.r.t. vion(x).

    Forward: the RK4 loop of RT:38-42 with Aave[n] = (A[n]+A[n-1])/2, A[-1]=0
    (RT:227-230), stage fields 2 Aave - A, Aave, Aave, A (RT:165-169).
    Objective: absorbed energy Etot(u_N, A[N-1]) - Etot(u_0, 0), or the final
    current Je(u_N, A[N-1]).  Backward: discrete adjoint of every RK4 stage.
    """
    A = np.asarray(A, dtype=np.float64)
    N = A.size
    Aave = np.empty(N)
    Aave[0] = 0.5 * (A[0] + 0.0)
    Aave[1:] = 0.5 * (A[1:] + A[:-1])
    c = [0.5 * dt, 0.5 * dt, dt]
    states = [u0.copy()]
    u = u0.copy()
    for n in range(N):
        u = rk4_step(S, u, Aave[n], A[n], dt)
        states.append(u)
    L = objective_value(S, u, A[-1], objective, u0)
    lam = objective_grad_u(S, u, A[-1], objective)
    gA = np.zeros(N)
    gA[-1] += objective_dA(S, u, A[-1], objective)
    gAave = np.zeros(N)
    gvion = np.zeros(S.NG)
    if objective == "energy":   # Eion = sum vion rho dvcell at both ends
        gvion += (ubk_dns(S, u) - ubk_dns(S, u0)) * S.dvcell
    for n in range(N - 1, -1, -1):
        un = states[n]
        Am = 2.0 * Aave[n] - A[n]
        a = [Am, Aave[n], Aave[n], A[n]]
        # recompute the stage inputs
        h = lambda w, f: -1j * ubkwbk_hwbk(S, w, w, f)
        us = [un]
        k1 = h(un, a[0])
        us.append(un + c[0] * k1)
        k2 = h(us[1], a[1])
        us.append(un + c[1] * k2)
        k3 = h(us[2], a[2])
        us.append(un + c[2] * k3)
        lam_k = [dt / 6.0 * lam, dt / 3.0 * lam, dt / 3.0 * lam, dt / 6.0 * lam]
        lam_u = lam.copy()
        ga = [0.0] * 4
        for s in range(3, -1, -1):
            ga[s] = _field_grad(S, lam_k[s], us[s], a[s])
            gvion += np.sum(np.imag(np.conj(lam_k[s]) * us[s]), axis=(0, 1))
            lu = hf_vjp(S, us[s], lam_k[s], a[s])
            lam_u = lam_u + lu
            if s > 0:
                lam_k[s - 1] = lam_k[s - 1] + c[s - 1] * lu
        lam = lam_u
        # stage fields -> (Aave[n], A[n]) : Am = 2 Aave - A
        gAave[n] += ga[1] + ga[2] + 2.0 * ga[0]
        gA[n] += ga[3] - ga[0]
    # Aave[n] = (A[n] + A[n-1]) / 2
    gA += 0.5 * gAave
    gA[:-1] += 0.5 * gAave[1:]
    return L, gA, gvion
