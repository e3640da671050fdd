"""Drop-in driver: the reference program's flow with its input and output files.

``python -m mattohf_gb300.driver < name_file`` reads the input-file name from
standard input (src/mATTOHF.f90:45, list-directed, quotes stripped; an empty
name keeps every default), then runs Initialization, the Gaussian guess and
Gram-Schmidt, the ground-state SCF and the real-time propagation on the GPU
and writes the reference's output files in its formats:

  potential.out            rx, vion                       (src/Prep_periodic_ion_potential.f90:23-27)
  vk.out                   Gx+kx, k_vCk(Gx+kx)            (src/Initialization.f90:149-155)
  <sys>_GSinfo.out         SCF history + energy components (src/GS_calculation.f90:21-24, 49-52, 63-90)
  <sys>_DoS.out, _band.out band energies and broadened DoS (src/GS_calculation.f90:93-118, 239-265)
  <sys>_EtotNJEAt.out      time, Etot, dEtot, Nele, dNele, J, E, A  (src/RT_calculation.f90:22-24, 52-53)
  <sys>_JEAF.out, _sigmaeps.out, _JEAF_window.out     (src/RT_calculation.f90:246-351)
  <sys>_dipole.out         time, P = -int J dt (extension; trapezoid from J(0))

Only the hot path runs on the GPU (all through ``libmattohf.so``); the files
are written on the host.
"""
from __future__ import annotations

import ctypes as C
import math
import sys
import time
from typing import List

import numpy as np

from . import _capi
from .api import Context
from .inputs import ATOMFLUENCE, ATOMTIME, HARTREE, PI, RunConfig, define_afield, dipole_from_current, read_input, _powi

_D = C.POINTER(C.c_double)


def fortran_e(x: float, w: int = 20, d: int = 12, e: int = 2) -> str:
    """Fortran Ew.d (Ee) edit descriptor: 0.ddddE+xx right-justified in w columns."""
    x = float(x)
    if not math.isfinite(x):
        s = "NaN" if math.isnan(x) else ("Infinity" if x > 0 else "-Infinity")
        return s.rjust(w)
    if x == 0.0:
        mant, ex = "0" * d, 0
        neg = math.copysign(1.0, x) < 0
    else:
        neg = x < 0
        t = f"{abs(x):.{d - 1}e}"
        digits, exp = t.split("e")
        mant = digits.replace(".", "")
        ex = int(exp) + 1
    if abs(ex) < 10 ** e:
        es = ("E+" if ex >= 0 else "E-") + str(abs(ex)).zfill(e)
    else:
        es = ("+" if ex >= 0 else "-") + str(abs(ex)).zfill(e + 1)
    s = ("-" if neg else "") + "0." + mant + es
    return s.rjust(w) if len(s) <= w else "*" * w


def _row(values, w=20, d=12, e=2) -> str:
    return "".join(fortran_e(v, w, d, e) for v in values)


def fortran_f(x: float, w: int = 12, d: int = 8) -> str:
    """Fortran Fw.d: asterisks when the value does not fit, Infinity for +-inf."""
    x = float(x)
    if math.isinf(x):
        s = "Infinity" if x > 0 else "-Infinity"
        return s.rjust(w)
    s = f"{x:.{d}f}"
    if len(s) > w and s.startswith(("0.", "-0.")):
        s = s.replace("0.", ".", 1)
    return s.rjust(w) if len(s) <= w else "*" * w


HUGE = float(np.finfo(np.float64).max)   # Fortran huge(1.d0): minval of an empty section
GSINFO_HEADER = ("#iter, Etotscf(iter), Etoscf(iter)-Etotscf(iter-1), ,sum(abs(dnsscf(:,iter+1)-dnsscf(:,iter)))"
                 "/dble(NG)          sum(epserrorbk)/dble(NB*NK),maxval(epserrorbk),Fundamental gap, Optical Gap")


def band_record(ik: int, kx: float, errsum: float, eps_k) -> str:
    """'(i5,3e20.12,4x,1e20.12,4x,1000e20.12)' (src/GS_calculation.f90:102, 114): the
    first group takes kx, the mean residual and epsbk(1); each 4x and the
    group after it appear only while bands remain."""
    items = [kx, errsum] + [float(v) for v in eps_k]
    s = f"{ik:5d}" + _row(items[:3])
    if len(items) > 3:
        s += "    " + _row(items[3:4])
    if len(items) > 4:
        s += "    " + _row(items[4:])
    return s


def gap_columns(eps: np.ndarray, NBocc: int):
    """The last two GSinfo columns (src/GS_calculation.f90:51-52).  With every band
    occupied, minval over the empty conduction section is huge(1.d0), and the
    second column reads epsbk(NB+1,ik), i.e. epsbk(1,ik+1) in column-major
    storage; the k-point ik = NK, whose read lies past the array, is left out."""
    NK, NB = eps.shape
    vmax = eps[:, :NBocc].max()
    if NBocc < NB:
        return [eps[:, NBocc:].min() - vmax, float(np.min(eps[:, NBocc] - eps[:, NBocc - 1]))]
    return [HUGE - vmax, HUGE if NK == 1 else float(np.min(eps[1:, 0] - eps[:-1, NB - 1]))]


def read_name(stream) -> str:
    line = stream.readline()
    s = line.strip()
    if s[:1] in ("'", '"'):
        end = s.find(s[0], 1)
        s = s[1:end] if end > 0 else s[1:]
    else:
        s = s.split()[0] if s.split() else ""
    return s


def make_dos(eps: np.ndarray, occ: np.ndarray, n: int = 10000):
    """Gaussian-broadened DoS on the reference's energy mesh (src/GS_calculation.f90:93-97, 239-265)."""
    lo, hi = eps.min(), eps.max()
    emin = lo - 0.1 * (hi - lo)
    emax = hi + 0.1 * (hi - lo)
    e = emin + (emax - emin) * np.arange(n) / float(n)
    width = 5.0 * (e[1] - e[0])
    dos = np.zeros(n)
    docc = np.zeros(n)
    for ik in range(eps.shape[0]):
        occmax = occ[ik].max()
        for ib in range(eps.shape[1]):
            val = np.exp(-(eps[ik, ib] - e) ** 2 / width ** 2)
            dos += occmax * val
            docc += occ[ik, ib] * val
    return e, dos / (width * math.sqrt(PI)), docc / (width * math.sqrt(PI))


def fourier(cfg: RunConfig, time_, J, J0, E, A, window: bool, device: int = 0):
    """FourierTr (RT:246-303) or WindowFourierTr (RT:305-351) through mattohf_fourier."""
    lib = _capi.load()
    nt = time_.size
    if window:
        Tp = cfg.Tpulse / ATOMTIME
        ntp = int(min(Tp / cfg.dt, float(nt)))
        filt = np.zeros(nt)
        for it in range(ntp):
            filt[it] = _powi(math.sin(PI * time_[it] / Tp), cfg.nenvelope)
    else:
        tn = time_ / time_[nt - 1] if time_[nt - 1] != 0 else np.zeros(nt)
        filt = 1.0 - 3.0 * tn ** 2 + 2.0 * tn ** 3
    out = np.empty((cfg.Nomega, 7))
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (time_, J, E, A, filt)]
    st = lib.mattohf_fourier(device, nt, *(a.ctypes.data_as(_D) for a in arrs[:2]), C.c_double(J0),
                             arrs[2].ctypes.data_as(_D), arrs[3].ctypes.data_as(_D), arrs[4].ctypes.data_as(_D),
                             cfg.Nomega, C.c_double(cfg.omegaM), C.c_double(cfg.dt), out.ctypes.data_as(_D))
    if st != _capi.OK:
        raise RuntimeError(f"mattohf_fourier status {st}")
    return out


def run(cfg: RunConfig, out_dir: str = ".", rt_chunk: int = 1000, log=print) -> dict:
    import os
    p = lambda name: os.path.join(out_dir, name)
    sysn = cfg.sys_name.strip()
    t_all = time.perf_counter()
    ctx = Context(cfg)
    g = ctx.grids()
    NG, NK, NB, NBocc = cfg.NG, cfg.NK, cfg.NB, cfg.NBocc
    with open(p("potential.out"), "w") as fh:
        for x, v in zip(g["rx"], ctx.vion):
            fh.write(f" {float(x)!r:>24} {float(v)!r:>24}\n")
    vCG, vCq = ctx.coulomb()
    with open(p("vk.out"), "w") as fh:
        kk = np.add.outer(g["Gx"], g["kx"])          # k_vCk(Gx(ig)+kx(ik)), I:149-155
        vk = ctx.vck(kk.ravel()).reshape(kk.shape)
        for ig in range(NG):
            for ik in range(NK):
                fh.write(f" {float(kk[ig, ik])!r:>24} {float(vk[ig, ik])!r:>24}\n")
    ctx.Init_wf()
    ctx.Gram_Schmidt()
    occ = np.zeros((NK, NB))
    occ[:, :NBocc] = 2.0 / NK
    e0 = ctx.observables(0.0)
    log(f" Number of particle per cell {float(e0['Nele'])!r}")
    log(f" Total energy at initial = {float(e0['Etot'])!r}")
    # ---- ground state (GS:26-121)
    t_gs = time.perf_counter()
    dprev = ctx.ubk_dns(ctx.get_orbitals())
    Et_prev = e0["Etot"]
    lines: List[str] = [GSINFO_HEADER]
    eps = err = None
    for it in range(1, cfg.Nscf + 1):
        r = ctx.GS_calculation(1, cfg.NCG)
        eps, err = r["epsbk"], r["epserrorbk"]
        Et = r["Etot"][1]
        dnew = 0.5 * ctx.ubk_dns(ctx.get_orbitals()) + 0.5 * dprev
        dd = np.sum(np.abs(dnew - dprev)) / NG
        dprev = dnew
        lines.append("  " + f"{it:5d}" + _row([Et, Et - Et_prev, dd, err.sum() / (NB * NK), err.max()] +
                                              gap_columns(eps, NBocc)))
        log(f"iter, Etotscf(iter), JeGS ={it:4d}{Et:14.8f}{Et - Et_prev:12.4E}  {r['Je'][0]:12.4E}")
        Et_prev = Et
    ec = ctx.observables(0.0)
    for lab, key in (("Ekin ", "Ekin"), ("Eion ", "Eion"), ("EH   ", "EH"), ("Exc  ", "Exc")):
        lines.append(f"#{lab} at SCF:" + fortran_f(ec[key]))
    if eps is not None:
        # src/GS_calculation.f90:75-90; the conduction-bottom line prints maxval
        # of the conduction bands, as the reference does
        fund, opt = gap_columns(eps, NBocc)
        for lab, v in (("#Min. value of the spectra: minval(epsbk)    =", eps.min()),
                       ("#Max. value of the spectra: maxval(epsbk)    =", eps.max()),
                       ("#Valence top: maxval(epsbk(:NBocc,:))        =", eps[:, :NBocc].max()),
                       ("#Conduction bottom: minval(epsbk(NBocc+1:,:))=",
                        eps[:, NBocc:].max() if NBocc < NB else -HUGE),
                       ("#Fundamental gap: ", fund),
                       ("#Min. gap among same k-point: ", opt)):
            # +-huge(1.d0) in eV overflows to +-Infinity, as the reference's
            # own product does (Python floats overflow without a warning)
            lines.append(lab + fortran_f(v) + " =" + fortran_f(float(v) * HARTREE) + " [eV]")
    with open(p(f"{sysn}_GSinfo.out"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    if eps is not None:
        e, dos, docc = make_dos(eps, occ)
        with open(p(f"{sysn}_DoS.out"), "w") as fh:
            fh.write(" # ik,kx(ik),  sum(epserrorbk(:,ik))/dble(NB),  epsbk(:,ik)\n")
            for ik in range(NK):
                fh.write("# " + band_record(ik + 1, g["kx"][ik], err[ik].sum() / NB, eps[ik]) + "\n")
            for i in range(e.size):
                fh.write(_row([e[i], dos[i], docc[i]], e=3) + "\n")
        with open(p(f"{sysn}_band.out"), "w") as fh:
            fh.write(" # ik,kx(ik),  sum(epserrorbk(:,ik))/dble(NB),  epsbk(:,ik)\n")
            for ik in range(NK):
                fh.write(band_record(ik + 1, g["kx"][ik], err[ik].sum() / NB, eps[ik]) + "\n")
    t_gs = time.perf_counter() - t_gs
    # ---- real time (RT:2-69)
    t_rt = time.perf_counter()
    time_, A, Aave, E = define_afield(cfg)
    ini = ctx.observables(0.0)
    Etotm1, Nelem1, Jtotm1 = ini["Etot"], ini["Nele"], ini["Je"]
    NT = cfg.NT
    Et = np.empty(NT)
    Je = np.empty(NT)
    Ne = np.empty(NT)
    for s0 in range(0, NT, rt_chunk):
        s1 = min(NT, s0 + rt_chunk)
        Et[s0:s1], Je[s0:s1], Ne[s0:s1] = ctx.rk4_run(A[s0:s1], Aave[s0:s1], cfg.dt)
        log(f"{s1:6d} {time_[s1 - 1]:14.6E}{Et[s1 - 1]:14.6E}{Et[s1 - 1] - Etotm1:14.6E}")
    with open(p(f"{sysn}_EtotNJEAt.out"), "w") as fh:
        fh.write("#time(it), Etot(it)-Etot0, N(it)-N0, J(it), E(it), A(it)\n")
        for it in range(NT):
            fh.write(_row([time_[it], Et[it], Et[it] - Etotm1, Ne[it], Ne[it] - Nelem1, Je[it], E[it], A[it]]) + "\n")
    # extension (no reference counterpart): dipole P = -int J dt, trapezoid from J(0)
    P = dipole_from_current(Je, Jtotm1, cfg.dt)
    with open(p(f"{sysn}_dipole.out"), "w") as fh:
        fh.write("#time(it), P(it)\n")
        for it in range(NT):
            fh.write(_row([time_[it], P[it]]) + "\n")
    t_rt = time.perf_counter() - t_rt
    # ---- spectra (RT:64-65)
    ft = fourier(cfg, time_, Je, Jtotm1, E, A, window=False)
    with open(p(f"{sysn}_JEAF.out"), "w") as fh:
        fh.write("#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n")
        for r in ft:
            fh.write(_row(r) + "\n")
    if cfg.field_option == "LR":
        JF = ft[:, 1] + 1j * ft[:, 2]
        sigma = -JF / cfg.dAc
        eps_w = 4.0 * PI * 1j * sigma / ft[:, 0]
        with open(p(f"{sysn}_sigmaeps.out"), "w") as fh:
            fh.write("#omega(iomega), sigma(iomega), eps(iomega)\n")
            for w_, s_, e_ in zip(ft[:, 0], sigma, eps_w):
                fh.write(_row([w_, s_.real, s_.imag, e_.real, e_.imag]) + "\n")
    else:
        fw = fourier(cfg, time_, Je, Jtotm1, E, A, window=True)
        with open(p(f"{sysn}_JEAF_window.out"), "w") as fh:
            fh.write("#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n")
            for r in fw:
                fh.write(_row(r) + "\n")
    log(f"Time for GS calculatoin ={t_gs:12.4E} [sec]")
    log(f"Time for RT calculatoin ={t_rt:12.4E} [sec]")
    log(f"Time for an interaction in RT ={t_rt / max(NT, 1):12.4E} [sec]")
    log(f"Fluence of the field: {float(np.sum(E ** 2) * cfg.dt * ATOMFLUENCE)!r} J/cm^2")
    ctx.close()
    return {"Etot": Et, "Je": Je, "Nele": Ne, "P": P, "J0": Jtotm1, "A": A, "E": E, "time": time_, "t_rt": t_rt,
            "t_total": time.perf_counter() - t_all}


def main(argv=None) -> int:
    name = read_name(sys.stdin)
    cfg = read_input(name) if name else RunConfig()
    run(cfg)
    return 0


if __name__ == "__main__":
    sys.exit(main())
