"""The reference program's flow and output files, restated — TEST INFRASTRUCTURE ONLY.

Pins the drop-in drivers' files (potential.out, vk.out, <sys>_GSinfo.out,
<sys>_DoS.out, <sys>_band.out, <sys>_EtotNJEAt.out, <sys>_JEAF.out,
<sys>_JEAF_window.out or <sys>_sigmaeps.out) independently of them: every
number comes from the numpy oracle (``mattohf_oracle``) and every record is
formatted here from the reference's Fortran edit descriptors.  Only the test
suite imports it.

parity unpinned: the reference cannot be compiled here (no Fortran compiler);
the formats are read from its source.

Follows:
  Program Main               src/mATTOHF.f90:90-116 (order of the phases)
  Prep_periodic_ion_potential src/Prep_periodic_ion_potential.f90:23-27 (potential.out, list-directed)
  Initialization              src/Initialization.f90:148-155 (vk.out, list-directed)
  GS_calculation              src/GS_calculation.f90:21-24, 49-52, 63-118 (GSinfo, DoS, band)
  Make_DoS                    src/GS_calculation.f90:239-265
  RT_calculation              src/RT_calculation.f90:21-24, 52-53 (EtotNJEAt)
  FourierTr                   src/RT_calculation.f90:276-299 (JEAF, sigmaeps)
  WindowFourierTr             src/RT_calculation.f90:339-348 (JEAF_window)
The dipole file is an extension of the drivers and has no reference record.
"""
from __future__ import annotations

import math
import os
from typing import Optional

import numpy as np

from . import mattohf_oracle as O

HUGE = np.finfo(np.float64).max      # Fortran huge(1.d0): minval of an empty section
NDOS = 10000                          # GS:9

GSINFO_HEADER = ("#iter, Etotscf(iter), Etoscf(iter)-Etotscf(iter-1), ,sum(abs(dnsscf(:,iter+1)-dnsscf(:,iter)))"
                 "/dble(NG) " + "         sum(epserrorbk)/dble(NB*NK),maxval(epserrorbk),Fundamental gap, Optical Gap")
BAND_HEADER = " # ik,kx(ik),  sum(epserrorbk(:,ik))/dble(NB),  epsbk(:,ik)"


# ---------------------------------------------------------------------------
# Fortran edit descriptors
# ---------------------------------------------------------------------------
def ew(x: float, w: int = 20, d: int = 12, e: Optional[int] = None) -> str:
    """Ew.d (e is None) or Ew.dEe: a 0.d...d mantissa with d digits and an
    exponent field; for Ew.d a two-digit exponent prints as E+dd and a
    three-digit one as +ddd.  Output wider than w prints w asterisks."""
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("Infinity" if x > 0 else "-Infinity").rjust(w)
    if x == 0.0:
        digits, ex = "0" * d, 0
    else:
        # d significant digits, correctly rounded, as 0.ddd x 10^ex
        m, p = f"{abs(x):.{d - 1}e}".split("e")
        digits, ex = m.replace(".", ""), int(p) + 1
    sign = "-" if (x < 0 or (x == 0.0 and math.copysign(1.0, x) < 0)) else ""
    if e is None:
        if abs(ex) <= 99:
            exp = "E" + ("+" if ex >= 0 else "-") + f"{abs(ex):02d}"
        elif abs(ex) <= 999:
            exp = ("+" if ex >= 0 else "-") + f"{abs(ex):03d}"
        else:
            return "*" * w
    else:
        if abs(ex) >= 10 ** e:
            return "*" * w
        exp = "E" + ("+" if ex >= 0 else "-") + f"{abs(ex):0{e}d}"
    s = sign + "0." + digits + exp
    return s.rjust(w) if len(s) <= w else "*" * w


def fw(x: float, w: int = 12, d: int = 8) -> str:
    """Fw.d; output wider than w prints w asterisks, infinities as Infinity."""
    x = float(x)
    if math.isinf(x):
        s = "Infinity" if x > 0 else "-Infinity"
        return s.rjust(w) if len(s) <= w else ("Inf" if x > 0 else "-Inf").rjust(w)
    if math.isnan(x):
        return "NaN".rjust(w)
    s = f"{x:.{d}f}"
    if s.startswith("0."):
        s = s if len(s) <= w else s[1:]
    elif s.startswith("-0."):
        s = s if len(s) <= w else "-" + s[2:]
    return s.rjust(w) if len(s) <= w else "*" * w


def ew_list(xs, w=20, d=12, e=None) -> str:
    return "".join(ew(x, w, d, e) for x in xs)


def list_directed(*xs) -> str:
    """A list-directed record of reals (the drivers and the reference differ
    in its layout, which the standard leaves to the processor; only the values
    are compared)."""
    return " " + " ".join(f"{float(x)!r:>24}" for x in xs)


def band_record(ik: int, kx: float, errsum: float, eps_k: np.ndarray) -> str:
    """'(i5,3e20.12,4x,1e20.12,4x,1000e20.12)' with ik, kx, errsum, epsbk(:,ik)
    (GS:102, 114): the first group takes kx, errsum and epsbk(1); the 4x and
    the next group follow only while items remain."""
    items = [kx, errsum] + list(eps_k)
    s = f"{ik:5d}" + ew_list(items[:3])
    if len(items) > 3:
        s += "    " + ew(items[3])
    if len(items) > 4:
        s += "    " + ew_list(items[4:])
    return s


# ---------------------------------------------------------------------------
# Make_DoS (GS:93-97, 239-265)
# ---------------------------------------------------------------------------
def dos_mesh(eps: np.ndarray):
    lo, hi = eps.min(), eps.max()
    epsmin = lo - 0.1 * (hi - lo)
    epsmax = hi + 0.1 * (hi - lo)
    return np.array([epsmin + (epsmax - epsmin) * float(i) / float(NDOS) for i in range(NDOS)])


def make_dos(eps: np.ndarray, occbk: np.ndarray, e: np.ndarray):
    """eps, occbk: (NK, NB); loops ik -> ib as GS:252-259."""
    ewidth = 5.0 * (e[1] - e[0])
    dos = np.zeros(e.size)
    docc = np.zeros(e.size)
    for ik in range(eps.shape[0]):
        occmax = occbk[ik].max()
        for ib in range(eps.shape[1]):
            val = np.exp(-(eps[ik, ib] - e) ** 2 / ewidth ** 2)
            dos = dos + occmax * val
            docc = docc + occbk[ik, ib] * val
    return dos / (ewidth * math.sqrt(O.PI)), docc / (ewidth * math.sqrt(O.PI))


def gaps(eps: np.ndarray, NBocc: int):
    """The last two GSinfo columns (GS:51-52): minval(epsbk(NBocc+1:,:)) -
    maxval(epsbk(:NBocc,:)) and minval(epsbk(NBocc+1,:) - epsbk(NBocc,:)).

    With every band occupied the first section is empty, so Fortran's minval
    gives huge(1.d0).  The second then reads epsbk(NB+1,ik), past the first
    dimension: in column-major storage that is epsbk(1,ik+1) for ik < NK and
    lies outside the array for ik = NK, so only ik < NK take part here (and
    no k-point at all for NK = 1, which gives huge(1.d0) again)."""
    NK, NB = eps.shape
    vmax = eps[:, :NBocc].max()
    if NBocc < NB:
        return eps[:, NBocc:].min() - vmax, float(np.min(eps[:, NBocc] - eps[:, NBocc - 1]))
    fund = HUGE - vmax
    if NK == 1:
        return fund, HUGE
    return fund, float(np.min(eps[1:, 0] - eps[:-1, NB - 1]))


# ---------------------------------------------------------------------------
# The program
# ---------------------------------------------------------------------------
def run_program(cfg: O.Config, out_dir: str, vCk=O.k_vCk) -> dict:
    """Main (M:90-116): initialization and its debug files, Init_wf and
    Gram_Schmidt, GS_calculation with its files, RT_calculation with its file,
    FourierTr and WindowFourierTr.  Returns the arrays it wrote."""
    p = lambda name: os.path.join(out_dir, name)
    sysn = cfg.sys_name.strip()
    S = O.make_system(cfg, vCk=vCk)
    NK, NB, NBocc, NG = cfg.NK, cfg.NB, cfg.NBocc, cfg.NG
    with open(p("potential.out"), "w") as fh:
        for x, v in zip(S.rx, S.vion):
            fh.write(list_directed(x, v) + "\n")
    with open(p("vk.out"), "w") as fh:
        for ig in range(NG):
            for ik in range(NK):
                q = S.Gx[ig] + S.kx[ik]
                fh.write(list_directed(q, vCk(np.array([q]), cfg.acell, NG, NK)[0]) + "\n")
    u = O.gram_schmidt(S, O.init_wf(S))
    # ---- GS_calculation (GS:21-118)
    gs = O.gs_calculation(S, u)
    lines = [GSINFO_HEADER]
    for it in range(cfg.Nscf):
        eps, err = gs.eps_hist[it], gs.err_hist[it]
        fund, opt = gaps(eps, NBocc)
        lines.append("  " + f"{it + 1:5d}" + ew_list([gs.Etot[it + 1], gs.Etot[it + 1] - gs.Etot[it], gs.dnsdiff[it],
                                                      err.sum() / float(NB * NK), err.max(), fund, opt]))
    Ec = gs.Ecomps
    for lab, v in zip(("#Ekin  at SCF:", "#Eion  at SCF:", "#EH    at SCF:", "#Exc   at SCF:"), Ec):
        lines.append(lab + fw(v))
    eps, err = gs.epsbk, gs.epserrorbk
    H = O.HARTREE
    vtop = eps[:, :NBocc].max()
    cbot = eps[:, NBocc:].max() if NBocc < NB else -HUGE       # the reference prints maxval here (GS:81-82)
    fund, opt = gaps(eps, NBocc)
    for lab, v in (("#Min. value of the spectra: minval(epsbk)    =", eps.min()),
                   ("#Max. value of the spectra: maxval(epsbk)    =", eps.max()),
                   ("#Valence top: maxval(epsbk(:NBocc,:))        =", vtop),
                   ("#Conduction bottom: minval(epsbk(NBocc+1:,:))=", cbot),
                   ("#Fundamental gap: ", fund),
                   ("#Min. gap among same k-point: ", opt)):
        with np.errstate(over="ignore"):
            vH = v * H                        # huge * Hartree overflows to Infinity, as in Fortran
        lines.append(lab + fw(v) + " =" + fw(vH) + " [eV]")
    with open(p(f"{sysn}_GSinfo.out"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    e = dos_mesh(eps)
    dos, docc = make_dos(eps, S.occbk, e)
    with open(p(f"{sysn}_DoS.out"), "w") as fh:
        fh.write(BAND_HEADER + "\n")
        for ik in range(NK):
            fh.write("# " + band_record(ik + 1, S.kx[ik], err[ik].sum() / float(NB), eps[ik]) + "\n")
        for i in range(NDOS):
            fh.write(ew_list([e[i], dos[i], docc[i]], e=3) + "\n")
    with open(p(f"{sysn}_band.out"), "w") as fh:
        fh.write(BAND_HEADER + "\n")
        for ik in range(NK):
            fh.write(band_record(ik + 1, S.kx[ik], err[ik].sum() / float(NB), eps[ik]) + "\n")
    # ---- RT_calculation (RT:21-60)
    rt = O.rt_calculation(S, gs.ubk)
    with open(p(f"{sysn}_EtotNJEAt.out"), "w") as fh:
        fh.write("#time(it), Etot(it)-Etot0, N(it)-N0, J(it), E(it), A(it)\n")
        for it in range(cfg.NT):
            fh.write(ew_list([rt.time[it], rt.Etot[it], rt.Etot[it] - rt.Etot0, rt.Nele[it], rt.Nele[it] - rt.Nele0,
                              rt.Jtot[it], rt.E[it], rt.A[it]]) + "\n")
    # ---- FourierTr, WindowFourierTr (RT:64-65, 246-351)
    omega, JF, EF, AF, sigma, epsw = O.fourier_tr(cfg, rt.time, rt.Jtot, rt.Jtot0, rt.E, rt.A)
    with open(p(f"{sysn}_JEAF.out"), "w") as fh:
        fh.write("#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n")
        for i in range(cfg.Nomega):
            fh.write(ew_list([omega[i], JF[i].real, JF[i].imag, EF[i].real, EF[i].imag, AF[i].real, AF[i].imag])
                     + "\n")
    if cfg.field_option == "LR":
        with open(p(f"{sysn}_sigmaeps.out"), "w") as fh:
            fh.write("#omega(iomega), sigma(iomega), eps(iomega)\n")
            for i in range(cfg.Nomega):
                fh.write(ew_list([omega[i], sigma[i].real, sigma[i].imag, epsw[i].real, epsw[i].imag]) + "\n")
    else:
        w2, JF2, EF2, AF2 = O.window_fourier_tr(cfg, rt.time, rt.Jtot, rt.Jtot0, rt.E, rt.A)
        with open(p(f"{sysn}_JEAF_window.out"), "w") as fh:
            fh.write("#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n")
            for i in range(cfg.Nomega):
                fh.write(ew_list([w2[i], JF2[i].real, JF2[i].imag, EF2[i].real, EF2[i].imag, AF2[i].real,
                                  AF2[i].imag]) + "\n")
    return {"gs": gs, "rt": rt, "eps": eps, "dos": dos}
