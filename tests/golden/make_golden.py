"""Generate the golden fixtures in this folder from the oracle.

The reference ships no golden vectors and cannot be built here, so these
fixtures are the oracle's own outputs on small seeded inputs (``parity
unpinned``: they pin the CUDA path to the oracle and the oracle to itself
across changes; the oracle is pinned to physics by tests/test_oracle.py).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import mattohf_oracle as O  # noqa: E402

CASES = {
    # one ion per cell, all bands occupied (the small plain configuration's shape, reduced)
    "hf_ng32_nk4": dict(acell=10.0, NG=32, NK=4, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0],
                        Rion=[0.5], Kion=[1], dt=0.005, NT=6, NCG=4, Nscf=3,
                        field_option="LP", omegac=0.057 * O.HARTREE, Tpulse=100 * O.ATOMTIME,
                        E0=0.05 * 0.057 * O.ATOMFIELD, nenvelope=2, phiCEP=0.057 * 100 / (4 * O.PI) % 1.0),
    # two species, odd NK, unoccupied bands, linear-response kick
    "hf_ng16_nk3_unocc": dict(acell=8.0, NG=16, NK=3, NB=3, NBocc=1, Zeff=[1.5, 0.5],
                              alpha=[1.0, 0.7], Rion=[0.25, 0.75], Kion=[1, 2], dt=0.01, NT=4,
                              NCG=2, Nscf=2, field_option="LR", dAc=0.01),
}


def run_case(name, kw):
    cfg = O.Config(**kw)
    S = O.make_system(cfg)
    rng = np.random.default_rng(1234)
    u = O.gram_schmidt(S, O.init_wf(S))
    w = rng.standard_normal(u.shape) + 1j * rng.standard_normal(u.shape)
    A = 0.137
    hw = O.ubkwbk_hwbk(S, u, w, A)
    vF = O.ubkwbk_vFwbk(S, u, w)
    tw = O.ubk_tubk(S, w, A)
    Ec = O.ubk_Ecomps(S, u, A)
    Je = O.ubk_Je(S, u, A)
    rt = O.rt_calculation(S, u, nt=cfg.NT)
    gs = O.gs_calculation(S, u, nscf=cfg.Nscf)
    out = dict(u=u, w=w, A=np.array(A), hw=hw, vF=vF, tw=tw, Ecomps=Ec, Je=np.array(Je),
               vion=S.vion, vCG=S.vCG, vCGkk=S.vCGkk, rt_Etot=rt.Etot, rt_Jtot=rt.Jtot,
               rt_Nele=rt.Nele, rt_u=rt.ubk, rt_A=rt.A, rt_dipole=rt.dipole,
               gs_Etot=gs.Etot, gs_eps=gs.epsbk, gs_err=gs.epserrorbk, gs_Je=gs.Je)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    with open(os.path.join(HERE, f"{name}.json"), "w") as fh:
        json.dump(dataclasses.asdict(cfg), fh, indent=1, sort_keys=True)


# long real-time runs: error accumulation over hundreds of steps
LONG_CASES = {
    # the CPU-runnable configuration's shape, pulse and step count, at a stable dt
    "rt2000_ng64_nk8": dict(acell=10.0, NG=64, NK=8, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0],
                           Rion=[0.5], Kion=[1], dt=0.01, NT=2000,
                           field_option="LP", omegac=0.057 * O.HARTREE, Tpulse=100 * O.ATOMTIME,
                           E0=0.05 * 0.057 * O.ATOMFIELD, nenvelope=2,
                           phiCEP=0.057 * 100 / (4 * O.PI) % 1.0),
}


def run_long(name, kw):
    cfg = O.Config(**kw)
    S = O.make_system(cfg)
    u = O.gram_schmidt(S, O.init_wf(S))
    rt = O.rt_calculation(S, u, nt=cfg.NT)
    out = dict(u0=u, rt_A=rt.A, rt_Etot=rt.Etot, rt_Jtot=rt.Jtot, rt_Nele=rt.Nele, rt_u=rt.ubk)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    with open(os.path.join(HERE, f"{name}.json"), "w") as fh:
        json.dump(dataclasses.asdict(cfg), fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    only = sys.argv[1:]
    for n, kw in CASES.items():
        if not only or n in only:
            run_case(n, kw)
            print("wrote", n)
    for n, kw in LONG_CASES.items():
        if not only or n in only:
            run_long(n, kw)
            print("wrote", n)
