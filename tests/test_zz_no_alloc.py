"""Allocation-free exchange entry point (mattohf_fock_noalloc), through the C ABI.

Callers that cannot allocate device memory where they need the exchange term
(a host code with a fixed device arena, a pool that must not grow, a loop that
must not take the allocator's locks) pass their own device buffers; the
library's scratch is a fixed 16 MiB device array.  This file is named to be
collected last.  It runs on its own in a fresh process as well as after the
other GPU tests.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the operator tolerance of the parity tests


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_fock_noalloc_matches_fock(built_lib):
    import torch
    from mattohf_gb300 import Context, RunConfig, _capi

    cfg = RunConfig(acell=9.0, NG=128, NK=8, NB=3, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
    nbw = 4
    with Context(cfg) as ctx:
        _, vCq = ctx.coulomb()
        d_vcq = torch.from_numpy(np.ascontiguousarray(vCq)).cuda()
        rng = np.random.default_rng(99)
        for call in range(2):  # two calls in a row share (and reuse) the scratch array
            u = rng.standard_normal((cfg.NK, cfg.NB, cfg.NG)) + 1j * rng.standard_normal((cfg.NK, cfg.NB, cfg.NG))
            w = rng.standard_normal((cfg.NK, nbw, cfg.NG)) + 1j * rng.standard_normal((cfg.NK, nbw, cfg.NG))
            ref = ctx.ubkwbk_vFwbk(u, w)          # existing entry point (context, host buffers)
            d_u = torch.from_numpy(u.view(np.float64).copy()).cuda()
            d_w = torch.from_numpy(w.view(np.float64).copy()).cuda()
            d_out = torch.full_like(d_w, float("nan"))
            torch.cuda.synchronize()
            st = built_lib.mattohf_fock_noalloc(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, nbw, d_vcq.data_ptr(),
                                                d_u.data_ptr(), d_w.data_ptr(), d_out.data_ptr(), None)
            assert st == _capi.OK, st
            torch.cuda.synchronize()
            got = d_out.cpu().numpy().view(np.complex128).reshape(ref.shape)
            assert _rel(got, ref) <= TOL, (call, _rel(got, ref))


def test_fock_noalloc_matches_oracle_ng512(built_lib):
    """A second shape, NG=512, NK=4, NB=NBocc=4 with nbw=4, against the oracle's
    ubkwbk_vFwbk (src/Functions.f90:237-261) with the context's Coulomb table;
    two calls in a row."""
    import torch
    from mattohf_gb300 import Context, RunConfig, _capi
    from conftest import to_oracle_config
    from oracle import mattohf_oracle as O

    cfg = RunConfig(acell=11.0, NG=512, NK=4, NB=4, NBocc=4, Zeff=[1.0], alpha=[1.0], Rion=[0.3], Kion=[1])
    nbw = 4
    with Context(cfg) as ctx:
        vCG, vCq = ctx.coulomb()
    S = O.make_system(to_oracle_config(cfg), vCk=lambda k, *a: np.zeros(np.shape(k)))
    NK = cfg.NK
    S.vCGkk = vCq[(np.arange(NK)[:, None] - np.arange(NK)[None, :] + NK - 1).reshape(-1)]
    S.vCG = vCG
    d_vcq = torch.from_numpy(np.ascontiguousarray(vCq)).cuda()
    rng = np.random.default_rng(7)
    for call in range(2):
        u = O.gram_schmidt(S, rng.standard_normal((NK, cfg.NB, cfg.NG)) + 1j * rng.standard_normal((NK, cfg.NB, cfg.NG)))
        w = u if call == 1 else rng.standard_normal((NK, nbw, cfg.NG)) + 1j * rng.standard_normal((NK, nbw, cfg.NG))
        ref = O.ubkwbk_vFwbk(S, u, w)
        d_u = torch.from_numpy(u.view(np.float64).copy()).cuda()
        d_w = torch.from_numpy(np.ascontiguousarray(w).view(np.float64).copy()).cuda()
        d_out = torch.full_like(d_w, float("nan"))
        torch.cuda.synchronize()
        st = built_lib.mattohf_fock_noalloc(cfg.NG, NK, cfg.NB, cfg.NBocc, nbw, d_vcq.data_ptr(), d_u.data_ptr(),
                                            d_w.data_ptr(), d_out.data_ptr(), None)
        assert st == _capi.OK, st
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.complex128).reshape(ref.shape)
        assert _rel(got, ref) <= TOL, (call, _rel(got, ref))


def test_fock_noalloc_rejects_oversize(built_lib):
    """Sizes whose partial sums exceed the fixed scratch are refused before any launch."""
    from mattohf_gb300 import _capi
    fake = 256  # never dereferenced: the size check comes first
    st = built_lib.mattohf_fock_noalloc(512, 64, 8, 8, 64, fake, fake, fake, fake, None)
    assert st == _capi.ERR_TOO_LARGE
