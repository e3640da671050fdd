"""Benchmark: TDHF RK4 steps/s of the exchange-dominated plain run on GB300.

Workload (one "step" = one RT_RK4_ubk step plus the per-step Nele, Etot and
Jtot of src/RT_calculation.f90:38-60, as timed by src/mATTOHF.f90:124):
  a = 10 bohr, NG = 256, NK = 64, NB = NBocc = 4, two ions per cell at a/4 and
  3a/4 with charges 1.5 and 0.5 (softening 1), soft-Coulomb e-e, HF exchange,
  LP pulse A0 = 0.1, w = 0.057, T = 600 a.u.  dt = 7e-4 a.u. (the configured
  dt = 0.01 is RK4-unstable for this grid; per-step cost does not depend on dt).
  Initial state: the reference's Gaussian guess, Gram-Schmidt, 3 SCF
  iterations (Krylov dim 16).  Synthetic inputs; no data files.

Lines printed (rank 0): one JSON object.  `--impl reference` times the CPU
restatement of the reference loop nest on all host cores instead.
N > 1 (torchrun): replicas only — every rank advances its own independent run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(acell=10.0, NG=256, NK=64, NB=4, NBocc=4, Zeff=[1.5, 0.5], alpha=[1.0, 1.0],
                Rion=[0.25, 0.75], Kion=[1, 2])
PULSE = dict(A0=0.1, w=0.057, T=600.0)
DT = 7e-4
# DRAM bytes (read + write) of one symmetric-exchange launch on WORKLOAD, ncu
FOCK_SYM_DRAM_BYTES_NG256_NK64_NB4 = 1_242_624 + 7_576_064
NSCF_INIT, NCG_INIT = 3, 4
METRIC = "TDHF RK4 steps/s"
WORKLOAD_NAME = ("plain HF RK4, exchange-dominated: a=10, NG=256, NK=64, Nocc=NB=4, "
                 "2 ions (1.5@a/4, 0.5@3a/4), A0=0.1 w=0.057 T=600, dt=7e-4 (stable)")


def fock_flops_per_apply(NG, NK, NB, NBocc):
    """Algorithmic FLOPs of one ubkwbk_vFwbk: P*(2 FFTs + 16 NG), FFT = 5 N log2 N."""
    L = int(np.log2(NG))
    P = NK * NK * NB * NBocc
    return P * (10 * NG * L + 16 * NG)


def fock_sym_flops_per_apply(NG, NK, NBocc):
    """Executed algorithmic FLOPs of the symmetric exchange (w == u, NB == NBocc).

    M = NK*NBocc occupied orbitals; M(M+1)/2 unordered pairs each take two
    FFTs (5 N log2 N) plus 16 N pointwise; the M(M-1)/2 off-diagonal pairs add
    the second accumulation (8 N).
    """
    L = int(np.log2(NG))
    M = NK * NBocc
    return M * (M + 1) // 2 * (10 * NG * L + 16 * NG) + M * (M - 1) // 2 * 8 * NG


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: the timed region begins after its first sample
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def bench_config(cfg):
    """The workload description printed by both arms (identical dicts)."""
    return {"workload": WORKLOAD_NAME, "NG": cfg.NG, "NK": cfg.NK, "NB": cfg.NB, "NBocc": cfg.NBocc,
            "dt": cfg.dt, "parallelism": "replicas",
            "l2": "inputs resident; the GPU arm writes 512 MiB (> L2) between timed steps"}


def make_cfg():
    from mattohf_gb300 import RunConfig
    return RunConfig.from_pulse(PULSE["A0"], PULSE["w"], PULSE["T"], dt=DT, NCG=NCG_INIT,
                                Nscf=NSCF_INIT, **WORKLOAD)


def initial_state(ctx, timing=None):
    ctx.Init_wf()
    ctx.Gram_Schmidt()
    ctx.GS_calculation(1, NCG_INIT)         # warm-up (tables, buffers, kernel attributes)
    ctx.Init_wf()
    ctx.Gram_Schmidt()
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.GS_calculation(NSCF_INIT, NCG_INIT)
    ctx.synchronize()
    if timing is not None:
        timing["gs_scf_iterations_per_s"] = NSCF_INIT / (time.perf_counter() - t0)
    return ctx.get_orbitals()


def fields(cfg, n):
    from mattohf_gb300 import define_afield
    # steps from the start of the pulse; NT large enough for n steps
    import dataclasses
    c = dataclasses.replace(cfg, NT=max(n, 1))
    _, A, Aave, _ = define_afield(c)
    return A, Aave


class CPUPort:
    """The oracle's C restatement (OpenMP over output columns, all host threads)."""

    def __init__(self, cfg, tables=None):
        import ctypes as C
        from oracle import build_cref
        from oracle import mattohf_oracle as O
        self.C = C
        self.lib = build_cref.load()
        self.D = C.POINTER(C.c_double)
        self.cfg = cfg
        ocfg = O.Config(**{k: getattr(cfg, k) for k in O.Config.__dataclass_fields__})
        vion = O.ion_potential(ocfg, np.arange(cfg.NG) / cfg.NG * cfg.acell)
        vCG, vCq = tables if tables is not None else (None, None)
        D = self.D
        t0 = time.perf_counter()
        self.h = self.lib.cref_create(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, cfg.acell, 1,
                                      vion.ctypes.data_as(D),
                                      None if vCG is None else vCG.ctypes.data_as(D),
                                      None if vCq is None else vCq.ctypes.data_as(D))
        self.setup_s = time.perf_counter() - t0
        self.threads = int(self.lib.cref_threads())

    def run(self, u0, steps: int, A, Aave) -> float:
        C, D = self.C, self.D
        u = np.ascontiguousarray(u0.copy())
        E, J, N = np.empty(steps), np.empty(steps), np.empty(steps)
        t0 = time.perf_counter()
        self.lib.cref_rk4_run(self.h, u.view(np.float64).ctypes.data_as(D), steps, C.c_double(self.cfg.dt),
                              A.ctypes.data_as(D), Aave.ctypes.data_as(D), E.ctypes.data_as(D),
                              J.ctypes.data_as(D), N.ctypes.data_as(D))
        return time.perf_counter() - t0

    def close(self):
        self.lib.cref_destroy(self.h)


def run_reference(args, dist):
    """--impl reference: the CPU restatement of the reference loop nest, all host cores."""
    if dist.rank != 0:
        return
    cfg = make_cfg()
    from oracle import mattohf_oracle as O
    ocfg = O.Config(**{k: getattr(cfg, k) for k in O.Config.__dataclass_fields__})
    S = O.make_system(ocfg, vCk=lambda k, *a: np.zeros(np.shape(k)), with_vion=True)
    u0 = O.gram_schmidt(S, O.init_wf(S))
    port = CPUPort(cfg)          # builds its own Coulomb tables (not timed)
    A, Aave = fields(cfg, 2)
    for _ in range(args.warmup):
        port.run(u0, 1, A, Aave)
    times = [port.run(u0, 1, A, Aave) for _ in range(args.steps)]
    port.close()
    per_step = float(np.mean(times))
    v = 1.0 / per_step
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": bench_config(cfg),
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": port.threads, "kind": "port",
                             "sample": "1 RK4+observable step per timed step; Coulomb tables built "
                                       f"once outside the timing ({port.setup_s:.1f} s)"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, dist):
    from mattohf_gb300 import Context, _capi
    dev = dist.local
    cfg = make_cfg()
    ctx = Context(cfg, device=dev)
    lib = ctx.lib
    gs_timing = {}
    u0 = initial_state(ctx, gs_timing)
    K, W = args.steps, args.warmup
    A, Aave = fields(cfg, W + K)
    # --- timed region: one mattohf_rk4_run of K steps (graph replay); the
    #     library brackets every step with CUDA events on its stream and writes
    #     512 MiB (> L2) between steps, outside the events.
    import ctypes as C
    ctx.set_option(_capi.OPT_L2_FLUSH, 512 << 20)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:W], Aave[:W], cfg.dt)          # warm-up incl. graph capture
    dist.barrier()
    ctx.synchronize()
    with ClockSampler(dev) as clk:
        ctx.rk4_run(A[W:W + K], Aave[W:W + K], cfg.dt)
    ctx.synchronize()
    dist.barrier()
    run_ms, _, _ = ctx.last_run_timing()
    ctx.set_option(_capi.OPT_L2_FLUSH, 0)
    total_ms = dist.max(run_ms)
    ms_per_step = total_ms / K
    value = dist.ws * K / (total_ms * 1e-3)
    clocks = clk.summary()

    # --- dominant kernel (Fock pair kernel): per-launch CUDA-event time
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 1)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:2], Aave[:2], cfg.dt)
    _, fock_ms, nf = ctx.last_run_timing()
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 0)
    flops = fock_sym_flops_per_apply(cfg.NG, cfg.NK, cfg.NBocc)
    achieved = flops / (fock_ms / nf * 1e-3) / 1e12
    peak = C.c_double()
    lib.mattohf_diag_fp64_peak(dev, C.byref(peak))
    dmma = C.c_double()
    lib.mattohf_diag_dmma_peak(dev, C.byref(dmma))
    # dram__bytes_read.sum + dram__bytes_write.sum of one k_fock_sym<256> launch on
    # this workload, from the ncu capture in profiles/k_fock_sym_ng256_nk64_nb4.md
    prof_traffic = None
    if (cfg.NG, cfg.NK, cfg.NBocc) == (256, 64, 4):
        prof_traffic = FOCK_SYM_DRAM_BYTES_NG256_NK64_NB4

    # --- the same timed region with the exchange transforms in double-float
    #     arithmetic (MATTOHF_OPT_FOCK_DF64; parity-tested at the FP64 tolerances)
    ctx.set_option(_capi.OPT_FOCK_DF64, 1)
    ctx.set_option(_capi.OPT_L2_FLUSH, 512 << 20)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:W], Aave[:W], cfg.dt)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[W:W + K], Aave[W:W + K], cfg.dt)
    df_ms, _, _ = ctx.last_run_timing()
    ctx.set_option(_capi.OPT_L2_FLUSH, 0)
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 1)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:2], Aave[:2], cfg.dt)
    _, df_fock_ms, df_nf = ctx.last_run_timing()
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 0)
    ctx.set_option(_capi.OPT_FOCK_DF64, 0)
    double_float = {"value": K / (df_ms * 1e-3), "unit": "steps/s", "ms_per_step": df_ms / K,
                    "fock_launch_ms": df_fock_ms / df_nf,
                    "note": "exchange pair transforms in double-float (2xFP32, 48-bit significand) on the "
                            "FP32 pipe; parity within the FP64 tolerances (1e-12 per apply, 1e-10 RT)"}

    # --- end to end through the public C ABI with host buffers
    Ke = K
    ue = np.ascontiguousarray(u0)
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.set_orbitals(ue)
    E, J, N = ctx.rk4_run(A[W:W + Ke], Aave[W:W + Ke], cfg.dt)
    uo = ctx.get_orbitals()
    t_e2e = time.perf_counter() - t0
    t_e2e = dist.max(t_e2e)
    h2d = ue.nbytes + 2 * 8 * Ke
    d2h = uo.nbytes + 3 * 8 * Ke
    e2e = {"value": dist.ws * Ke / t_e2e, "unit": "steps/s", "h2d_bytes_per_step": h2d / Ke,
           "d2h_bytes_per_step": d2h / Ke}

    cpu = None
    if dist.rank == 0 and dist.ws == 1 and not args.no_cpu:
        port = CPUPort(cfg, tables=ctx.coulomb())
        steps_cpu = args.cpu_steps
        Ac, Aavec = fields(cfg, steps_cpu)
        t = port.run(u0, steps_cpu, Ac, Aavec)
        thr = port.threads
        # the same port on one core (one step)
        port.lib.cref_set_threads(1)
        t1 = port.run(u0, 1, Ac, Aavec)
        port.lib.cref_set_threads(thr)
        port.close()
        cpu = {"value": steps_cpu / t, "unit": "steps/s", "cores": thr, "kind": "port",
               "sample": f"{steps_cpu} RK4+observable steps of the same workload (C restatement, "
                         f"OpenMP over output columns)",
               "one_core": {"value": 1.0 / t1, "unit": "steps/s", "cores": 1, "sample": "1 step"}}
    # per step: 4 stages x (k_dens_partial, k_density, kinetic k_combine pass, k_fock_sym,
    # k_sym_reduce, exchange k_combine pass) + k_ex_finalize + observables (k_dens_partial,
    # k_density, k_combine, k_obs_reduce); per run: the closing exchange apply (7 launches)
    launches_per_step = 4 * 6 + 1 + 4
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.ws, "steps": K,
            "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(cfg), "graph": True,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                         "frac": achieved / peak.value if peak.value else None,
                         "traffic": prof_traffic, "kernel": "k_fock_sym",
                         "flops_per_launch": flops, "launch_ms": fock_ms / nf,
                         "peak_source": "measured DFMA throughput on this GPU (mattohf_diag_fp64_peak)",
                         "fp64_tensor_peak": dmma.value,
                         "fp64_tensor_peak_source": "measured DMMA (mma.sync m8n8k4 f64) throughput, "
                                                    "mattohf_diag_dmma_peak",
                         "hbm_peak_gbs": hbm_peak(),
                         "flops_model": "symmetric exchange: M(M+1)/2 pairs x (10 N log2 N + 16 N) + M(M-1)/2 x 8 N, M = NK*NBocc"},
            "ground_state": {"value": gs_timing.get("gs_scf_iterations_per_s"), "unit": "SCF iterations/s",
                             "note": f"GS_calculation, Krylov dim NB*NCG = {cfg.NB * NCG_INIT}, "
                                     f"{2 * NCG_INIT + 2} h-applies per iteration, host wall clock"},
            "cpu_baseline": cpu, "e2e": e2e, "double_float_exchange": double_float, "gpu_launches": launches_per_step * K + 7, "clocks": clocks}
    ctx.close()
    if dist.rank == 0 and dist.ws == 1 and not args.no_extras:
        # the metric's other clauses, each on its own workload (outside the
        # timed region above): the CPU-runnable configuration, the batched
        # ensemble against the plain one-run-at-a-time path, and the adjoint
        line["small"] = measure_small()
        line["ensemble"] = measure_ensemble(args.runs, args.ens_steps, args.ens_warmup)
        line["adjoint"] = measure_adjoint(args.adj_steps, args.fd_samples)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


ENSEMBLE_DT = 1.5e-3
ADJ_DT = 2.5e-3


def hbm_peak():
    """Measured copy bandwidth of this GPU pool (MEASURED_PEAKS.json), or None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh).get("hbm_gbs")
    except (OSError, ValueError):
        return None


def measure_ensemble(R: int, K: int, W: int, with_df: bool = True) -> dict:
    """Batched ensemble of independent runs vs the same runs one at a time.

    R runs (256 by default), seed 1: NK in {8,16,32,64}, Nocc = NB in {1..4},
    NG = 128, a in U[8,14], A0 log-uniform in [0.005, 0.2], w in U[0.03, 0.1],
    T = 200; one ion (Z=2, alpha=1) at a/2; dt = 1.5e-3 (the configured 0.02
    is RK4-unstable at NG = 128).  Initial state: Gaussian guess + Gram-Schmidt.
    Device time of K graph-replayed ensemble steps after W warm-up steps; the
    plain path is every member's own graph-replayed loop, one run at a time.
    """
    import math
    from mattohf_gb300 import Batch, RunConfig, define_afield, _capi
    import ctypes as C
    import dataclasses
    rng = np.random.default_rng(1)
    nks = rng.choice([8, 16, 32, 64], size=R)
    noc = rng.integers(1, 5, size=R)
    acell = rng.uniform(8.0, 14.0, size=R)
    A0 = np.exp(rng.uniform(math.log(0.005), math.log(0.2), size=R))
    w = rng.uniform(0.03, 0.1, size=R)
    cfgs = [RunConfig.from_pulse(float(A0[r]), float(w[r]), 200.0, acell=float(acell[r]), NG=128,
                                 NK=int(nks[r]), NB=int(noc[r]), NBocc=int(noc[r]), Zeff=[2.0],
                                 alpha=[1.0], Rion=[0.5], Kion=[1], dt=ENSEMBLE_DT) for r in range(R)]
    t0 = time.perf_counter()
    b = Batch(cfgs)
    setup_s = time.perf_counter() - t0
    A = np.empty((R, W + K))
    for r, c in enumerate(cfgs):
        A[r] = define_afield(dataclasses.replace(c, NT=W + K))[1]
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    u0 = []
    for r in range(R):
        b[r].Init_wf()
        b[r].Gram_Schmidt()
        u0.append(b[r].get_orbitals())
    # the autotuner picks the exchange tile shared by the runs' tile pairs
    # (outside the timed region; it restores the orbitals)
    t0 = time.perf_counter()
    tuned = b.autotune(steps=max(2, min(K, 5)))
    tune_s = time.perf_counter() - t0
    b.rk4_run(A[:, :W], Aave[:, :W], ENSEMBLE_DT)
    b.rk4_run(A[:, W:], Aave[:, W:], ENSEMBLE_DT)
    t_batch = b.last_run_ms()
    t_batch_df = None
    if with_df:
        # the same batch with the exchange transforms in double-float arithmetic
        for r in range(R):
            b[r].set_orbitals(u0[r])
        b.set_option(_capi.OPT_FOCK_DF64, 1)
        b.rk4_run(A[:, :W], Aave[:, :W], ENSEMBLE_DT)
        b.rk4_run(A[:, W:], Aave[:, W:], ENSEMBLE_DT)
        t_batch_df = b.last_run_ms()
        b.set_option(_capi.OPT_FOCK_DF64, 0)
    # the same runs one at a time through each member's own (graph-replayed) path
    t_plain = 0.0
    for r in range(R):
        m = b[r]
        m.set_orbitals(u0[r])
        m.rk4_run(A[r, :W], Aave[r, :W], ENSEMBLE_DT)
        m.rk4_run(A[r, W:], Aave[r, W:], ENSEMBLE_DT)
        t_plain += m.last_run_timing()[0]
    b.close()
    kb = float(sum(c.NK * c.NB for c in cfgs))
    # executed algorithmic FP64 work of one ensemble step: 4 symmetric exchange
    # applies per run (the first stage's doubles as the previous step's Ex)
    flops_step = float(sum(4 * fock_sym_flops_per_apply(c.NG, c.NK, c.NBocc) for c in cfgs))
    peak = C.c_double()
    _capi.load().mattohf_diag_fp64_peak(0, C.byref(peak))
    achieved = flops_step * K / (t_batch * 1e-3) / 1e12
    out = {"metric": "TDHF RK4 steps/s (ensemble aggregate)", "value": R * K / (t_batch * 1e-3),
           "unit": "run-steps/s", "steps": K, "warmup": W, "higher_is_better": True,
           "plain_value": R * K / (t_plain * 1e-3), "batched_over_plain": t_plain / t_batch,
           "kpoint_orbital_steps_per_s": kb * K / (t_batch * 1e-3),
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                        "frac": achieved / peak.value if peak.value else None,
                        "flops_per_step": flops_step,
                        "flops_model": "exchange only: 4 symmetric applies per run per step"},
           "double_float_exchange": None if t_batch_df is None else R * K / (t_batch_df * 1e-3),
           "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{R} runs, NK in {{8,16,32,64}}, Nocc in {{1..4}}, NG=128, a in [8,14], "
                                  f"dt={ENSEMBLE_DT}", "setup_s": setup_s,
                      "autotune": {"sym_tile": tuned["sym_tile"], "step_us": tuned["step_us"], "tune_s": tune_s}}}
    return out


def run_ensemble(args):
    print(json.dumps(measure_ensemble(args.runs, args.steps, args.warmup)), flush=True)


def measure_adjoint(nt: int, fd_samples: int) -> dict:
    """Adjoint gradient / forward time on the differentiation workload.

    a = 10, one ion (Z=2) at a/2, NK = 16, Nocc = NB = 2, NG = 128, nt steps
    (4000 by default) at dt = 2.5e-3 (the configured 0.025 is RK4-unstable
    here); control = the A0 = 0.05, w = 0.057, T = 100 pulse plus N(0, 1e-3)
    noise (seed 2); objective = absorbed energy; checkpoints every 100 steps,
    and the interval the library fits to free memory.  The gradient is checked
    by central differences of the plain forward on `fd_samples` random samples:
    at h = 1e-6 (the workload's step) with each sample's round-off bound, the
    larger spread between the quotient at h and those at 1.25 h and 0.8 h, and
    at h = 1e-4, where round-off is 100x smaller and truncation is O(h^2).
    """
    from mattohf_gb300 import Context, RunConfig, define_afield, aave_from_samples
    cfg = RunConfig.from_pulse(0.05, 0.057, 100.0, acell=10.0, NG=128, NK=16, NB=2, NBocc=2, Zeff=[2.0],
                               alpha=[1.0], Rion=[0.5], Kion=[1], dt=ADJ_DT, NT=nt)
    rng = np.random.default_rng(2)
    A = define_afield(cfg)[1] + 1e-3 * rng.standard_normal(nt)
    Aave = aave_from_samples(A)
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        ctx.GS_calculation(5, 4)
        u0 = ctx.get_orbitals()
        E0 = ctx.observables(0.0)["Etot"]
        # forward: the plain RT loop with per-step observables
        ctx.rk4_run(A[:50], Aave[:50], cfg.dt)       # warm-up and graph capture
        ctx.set_orbitals(u0)
        ctx.rk4_run(A, Aave, cfg.dt)
        t_fwd = ctx.last_run_timing()[0]
        ctx.set_orbitals(u0)
        ctx.adjoint(A[:50], cfg.dt, "energy", ckpt_every=10)   # warm-up
        ctx.set_orbitals(u0)
        L, g, gv = ctx.adjoint(A, cfg.dt, "energy", ckpt_every=100)
        _, t_adj = ctx.adjoint_timing()
        # checkpoint interval chosen by the library to fit device memory: here
        # every stage input fits, so the backward pass recomputes nothing
        ctx.set_orbitals(u0)
        L_auto, g_auto, _ = ctx.adjoint(A, cfg.dt, "energy", ckpt_every=0)
        _, t_adj_auto = ctx.adjoint_timing()
        auto_diff = float(np.max(np.abs(g_auto - g)) / np.max(np.abs(g)))

        def obj(Ax):
            ctx.set_orbitals(u0)
            E, _, _ = ctx.rk4_run(Ax, aave_from_samples(Ax), cfg.dt)
            return E[-1] - E0

        rows = []
        for i, n in enumerate(rng.choice(nt, size=fd_samples, replace=False)):
            q = {}
            # h = 1e-4 on the first 8 samples only (it serves as a cross-check)
            for h in ((1e-4, 1e-6, 1.25e-6, 0.8e-6) if i < 8 else (1e-6, 1.25e-6, 0.8e-6)):
                Ap, Am = A.copy(), A.copy()
                Ap[n] += h
                Am[n] -= h
                q[h] = (obj(Ap) - obj(Am)) / (2 * h)
            rows.append((g[n], q.get(1e-4, np.nan), q[1e-6],
                         max(abs(q[1e-6] - q[1.25e-6]), abs(q[1e-6] - q[0.8e-6]))))
    fd = {"samples": 0}
    if rows:
        gs_, f4, f6, spread = np.array(rows).T
        rel6 = np.abs(gs_ - f6) / np.abs(f6)
        bound6 = 1e-6 + 3 * spread / np.abs(f6)
        m4 = np.isfinite(f4)
        rel4 = np.abs(gs_[m4] - f4[m4]) / np.abs(f4[m4])
        fd = {"samples": int(fd_samples),
              "h1e-6": {"max_rel_err_per_sample": float(rel6.max()),
                        "median_rel_err": float(np.median(rel6)),
                        "normwise_rel_err": float(np.max(np.abs(gs_ - f6)) / np.max(np.abs(f6))),
                        "within_1e-6_plus_roundoff": int(np.sum(rel6 <= bound6)),
                        "max_roundoff_bound_rel": float((3 * spread / np.abs(f6)).max()),
                        "note": "round-off bound per sample = 3 x max(|fd(h) - fd(1.25 h)|, |fd(h) - fd(0.8 h)|)"},
              "h1e-4": {"samples": int(m4.sum()), "max_rel_err_per_sample": float(rel4.max())}}
    return {"metric": "adjoint-gradient/forward time ratio", "value": t_adj / t_fwd, "unit": "ratio",
            "higher_is_better": False, "forward_ms": t_fwd, "adjoint_ms": t_adj, "steps": nt,
            "objective": L,
            "auto_checkpoint": {"value": t_adj_auto / t_fwd, "adjoint_ms": t_adj_auto,
                                "note": "ckpt_every=0: all stage inputs stored, no recomputation",
                                "grad_rel_diff_vs_ckpt100": auto_diff},
            "fd": fd,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"a=10, NK=16, Nocc=2, NG=128, {nt} steps, pulse+N(0,1e-3), "
                                   "checkpoints every 100", "dt": cfg.dt}}


def run_adjoint(args):
    print(json.dumps(measure_adjoint(args.adj_steps, args.fd_samples)), flush=True)


def measure_small() -> dict:
    """The CPU-runnable configuration: a = 10, NG = 64, NK = 8, Nocc = NB = 2, one
    ion (Z=2, alpha=1) at a/2, pulse A0 = 0.05, w = 0.057, T = 100, 2000 RK4 steps
    at dt = 0.01 (the configured 0.02 is RK4-unstable at NG = 64), ground state
    from 20 SCF iterations with Krylov dim 8.  GPU steps/s (graph replay, per-step
    observables) against the C restatement on all host cores.
    """
    from mattohf_gb300 import Context, RunConfig, define_afield, aave_from_samples
    nt = 2000
    cfg = RunConfig.from_pulse(0.05, 0.057, 100.0, acell=10.0, NG=64, NK=8, NB=2, NBocc=2, Zeff=[2.0],
                               alpha=[1.0], Rion=[0.5], Kion=[1], dt=0.01, NT=nt, NCG=4)
    A = define_afield(cfg)[1]
    Aave = aave_from_samples(A)
    with Context(cfg) as ctx:
        ctx.Init_wf()
        ctx.Gram_Schmidt()
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.GS_calculation(20, cfg.NCG)
        ctx.synchronize()
        t_gs = time.perf_counter() - t0
        u0 = ctx.get_orbitals()
        # the autotuner picks the fused-stage CTAs per column and fused vs tiled
        # stepping (outside the timed region; it restores the orbitals)
        tuned = ctx.autotune(steps=50)
        ctx.rk4_run(A[:50], Aave[:50], cfg.dt)
        ctx.set_orbitals(u0)
        ctx.rk4_run(A, Aave, cfg.dt)
        t_gpu = ctx.last_run_timing()[0] * 1e-3
        tables = ctx.coulomb()
    port = CPUPort(cfg, tables=tables)
    ncpu = 200
    t_cpu = port.run(u0, ncpu, A[:ncpu], Aave[:ncpu])
    thr = port.threads
    port.close()
    return {"metric": "TDHF RK4 steps/s (CPU-runnable configuration)", "value": nt / t_gpu, "unit": "steps/s",
            "higher_is_better": True, "steps": nt, "dtype": "f64", "data": "synthetic",
            "ground_state_s": t_gs, "kpoint_orbital_steps_per_s": cfg.NK * cfg.NB * nt / t_gpu,
            "cpu_baseline": {"value": ncpu / t_cpu, "unit": "steps/s", "cores": thr, "kind": "port",
                             "sample": f"{ncpu} RK4+observable steps"},
            "config": {"workload": "a=10, NG=64, NK=8, Nocc=NB=2, 1 ion, A0=0.05 w=0.057 T=100, dt=0.01",
                       "graph": True, "autotune": tuned}}


def run_small(args):
    print(json.dumps(measure_small()), flush=True)


def measure_large(variants: int, K: int, W: int) -> dict:
    """The largest configuration: a = 12, NG = 512, NK = 128, NB = Nocc = 8,
    three ions (Z = 1 at a/6, a/2, 5a/6), `variants` pulse variants (A0 in
    U[0.02, 0.2], w in U[0.04, 0.08], T = 200, seed 3), dt = 2.5e-4 (the
    configured 0.01 is RK4-unstable here).  Every variant forward for a window
    of K steps as one batch, then the adjoint of the absorbed energy for every
    variant over the same window (mattohf_batch_adjoint: members in turn, each
    with its checkpoint segment fitted to the free device memory, and once with
    four segments and recomputation), and one variant alone with the
    double-float exchange."""
    import dataclasses
    from mattohf_gb300 import Batch, RunConfig, define_afield, _capi
    rng = np.random.default_rng(3)
    A0 = rng.uniform(0.02, 0.2, size=variants)
    w = rng.uniform(0.04, 0.08, size=variants)
    dt = 2.5e-4
    cfgs = [RunConfig.from_pulse(float(A0[r]), float(w[r]), 200.0, acell=12.0, NG=512, NK=128, NB=8, NBocc=8,
                                 Zeff=[1.0], alpha=[1.0], Rion=[1 / 6, 0.5, 5 / 6], Kion=[1, 1, 1], dt=dt,
                                 NT=W + K) for r in range(variants)]
    t0 = time.perf_counter()
    b = Batch(cfgs)
    setup_s = time.perf_counter() - t0
    A = np.stack([define_afield(c)[1] for c in cfgs])
    Aave = np.concatenate([0.5 * A[:, :1], 0.5 * (A[:, 1:] + A[:, :-1])], axis=1)
    b[0].Init_wf()
    b[0].Gram_Schmidt()
    u0 = b[0].get_orbitals()
    for r in range(1, variants):
        b[r].set_orbitals(u0)
    b.rk4_run(A[:, :W], Aave[:, :W], dt)                  # warm-up and graph capture
    for r in range(variants):
        b[r].set_orbitals(u0)
    b.rk4_run(A[:, W:], Aave[:, W:], dt)
    t_fwd = b.last_run_ms()
    for r in range(variants):
        b[r].set_orbitals(u0)
    b.adjoint(A[:, W:], dt, "energy", ckpt_every=0)
    t_adj = b.last_run_ms()
    for r in range(variants):
        b[r].set_orbitals(u0)
    b.adjoint(A[:, W:], dt, "energy", ckpt_every=max(1, K // 4))
    t_adj_ck = b.last_run_ms()
    m = b[0]
    m.set_option(_capi.OPT_FOCK_DF64, 1)
    m.set_orbitals(u0)
    m.rk4_run(A[0, :W], Aave[0, :W], dt)
    m.set_orbitals(u0)
    m.rk4_run(A[0, W:], Aave[0, W:], dt)
    t_df = m.last_run_timing()[0]
    m.set_option(_capi.OPT_FOCK_DF64, 0)
    b.close()
    return {"metric": "TDHF RK4 steps/s (largest shape, batched pulse variants)",
            "value": variants * K / (t_fwd * 1e-3), "unit": "run-steps/s",
            "kpoint_orbital_steps_per_s": variants * 128 * 8 * K / (t_fwd * 1e-3),
            "dtype": "f64", "data": "synthetic", "steps": K, "warmup": W,
            "variants": variants, "forward_ms": t_fwd,
            "adjoint": {"value": t_adj / t_fwd, "unit": "batched adjoint / batched forward time", "adjoint_ms": t_adj,
                        "checkpoint": "fitted to free memory (every stage input of the window stored)",
                        "four_segments": {"value": t_adj_ck / t_fwd, "adjoint_ms": t_adj_ck,
                                          "checkpoint": f"every {max(1, K // 4)} steps, recomputation"}},
            "double_float_exchange_one_variant": K / (t_df * 1e-3),
            "config": {"workload": f"a=12, NG=512, NK=128, Nocc=NB=8, 3 ions, {variants} pulse variants, "
                                   f"dt={dt}, window of {K} steps", "setup_s": setup_s}}


def run_large(args):
    print(json.dumps(measure_large(args.variants, args.steps, args.warmup)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="plain", choices=["plain", "ensemble", "adjoint", "large", "small"])
    ap.add_argument("--runs", type=int, default=256)
    ap.add_argument("--variants", type=int, default=32, help="pulse variants of --workload large")
    ap.add_argument("--adj-steps", type=int, default=4000)
    ap.add_argument("--fd-samples", type=int, default=32)
    ap.add_argument("--ens-steps", type=int, default=10, help="timed ensemble steps in the default line")
    ap.add_argument("--ens-warmup", type=int, default=3)
    ap.add_argument("--no-extras", action="store_true",
                    help="default line without the ensemble, adjoint and CPU-runnable fields")
    ap.add_argument("--profile-df", action="store_true",
                    help="with --profile-case / --profile-step: double-float exchange transforms")
    ap.add_argument("--profile-case", action="store_true",
                    help="small profiling case: 3 applies of h[u]u on the workload (no timing)")
    ap.add_argument("--profile-step", action="store_true",
                    help="profiling case: 3 RK4 steps of the workload without graph replay (no timing)")
    ap.add_argument("--profile-gs", action="store_true",
                    help="profiling case: one ground-state SCF iteration of the workload (no timing)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="profiling case: a 4-step adjoint on the differentiation shape (no timing)")
    ap.add_argument("--profile-small", action="store_true",
                    help="profiling case: 3 RK4 steps of the CPU-runnable shape through the fused stages (no timing)")
    ap.add_argument("--profile-extras", action="store_true",
                    help="profiling case: spectra, propagators, allocation-free exchange, double-float "
                         "ensemble step, separate-launch adjoint and the peak probes (no timing)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="profiling case: 2 batched steps of the first 32 runs of the ensemble mix (no timing)")
    args = ap.parse_args()
    if args.profile_extras:
        # the kernels outside the RK4 step: spectra at the exchange-dominated
        # workload's sizes, the Taylor / predictor-corrector propagators, the
        # allocation-free exchange, a double-float ensemble step, the separate-
        # launch adjoint with the current objective, and the two peak probes
        import ctypes as C
        import dataclasses
        import torch
        from mattohf_gb300 import build, Batch, Context, RunConfig, _capi
        from mattohf_gb300.driver import fourier
        build.build()
        lib = _capi.load()
        pk = C.c_double()
        lib.mattohf_diag_fp64_peak(0, C.byref(pk))
        lib.mattohf_diag_dmma_peak(0, C.byref(pk))
        cfg = dataclasses.replace(make_cfg(), NT=20000, Nomega=4000, omegaM=4.0)
        nt = cfg.NT
        t = cfg.dt * np.arange(nt)
        J = 1e-3 * np.sin(0.05 * np.arange(nt))
        Ef = 1e-2 * np.cos(0.05 * np.arange(nt))
        for window in (False, True):
            fourier(cfg, t, J, 0.0, Ef, Ef, window)
        small = RunConfig(acell=10.0, NG=64, NK=8, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
        with Context(small) as ctx:
            ctx.Init_wf()
            ctx.Gram_Schmidt()
            for v in ("TE", "TEPC", "TEPC2"):
                ctx.RT_TE_ubk(0.01, 0.002, v)
            ctx.set_option(_capi.OPT_SMALL_STAGES, 0)
            ctx.adjoint(0.01 * np.sin(0.3 * np.arange(1, 4)), 0.002, "current", ckpt_every=2)
            _, vCq = ctx.coulomb()
        noa = RunConfig(acell=9.0, NG=128, NK=8, NB=3, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
        with Context(noa) as ctx:
            _, vCq = ctx.coulomb()
        rng = np.random.default_rng(9)
        u = rng.standard_normal((8, 3, 128, 2))
        w = rng.standard_normal((8, 4, 128, 2))
        d_vcq = torch.from_numpy(np.ascontiguousarray(vCq)).cuda()
        d_u, d_w = torch.from_numpy(u).cuda(), torch.from_numpy(w).cuda()
        d_out = torch.empty_like(d_w)
        torch.cuda.synchronize()
        lib.mattohf_fock_noalloc(128, 8, 3, 2, 4, d_vcq.data_ptr(), d_u.data_ptr(), d_w.data_ptr(),
                                 d_out.data_ptr(), None)
        torch.cuda.synchronize()
        cfgs = [RunConfig(acell=10.0, NG=64, NK=k, NB=b, NBocc=b, Zeff=[2.0], alpha=[1.0], Rion=[0.5],
                          Kion=[1]) for k, b in [(8, 2), (16, 1), (4, 4)]]
        with Batch(cfgs) as bt:
            for r in range(len(cfgs)):
                bt[r].Init_wf()
                bt[r].Gram_Schmidt()
            bt.set_option(_capi.OPT_FOCK_DF64, 1)
            A = np.full((len(cfgs), 2), 0.01)
            bt.rk4_run(A, A, 0.002)
        return
    if args.profile_small:
        from mattohf_gb300 import build, Context, RunConfig, _capi
        build.build()
        cfg = RunConfig(acell=10.0, NG=64, NK=8, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
        with Context(cfg) as ctx:
            ctx.Init_wf()
            ctx.Gram_Schmidt()
            ctx.set_option(_capi.OPT_SMALL_STAGES, 1)
            ctx.set_option(_capi.OPT_GRAPH, 0)
            A = np.full(3, 0.01)
            ctx.rk4_run(A, A, 0.01)
        return
    if args.profile_batch:
        from mattohf_gb300 import build, Batch, RunConfig
        build.build()
        rng = np.random.default_rng(1)
        nks = rng.choice([8, 16, 32, 64], size=256)[:32]
        noc = rng.integers(1, 5, size=256)[:32]
        cfgs = [RunConfig(acell=10.0, NG=128, NK=int(k), NB=int(o), NBocc=int(o), Zeff=[2.0], alpha=[1.0],
                          Rion=[0.5], Kion=[1]) for k, o in zip(nks, noc)]
        with Batch(cfgs) as b:
            for r in range(len(cfgs)):
                b[r].Init_wf()
                b[r].Gram_Schmidt()
            A = np.full((len(cfgs), 2), 0.01)
            b.rk4_run(A, A, ENSEMBLE_DT)
        return
    if args.profile_gs:
        from mattohf_gb300 import build, Context
        build.build()
        with Context(make_cfg()) as ctx:
            ctx.Init_wf()
            ctx.Gram_Schmidt()
            ctx.GS_calculation(1, NCG_INIT)
        return
    if args.profile_adjoint:
        from mattohf_gb300 import build, Context, RunConfig
        build.build()
        cfg = RunConfig(acell=10.0, NG=128, NK=16, NB=2, NBocc=2, Zeff=[2.0], alpha=[1.0], Rion=[0.5], Kion=[1])
        with Context(cfg) as ctx:
            ctx.Init_wf()
            ctx.Gram_Schmidt()
            ctx.adjoint(0.01 * np.sin(0.3 * np.arange(1, 5)), ADJ_DT, "energy", ckpt_every=2)
        return
    if args.profile_step:
        from mattohf_gb300 import build, Context, _capi
        build.build()
        cfg = make_cfg()
        with Context(cfg) as ctx:
            rng = np.random.default_rng(0)
            shape = (cfg.NK, cfg.NB, cfg.NG)
            ctx.set_orbitals(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
            ctx.Gram_Schmidt()
            if args.profile_df:
                ctx.set_option(_capi.OPT_FOCK_DF64, 1)
            ctx.set_option(_capi.OPT_GRAPH, 0)
            A = np.full(3, 0.01)
            ctx.rk4_run(A, A, 1e-4)
        return
    if args.profile_case:
        from mattohf_gb300 import build, Context, _capi
        build.build()
        cfg = make_cfg()
        with Context(cfg) as ctx:
            if args.profile_df:
                ctx.set_option(_capi.OPT_FOCK_DF64, 1)
            rng = np.random.default_rng(0)
            u = rng.standard_normal((cfg.NK, cfg.NB, cfg.NG)) + 1j * rng.standard_normal((cfg.NK, cfg.NB, cfg.NG))
            for _ in range(3):
                ctx.ubkwbk_hwbk(u, u, 0.01)
        return
    dist = Dist()
    try:
        if args.workload == "ensemble":
            from mattohf_gb300 import build
            build.build()
            run_ensemble(args)
        elif args.workload == "adjoint":
            from mattohf_gb300 import build
            build.build()
            run_adjoint(args)
        elif args.workload == "large":
            from mattohf_gb300 import build
            build.build()
            run_large(args)
        elif args.workload == "small":
            from mattohf_gb300 import build
            build.build()
            run_small(args)
        elif args.impl == "reference":
            run_reference(args, dist)
        else:
            from mattohf_gb300 import build
            build.build()
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
