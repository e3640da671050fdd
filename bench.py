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
NSCF_INIT, NCG_INIT = 3, 4
METRIC = "TDHF RK4 steps/s"
WORKLOAD_NAME = ("plain HF RK4, exchange-dominated: a=10, NG=256, NK=64, Nocc=NB=4, "
                 "2 ions (1.5@a/4, 0.5@3a/4), A0=0.1 w=0.057 T=600, dt=7e-4 (stable)")


def fock_flops_per_apply(NG, NK, NB, NBocc):
    """Algorithmic FLOPs of one ubkwbk_vFwbk: P*(2 FFTs + 16 NG), FFT = 5 N log2 N."""
    L = int(np.log2(NG))
    P = NK * NK * NB * NBocc
    return P * (10 * NG * L + 16 * NG)


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
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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


def make_cfg():
    from mattohf_gb300 import RunConfig
    return RunConfig.from_pulse(PULSE["A0"], PULSE["w"], PULSE["T"], dt=DT, NCG=NCG_INIT,
                                Nscf=NSCF_INIT, **WORKLOAD)


def initial_state(ctx):
    ctx.Init_wf()
    ctx.Gram_Schmidt()
    ctx.GS_calculation(NSCF_INIT, NCG_INIT)
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
            "data": "synthetic", "config": {"workload": WORKLOAD_NAME, "NG": cfg.NG, "NK": cfg.NK,
                                              "NB": cfg.NB, "NBocc": cfg.NBocc, "dt": cfg.dt,
                                              "parallelism": "replicas"},
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
    u0 = initial_state(ctx)
    K, W = args.steps, args.warmup
    A, Aave = fields(cfg, W + K)
    # --- warm-up (graph capture happens here)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:W], Aave[:W], cfg.dt)
    # --- timed region: K steps, each its own graph replay bracketed by events,
    #     with an L2 flush (a 512 MiB write) between steps outside the events.
    import ctypes as C
    import torch
    torch.cuda.set_device(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    step_ms = []
    dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for i in range(K):
            flush.fill_(float(i))
            torch.cuda.synchronize()
            ctx.rk4_run(A[W + i:W + i + 1], Aave[W + i:W + i + 1], cfg.dt)
            run_ms, _, _ = ctx.last_run_timing()
            step_ms.append(run_ms)
    torch.cuda.synchronize()
    dist.barrier()
    total_ms = dist.max(float(np.sum(step_ms)))
    ms_per_step = total_ms / K
    value = dist.ws * K / (total_ms * 1e-3)
    clocks = clk.summary()

    # --- dominant kernel (Fock pair kernel): per-launch CUDA-event time
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 1)
    ctx.set_orbitals(u0)
    ctx.rk4_run(A[:2], Aave[:2], cfg.dt)
    _, fock_ms, nf = ctx.last_run_timing()
    ctx.set_option(_capi.OPT_KERNEL_TIMING, 0)
    flops = fock_flops_per_apply(cfg.NG, cfg.NK, cfg.NB, cfg.NBocc)
    achieved = flops / (fock_ms / nf * 1e-3) / 1e12
    peak = C.c_double()
    lib.mattohf_diag_fp64_peak(dev, C.byref(peak))
    prof_traffic = None
    tp = os.path.join(ROOT, "profiles", "fock_traffic.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            prof_traffic = json.load(fh).get("bytes_per_launch")

    # --- end to end through the public C ABI with host buffers
    Ke = K
    ue = np.ascontiguousarray(u0)
    torch.cuda.synchronize()
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
        port.close()
        cpu = {"value": steps_cpu / t, "unit": "steps/s", "cores": thr, "kind": "port",
               "sample": f"{steps_cpu} RK4+observable steps of the same workload (C restatement, "
                         f"OpenMP over output columns)"}
    launches_per_step = 4 * 3 + 4  # (density, Fock, combine) x 4 stages + observables
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.ws, "steps": K,
            "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "NG": cfg.NG, "NK": cfg.NK, "NB": cfg.NB,
                       "NBocc": cfg.NBocc, "dt": cfg.dt, "parallelism": "replicas" if dist.ws > 1 else "single",
                       "l2": "flushed (512 MiB write) between timed steps", "graph": True},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                         "frac": achieved / peak.value if peak.value else None,
                         "traffic": prof_traffic, "kernel": "k_fock",
                         "flops_per_launch": flops, "launch_ms": fock_ms / nf,
                         "peak_source": "measured DFMA throughput on this GPU (mattohf_diag_fp64_peak)"},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches_per_step * K, "clocks": clocks}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-case", action="store_true",
                    help="small profiling case: 3 applies of h[u]u on the workload (no timing)")
    args = ap.parse_args()
    if args.profile_case:
        from mattohf_gb300 import build, Context
        build.build()
        cfg = make_cfg()
        with Context(cfg) as ctx:
            rng = np.random.default_rng(0)
            u = rng.standard_normal((cfg.NK, cfg.NB, cfg.NG)) + 1j * rng.standard_normal((cfg.NK, cfg.NB, cfg.NG))
            for _ in range(3):
                ctx.ubkwbk_hwbk(u, u, 0.01)
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            from mattohf_gb300 import build
            build.build()
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
