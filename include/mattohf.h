/* C ABI of the GB300-native mATTOHF hot path.
 *
 * The reference (Fortran 90, Yasushi-Shinohara/mATTOHF) has no plugin API: its
 * hot path is a set of module procedures in src/Functions.f90 and external
 * subroutines in src/RT_calculation.f90 / src/GS_calculation.f90, operating on
 * global module state (src/Global_variables.f90).  Each entry point below
 * names the reference routine it replaces.  All functions are iso_c_binding
 * compatible: scalars by value, arrays as plain pointers, `int` status return.
 *
 * Array conventions
 *   orbitals   complex128 interleaved (re, im), Fortran layout ubk(1:NG,1:NB,1:NK),
 *              i.e. C [NK][NB][NG][2] doubles; blocks of `nbw` bands use
 *              [NK][nbw][NG][2].
 *   real grids double[NG]; per-band reals double[NK][NB] (= Fortran (NB,NK)).
 *   Host pointers are caller-owned; the library copies in and out.  Functions
 *   with the `_device` suffix take device pointers and run asynchronously on the
 *   context's stream.
 *
 * Threading: one context per host thread; every call on a context is ordered
 * on that context's CUDA stream.  The library never aborts or exits.
 */
#ifndef MATTOHF_H
#define MATTOHF_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MATTOHF_OK 0
#define MATTOHF_ERR_ARG 1        /* invalid argument or configuration */
#define MATTOHF_ERR_CUDA 2       /* a CUDA runtime call failed */
#define MATTOHF_ERR_NONFINITE 3  /* non-finite state detected (e.g. unstable dt) */
#define MATTOHF_ERR_TIMEOUT 4    /* a bounded device wait gave up */
#define MATTOHF_ERR_NOTCONV 5    /* eigensolver / orthonormalisation did not converge */
#define MATTOHF_ERR_ALLOC 6      /* device allocation failed */
#define MATTOHF_ERR_STATE 7      /* call not valid in the context's current state */
#define MATTOHF_ERR_TOO_LARGE 8  /* problem does not fit a fixed-size scratch area */

/* options for mattohf_set_option */
#define MATTOHF_OPT_GRAPH 1        /* 1: replay RK4 steps from a captured CUDA graph (default 1) */
#define MATTOHF_OPT_FOCK_CHUNKS 2  /* pair chunks per Fock output column; 0 = automatic */
#define MATTOHF_OPT_KERNEL_TIMING 3 /* 1: bracket every Fock launch with CUDA events (no graph) */
#define MATTOHF_OPT_SYMMETRIC 4    /* 1: use the occupied-pair Hermitian symmetry when w == u (default 1) */
#define MATTOHF_OPT_FOCK_DF64 6   /* 1: symmetric exchange transforms in double-float (2 x FP32, 48-bit
                                      significand) arithmetic on the FP32 pipe; default 0 (FP64) */
#define MATTOHF_OPT_SYM_TILE 7     /* symmetric-exchange tile size (orbitals per CTA side); 0 = automatic */
#define MATTOHF_OPT_SMALL_STAGES 8 /* mattohf_rk4_run with one fused launch per RK4 stage (one CTA per
                                      column; for small problems): 0 off, 1 on, 2 automatic (default) */
#define MATTOHF_OPT_L2_FLUSH 5     /* >0: bytes written between RK4 steps of mattohf_rk4_run, which then
                                      reports the summed per-step device time (benchmarking) */
#define MATTOHF_OPT_SMALL_CTAS 9   /* CTAs per output column of the fused stages (the exchange pairs of a
                                      column are split over them); 0 = automatic (default) */

typedef struct mattohf_ctx mattohf_ctx;

/* Run configuration: the subset of src/Global_variables.f90 the hot path
 * reads (NG, NK, NB, NBocc, acell, functional) plus the atoms block of
 * src/mATTOHF.f90:229-240 (species charges/softening, ion positions in reduced
 * coordinates, 1-based species index). */
typedef struct mattohf_config {
  int NG;              /* grid points per cell: power of two, 16..512 */
  int NK;              /* k-points */
  int NB;              /* bands */
  int NBocc;           /* occupied bands, 1..NB */
  double acell;        /* lattice constant [bohr] */
  int functional_hf;   /* 1: 'HF' (Fock exchange on), 0: Hartree only */
  int device;          /* CUDA device ordinal */
  int nspecies;
  const double* Zeff;  /* [nspecies] */
  const double* alpha; /* [nspecies] */
  int nion;
  const double* Rion;  /* [nion] reduced positions */
  const int* Kion;     /* [nion] 1-based species index */
} mattohf_config;

/* Initialization (src/Initialization.f90:2-276) + Prep_periodic_ion_potential
 * (src/Prep_periodic_ion_potential.f90:2-31): grids, soft-Coulomb tables
 * k_vCk (src/Functions.f90:33-52), occupations, ion potential. */
int mattohf_create(const mattohf_config* cfg, mattohf_ctx** out);
int mattohf_destroy(mattohf_ctx* ctx);
const char* mattohf_last_error(const mattohf_ctx* ctx);
const char* mattohf_status_string(int status);
int mattohf_set_option(mattohf_ctx* ctx, int option, long long value);

/* Grids of src/Initialization.f90:93-112 and cell factors (I:46-49, I:62):
 * rx[NG], Gx[NG], kx[NK], cell[3] = {vcell, dvcell, bx}.  Any pointer may be NULL. */
int mattohf_get_grids(mattohf_ctx* ctx, double* rx, double* Gx, double* kx, double* cell);
/* Coulomb tables: vCG[NG] (I:143-146) and vCq[(2NK-1)][NG] = k_vCk(Gx+kx(kr)-kx(kc))
 * indexed by kr-kc+NK-1 (the distinct columns of vCGkk, I:130-137). */
int mattohf_get_coulomb(mattohf_ctx* ctx, double* vCG, double* vCq);
/* k_vCk (src/Functions.f90:33-52) of this cell at n arbitrary arguments q (the
 * debug table vk.out of src/Initialization.f90:149-155 uses q = Gx + kx). */
int mattohf_vck(mattohf_ctx* ctx, const double* q, int n, double* out);
/* Ion potential vion[NG]; set replaces it. */
int mattohf_get_vion(mattohf_ctx* ctx, double* vion);
int mattohf_set_vion(mattohf_ctx* ctx, const double* vion);

/* Device-resident orbitals ubk (the state of RT_calculation / GS_calculation). */
int mattohf_set_orbitals(mattohf_ctx* ctx, const double* ubk);
int mattohf_get_orbitals(mattohf_ctx* ctx, double* ubk);
/* Init_wf + quickrnd (src/mATTOHF.f90:159-196): the reference's Gaussian guess. */
int mattohf_init_wf(mattohf_ctx* ctx);
/* Gram_Schmidt (src/mATTOHF.f90:134-157) on the device orbitals. */
int mattohf_gram_schmidt(mattohf_ctx* ctx);

/* ubkwbk_hwbk (src/Functions.f90:187-209): hwbk = h[ubk](A) wbk.
 * ubk [NK][NB][NG], wbk/hwbk [NK][nbw][NG] complex128, host memory. */
int mattohf_hpsi(mattohf_ctx* ctx, const double* ubk, const double* wbk, int nbw, double A,
                 double* hwbk);
/* Same on device pointers, asynchronous on the context stream. */
int mattohf_hpsi_device(mattohf_ctx* ctx, const double* d_ubk, const double* d_wbk, int nbw,
                        double A, double* d_hwbk);
/* One rank's share of a run split over ranks by OUTPUT k-point.  The reference
 * splits the (k,k') pairs of ubkwbk_vFwbk over MPI ranks (NKK ranges,
 * src/Initialization.f90:64-76, loop src/Functions.f90:247) and all-reduces
 * the whole result (src/Functions.f90:258).  Here each rank owns whole output
 * k-points k0 .. k0+nkl-1: it needs the occupied orbitals of every k-point (one
 * all-gather by the caller) and no reduction of the result.
 * d_uocc: [NK][NBocc][NG] occupied orbitals of all k-points; d_wbk, d_hwbk:
 * [nkl][nbw][NG]; all device memory, asynchronous on the context stream.
 * term 0 = h[u] w (ubkwbk_hwbk rows), 1 = exchange only (ubkwbk_vFwbk rows),
 * 2 = kinetic only (ubk_tubk rows). */
int mattohf_hpsi_kslice_device(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl,
                               const double* d_wbk, int nbw, double A, int term, double* d_hwbk);
/* Observables of the k-slice [k0, k0+nkl) of a split run (d_ubk: [nkl][NB][NG]).
 * partial = {Ekin, Je, Ex} contributions of the slice (sum them over ranks);
 * scal = {Nele, Eion, EH} of the whole density (the same on every rank).
 * Etot = sum(Ekin) + Eion + EH + sum(Ex) (F:74-91, F:165-183, F:289-318).
 * Synchronous. */
int mattohf_observables_kslice_device(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl,
                                      const double* d_ubk, double A, double* partial, double* scal);
/* ubkwbk_vFwbk (src/Functions.f90:237-261): the Fock term alone. */
int mattohf_fock(mattohf_ctx* ctx, const double* ubk, const double* wbk, int nbw, double* vFwbk);
/* ubk_tubk (src/Functions.f90:212-234): the kinetic term alone. */
int mattohf_kinetic(mattohf_ctx* ctx, const double* wbk, int nbw, double A, double* tbk);
/* ubk_dns (F:55-71) and dns_vH (F:147-162). */
int mattohf_density(mattohf_ctx* ctx, const double* ubk, double* dns, double* vH);

/* ubk_Ecomps / ubk_Etot (F:74-91, F:265-286), ubk_Je (F:289-318) and
 * Nele = sum(dns)*dvcell (RT:43-45) of the device orbitals at field A.
 * Ecomps = {Ekin, Eion, EH, Exc}.  Any output pointer may be NULL. */
int mattohf_observables(mattohf_ctx* ctx, double A, double* Ecomps, double* Etot, double* Je,
                        double* Nele);

/* The reference's alternative propagators on the device orbitals (4th-order
 * Taylor expansion of exp(-i dt h), src/RT_calculation.f90:72-151):
 * variant 0 = RT_TE_ubk, 1 = RT_TEPC_ubk (predictor-corrector), 2 = RT_TEPC2_ubk. */
int mattohf_te_step(mattohf_ctx* ctx, int variant, double Aave, double dt);
/* RT_RK4_ubk (src/RT_calculation.f90:154-173): one RK4 step of the device
 * orbitals with stage fields 2*Aave-A, Aave, Aave, A. */
int mattohf_rk4_step(mattohf_ctx* ctx, double Aave, double A, double dt);
/* The RT_calculation loop body (RT:38-60) for nt steps: RK4 then Nele, Etot,
 * Jtot at A[it].  A, Aave: [nt] host arrays (Define_Afield, RT:175-244);
 * Etot, Je, Nele: [nt] host outputs (may be NULL).  Returns
 * MATTOHF_ERR_NONFINITE (with the first bad step in mattohf_last_error) if the
 * state overflows. */
int mattohf_rk4_run(mattohf_ctx* ctx, int nt, double dt, const double* A, const double* Aave,
                    double* Etot, double* Je, double* Nele);
/* Device time of the last mattohf_rk4_run in milliseconds (with
 * MATTOHF_OPT_L2_FLUSH: the sum of the per-step times, flushes excluded), and (with
 * MATTOHF_OPT_KERNEL_TIMING) the summed device time and launch count of the
 * Fock pair kernel inside it. */
int mattohf_last_run_timing(mattohf_ctx* ctx, double* run_ms, double* fock_ms, int* fock_launches);
/* Autotuner (no reference counterpart; the reference has no launch shapes).
 * Times, on the context's current orbitals, (1) the symmetric-exchange tile
 * size for one h[u]u exchange apply, (2) the CTAs per column of the fused
 * small-problem stages and (3) fused stages against the tiled step, with
 * `steps` graph-replayed mattohf_rk4_run steps (dt = 1e-4, A = 0) per
 * candidate, then keeps the fastest as MATTOHF_OPT_SYM_TILE,
 * MATTOHF_OPT_SMALL_CTAS and MATTOHF_OPT_SMALL_STAGES (0 or 1).  The orbitals
 * are restored.  out[3] (may be NULL): tile, CTAs per column (0 if the fused
 * stages do not apply), 1 if the fused stages won; us[3] (may be NULL):
 * microseconds of the exchange apply, of a tiled step and of a fused step. */
int mattohf_autotune(mattohf_ctx* ctx, int steps, int* out, double* us);

/* GS_calculation (src/GS_calculation.f90:2-121) SCF loop: per iteration
 * Gram_Schmidt, KS_ubk2_SVD (Krylov block of NB*ncg columns, GS:124-194),
 * Gram_Schmidt, Subspace_diag (GS:197-237), Etot, Je, epsbk, epserrorbk.
 * Etot_iter [nscf+1] (Etotscf(0:Nscf)), Je_iter [nscf], dnsdiff [nscf]
 * (sum|dnsscf(iter+1)-dnsscf(iter)|/NG), epsbk / epserrorbk [NK][NB] of the
 * last iteration.  Any output may be NULL. */
int mattohf_gs_run(mattohf_ctx* ctx, int nscf, int ncg, double* Etot_iter, double* Je_iter,
                   double* dnsdiff, double* epsbk, double* epserrorbk);
/* ubk_epsbk / ubk_epserrorbk (F:321-358) of the device orbitals, [NK][NB]. */
int mattohf_eps(mattohf_ctx* ctx, double* epsbk, double* epserrorbk);

int mattohf_synchronize(mattohf_ctx* ctx);

/* FourierTr / WindowFourierTr (src/RT_calculation.f90:246-351) on the GPU:
 * for omega_i = i/nomega*omegaM (i = 1..nomega), out[i-1][7] =
 * {omega, Re JF, Im JF, Re EF, Im EF, Re AF, Im AF} with
 * JF = sum_t e^{i omega t} filter (J - J0) dt, EF, AF likewise for E, A.
 * The caller supplies the filter (polynomial or envelope window). */
int mattohf_fourier(int device, int nt, const double* time, const double* J, double J0, const double* E,
                    const double* A, const double* filter, int nomega, double omegaM, double dt,
                    double* out);

/* ---- Adjoint gradient (no reference counterpart).  From the device orbitals
 * u0, runs nt RK4 steps with A[n] (Aave from A as in RT:227-230, stage
 * fields as in RT:165) and returns the objective
 *   objective 0: absorbed energy Etot(u_nt, A[nt-1]) - Etot(u0, 0)
 *   objective 1: final current Je(u_nt, A[nt-1])
 * with its gradient dLdA[nt] with respect to every field sample and
 * dLdvion[NG] with respect to the ion potential on the grid (either output
 * may be NULL).  Backward RK4 adjoint with checkpoints every ckpt_every
 * steps and recomputation between checkpoints; ckpt_every >= nt stores every
 * stage input in the forward pass (no recomputation); 0 picks that whenever it
 * fits in three quarters of the free device memory, else about sqrt(nt).
 * Requires NB == NBocc.  Leaves the orbitals at u_nt. */
int mattohf_adjoint(mattohf_ctx* ctx, int objective, int nt, double dt, const double* A, int ckpt_every,
                    double* L, double* dLdA, double* dLdvion);
/* Gradient with respect to the ion-potential parameters, by the chain rule
 * from a gradient on the grid (dLdvion[NG], e.g. from mattohf_adjoint) through
 * Prep_periodic_ion_potential (src/Prep_periodic_ion_potential.f90:10-20):
 * vion(x) = vraw(x) - max vraw, vraw(x) = -sum_ion sum_{icell=-4NK..4NK}
 * Zeff/sqrt((x - a Rion - a icell)^2 + alpha^2).  Outputs dLdZeff[nspecies],
 * dLdalpha[nspecies] (per species) and dLdRion[nion] (reduced positions).  The
 * max shift is differentiated at the first grid point attaining the maximum
 * (exact wherever the maximum is unique; one of the one-sided gradients at a
 * tie).  No reference counterpart (the reference has no gradients). */
int mattohf_ion_param_grad(mattohf_ctx* ctx, const double* dLdvion, double* dLdZeff, double* dLdalpha,
                           double* dLdRion);
/* Device times of the last mattohf_adjoint: the forward pass alone and the whole gradient. */
int mattohf_adjoint_timing(mattohf_ctx* ctx, double* forward_ms, double* total_ms);

/* ---- Batched ensemble (no reference counterpart: the reference runs one
 * system per process).  nruns independent runs with uneven NK, NB(=NBocc),
 * acell, ions and fields on one GPU, all with the same NG and device.  Each
 * member is an ordinary context (mattohf_batch_run) for set/get of orbitals,
 * Init_wf, Gram_Schmidt or a ground state; mattohf_batch_rk4_run then
 * advances all of them together, one graph replay per RK4 step.
 * A, Aave, Etot, Je, Nele are [nruns][nt]; dt is [nruns]. */
typedef struct mattohf_batch mattohf_batch;
int mattohf_batch_create(int nruns, const mattohf_config* cfgs, mattohf_batch** out);
int mattohf_batch_destroy(mattohf_batch* b);
const char* mattohf_batch_last_error(const mattohf_batch* b);
mattohf_ctx* mattohf_batch_run(mattohf_batch* b, int run);
int mattohf_batch_rk4_run(mattohf_batch* b, int nt, const double* dt, const double* A,
                          const double* Aave, double* Etot, double* Je, double* Nele);
int mattohf_batch_last_run_ms(mattohf_batch* b, double* ms);
/* Adjoint gradients of every member (mattohf_adjoint per run, no reference
 * counterpart): A [nruns][nt], dt [nruns]; L [nruns], dLdA [nruns][nt],
 * dLdvion [nruns][NG] (outputs may be NULL).  Members run one at a time, each
 * with all free device memory for its checkpoint segments (fitted to it when
 * ckpt_every <= 0) and released before the next member; a member's results are
 * those of mattohf_adjoint on it alone.  mattohf_batch_last_run_ms then gives
 * the summed device time; mattohf_adjoint_timing on a member its own.  Each
 * member is left at its final state. */
int mattohf_batch_adjoint(mattohf_batch* b, int objective, int nt, const double* dt, const double* A,
                          int ckpt_every, double* L, double* dLdA, double* dLdvion);
/* Batch options: MATTOHF_OPT_FOCK_DF64, and MATTOHF_OPT_SYM_TILE (the exchange
 * tile of every run's tile pairs; 0 = a CTA's teams, the default). */
int mattohf_batch_set_option(mattohf_batch* b, int option, long long value);
/* Batch autotuner: times every exchange tile (a CTA's teams, then halves down
 * to 1) over `steps` graph-replayed ensemble steps (dt = 1e-4, A = 0) on the
 * runs' current orbitals, restores them and keeps the fastest tile.  tile,
 * us (may be NULL): the tile kept and an ensemble step's time in microseconds. */
int mattohf_batch_autotune(mattohf_batch* b, int steps, int* tile, double* us);

/* Diagnostic (no reference counterpart): measured FP64 FMA throughput of
 * `device` in TFLOP/s (2 flops per DFMA), the roofline denominator of the
 * FP64-bound kernels. */
int mattohf_diag_fp64_peak(int device, double* tflops);
/* Measured FP64 tensor-core (DMMA, mma.sync m8n8k4 f64) throughput in TFLOP/s;
 * no reference counterpart.  Used to decide against a DFT-as-GEMM exchange. */
int mattohf_diag_dmma_peak(int device, double* tflops);

/* Exchange term vFwbk = ubkwbk_vFwbk(ubk, wbk) on caller-owned DEVICE buffers
 * without allocating any device memory.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc where they need the exchange
 * term (a host code with a fixed device arena, a shared memory pool that must
 * not grow, or a loop that must not take the allocator's locks).
 *   d_vCq   [(2NK-1)][NG] soft-Coulomb table as returned by mattohf_get_coulomb
 *   d_ubk   [NK][NB][NG] complex128;  d_wbk, d_vFwbk [NK][nbw][NG] complex128
 *   stream  cudaStream_t to enqueue on (NULL = default stream); asynchronous.
 * Scratch comes from one 16 MiB device array inside the library that every GPU
 * loading the library holds until exit.  The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress) and the device's
 * multiprocessor count with the device current, so make it before any stream
 * capture.  The cached address belongs to the CUDA runtime's primary context:
 * after cudaDeviceReset, or with another driver context current, do not call
 * this again in the same process.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  Returns
 * MATTOHF_ERR_TOO_LARGE when the twiddles, the table and one NK*nbw*NG
 * complex128 set of partial sums do not fit in 16 MiB. */
int mattohf_fock_noalloc(int NG, int NK, int NB, int NBocc, int nbw, const double* d_vCq,
                         const double* d_ubk, const double* d_wbk, double* d_vFwbk, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MATTOHF_H */
