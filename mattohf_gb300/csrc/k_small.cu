// Fused RK4 stage for small problems.
//
// For small grids and few orbitals every kernel of the general path is
// latency-bound, and a step of about 29 dependent launches costs more than the
// arithmetic.  Here one launch does a whole RK4 stage (src/RT_calculation.f90:
// 154-173).  Output column c = (k, b) is served by P CTAs (c, chunk) that form
// one thread-block cluster:
//   * the column's first CTA computes the density of the stage input
//     (F:55-71): its warps first sum |u|^2 over slices of the occupied
//     orbitals (in ik -> ib order within a slice, the uniform occupation
//     applied once); then the slices are added and the Hartree potential
//     formed (F:147-162).  At NG = 64 with several CTAs per column all eight
//     warps sum the slices and warps 0-1 then form vH as one 64-lane
//     transform pair (one point per lane); otherwise the kinetic warp skips
//     the slices and warp 7 forms vH.  A warp issues at most one FP64
//     instruction per ~64 cycles, so one warp alone would take about 4 us
//     for the sum;
//   * the CTAs apply the exchange of column c against their chunks of the
//     occupied orbitals (F:237-261, ordered pairs, no symmetry), one pair per
//     team, and each keeps its partial sum in shared memory.  With more than
//     one CTA per column the first CTA, which carries the density, the
//     kinetic and Hartree transforms and the Parseval sums, takes no pairs;
//     the others split them evenly on all eight warps;
//   * in the column's first CTA, warp 6 (at NG = 64 with several CTAs per
//     column, warps 6-7 as one 64-lane team) does the kinetic transform of
//     the column (F:212-234);
//   * each CTA pushes its partial into the shared memory of the CTAs that own
//     the grid points (distributed shared memory), the first CTA also vH and
//     T_A w; after a cluster barrier each CTA adds the P partials of its
//     points in chunk order and forms h w and the stage's RK4 update element
//     by element, into a buffer that is never the stage input, reading only
//     its own shared memory;
//   * stage 0 (or the closing pass, mode 4) also gathers the observables of
//     its input, i.e. of the previous step (F:74-119, F:165-183, F:289-318):
//     Ekin and Je per column by Parseval on a forward transform of the column
//     at the previous step's field (warp 3 of the first CTA, idle when a
//     column has several CTAs, else warp 6 with its kinetic transform),
//     <u|F u> from the CTAs' shares (each CTA's partial against w over all
//     points, pushed to the first CTA before the cluster barrier), and column
//     0's copy of the density and vH.  Stage 1 then forms Etot, Je, Nele on
//     an idle warp of column 0's
//     first CTA, so no stage-0 CTA waits for a global ticket; the closing pass
//     still has the last column to finish (global ticket) write them.
//     The step counter has a shadow: stage 0 copies the counter to it and
//     stage 3 reads the shadow (for its field) while block 0 writes the next
//     step's index to the counter, so no stage waits for a global ticket to
//     advance it.
// A ticket is an atomic counter taken after a fence; the CTA that draws the
// last number does the follow-up work.  No CTA waits on another column.
#include <cooperative_groups.h>

#include "fft.cuh"
#include "internal.h"

namespace mattohf {

constexpr int kSmallThreads = 256;
constexpr int kSmallWarps = kSmallThreads / 32;
// the latency FFT plans where few transforms run at a time and a warp's chain
// counts (NG <= 64); at NG = 128 the stage is bound by each SM's FP64 rate and
// the 16-lane plan balances better over the CTA's warps
template <int N>
constexpr int kSmallPlan = N <= 64 ? 1 : 0;

__device__ __forceinline__ double small_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int N>
struct SmallLayout {
  static constexpr int PW = Team<N, kSmallPlan<N>>::PER_WARP;
  static constexpr int NTEAM = kSmallWarps * PW;
  // pair teams of a single CTA (warps 0..5; warp 6 does the kinetic
  // transform and warp 7 the density and Hartree potential), the autotuner's
  // lower bound on the CTAs per column
  static constexpr int PAIR_TEAMS = (kSmallWarps - 2) * PW;
  // tw[N], bufs[NTEAM][N], F[N] (double2); rho[N], vh[N] (double); K[N] (double2);
  // then what the cluster's CTAs push to this one for its share of the grid
  // points: the P exchange partials (at most 2N + 2 kSmallMaxCtas doubles),
  // vH and T_A w (N and 2N doubles)
  static constexpr int RECV_F = 2 * N + 2 * kSmallMaxCtas;
  static constexpr size_t bytes = sizeof(double2) * (size_t)N * (3 + NTEAM) + sizeof(double) * 2 * (size_t)N +
                                  sizeof(double) * ((size_t)RECV_F + 3 * (size_t)N);
  // the adjoint's variant also stages its stage-store copy (N double2)
  static constexpr size_t bytes_adj = bytes + sizeof(double2) * (size_t)N;
};

// The global last CTA of an observable stage: the observables of the stage
// input (mode 0 with a previous step, mode 4) from the column buffer and this
// CTA's own density.  Run by one warp.
__device__ void small_finalize(const SmallStageArgs& a, const double* rho_s, const double* vh_s, int N) {
  const int lane = threadIdx.x & 31;
  const int idx = *a.it - 1;
  if (idx < 0) return;
  const int ncol = a.nk * a.nb;
  double ekin = 0.0, jre = 0.0, exr = 0.0;
  for (int c = lane; c < ncol; c += 32) {
    const int ib = c % a.nb;
    const double occ = ib < a.nbocc ? a.occ : 0.0;
    const double* cb = a.colbuf + (size_t)c * 4;
    ekin += occ * __ldcg(cb) * a.dvcell;
    jre += occ * __ldcg(cb + 1);
    if (ib < a.nbocc) exr += occ * __ldcg(cb + 2) * a.dvcell;
  }
  double sn = 0.0, si = 0.0, sh = 0.0;
  for (int ig = lane; ig < N; ig += 32) {
    sn += rho_s[ig];
    si += a.vion[ig] * rho_s[ig];
    sh += vh_s[ig] * rho_s[ig];
  }
  ekin = small_warp_sum(ekin);
  jre = small_warp_sum(jre);
  exr = small_warp_sum(exr);
  sn = small_warp_sum(sn);
  si = small_warp_sum(si);
  sh = small_warp_sum(sh);
  if (lane != 0) return;
  const double Nele = sn * a.dvcell, Eion = si * a.dvcell, EH = 0.5 * sh * a.dvcell;
  const double Ex = a.hf ? 0.5 * exr : 0.0;
  const double Etot = (ekin + Eion + EH) + Ex;
  const double Je = -(jre * a.dvcell / a.vcell);
  if (a.series_E) a.series_E[idx] = Etot;
  if (a.series_J) a.series_J[idx] = Je;
  if (a.series_N) a.series_N[idx] = Nele;
  if (a.out_obs) {
    a.out_obs[0] = Etot;
    a.out_obs[1] = ekin;
    a.out_obs[2] = Eion;
    a.out_obs[3] = EH;
    a.out_obs[4] = Ex;
    a.out_obs[5] = Je;
    a.out_obs[6] = Nele;
  }
  if (!(isfinite(Etot) && isfinite(Je) && isfinite(Nele)) && a.nonfinite) *a.nonfinite = 1;
}

// ADJ: the variant for the adjoint's forward and recompute passes, which also
// copies the stage input to the stage store or a checkpoint; the plain
// forward's variant carries none of that code or shared memory.
template <int N, bool ADJ>
__global__ void __launch_bounds__(kSmallThreads) k_small_stage(SmallStageArgs a) {
  using TM = Team<N, kSmallPlan<N>>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NTEAM = SmallLayout<N>::NTEAM;
  namespace cg = cooperative_groups;
  extern __shared__ double2 sm2[];
  double2* tw_s = sm2;                     // N
  double2* bufs = tw_s + N;                // NTEAM * N
  double2* F_s = bufs + NTEAM * N;         // N: with rho_s and vh_s, the density slices
  double* rho_s = reinterpret_cast<double*>(F_s + N);
  double* vh_s = rho_s + N;
  double2* K_s = reinterpret_cast<double2*>(vh_s + N);  // N: T_A w (the column's first CTA)
  double* recvF = reinterpret_cast<double*>(K_s + N);   // [P][2 per]: the partials of this CTA's points
  double* recvV = recvF + SmallLayout<N>::RECV_F;       // [per]: vH at this CTA's points
  double* recvK = recvV + N;                            // [2 per]: T_A w at this CTA's points
  double2* st_s = reinterpret_cast<double2*>(recvK + 2 * N);  // [per]: staged stage-store copy (ADJ)
  __shared__ int last_s;
  __shared__ double red_s[2][kSmallWarps];
  __shared__ double ex_s[kSmallMaxCtas][2];  // the first CTA: every CTA's share of <w|F>
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, team = warp * PW + lane / T;
  double2* buf = bufs + team * N;
  const int ncols = a.nk * a.nb;
  const int c = blockIdx.x / a.P;          // output column (k, b)
  const int chunk = blockIdx.x % a.P;      // rank in the column's cluster
  const int kr = c / a.nb, ib = c % a.nb;
  const int M = a.nk * a.nbocc;
  // This CTA's exchange pairs.  With more than one CTA per column the first
  // CTA takes none: its warps carry the density, the kinetic and Hartree
  // transforms and the Parseval sums, and the other CTAs split the pairs
  // evenly on all eight warps.  A single CTA runs them on warps 0-5.
  const int p0 = (a.P == 1 || chunk == 0) ? 0 : (M * (chunk - 1)) / (a.P - 1);
  const int p1 = a.P == 1 ? M : chunk == 0 ? 0 : (M * chunk) / (a.P - 1);
  const int workers = a.P == 1 ? kSmallWarps - 2 : chunk == 0 ? 0 : kSmallWarps;  // pair warps 0 .. workers-1
  const int worker_teams = workers * PW;
  const bool occupied = ib < a.nbocc;
  const bool obs = a.mode == 0 || a.mode == 4;
  const double2* wcol = a.u + (size_t)c * N;

  for (int i = tid; i < N; i += kSmallThreads) tw_s[i] = a.tw[i];
  __syncthreads();
  // Launched as a programmatic dependent of the previous stage: everything
  // above reads only constant tables.  Wait for the previous grid to complete
  // (and its writes to be visible) before touching the state or the scratch,
  // then let the next stage's grid start its own prologue.  Both are no-ops
  // without a programmatic dependency.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;");
  // every CTA of the cluster has started once this barrier phase completes;
  // it is waited for only before the first store to another CTA's memory
  asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory");
  if (a.it_out && blockIdx.x == 0 && tid == 0) *a.it_out = *a.it + a.it_inc;
  // the adjoint's passes: this CTA's points of the stage input, staged in
  // shared memory by an asynchronous copy now and written to the stage store
  // (recompute) or to a checkpoint (stage 0 of the forward pass) once the
  // first phase is done (no registers held, no latency exposed)
  auto ckpt_step = [&]() {
    if (!a.ckpt || a.mode != 0) return false;
    const int t = *a.it;
    return t == 0 || (t + a.ckpt_phase) % a.ckpt_every == 0;
  };
  if (ADJ && (a.store || ckpt_step())) {
    const int per_pts = (N + a.P - 1) / a.P, q_st = chunk * per_pts + tid;
    if (tid < per_pts && q_st < N) {
      const unsigned dst = (unsigned)__cvta_generic_to_shared(st_s + tid);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(wcol + q_st) : "memory");
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
  }
  // density, first part: sum of |u|^2 over slice j of the occupied orbitals at
  // point ig, one (j, ig) per thread and round.  F_s, rho_s and vh_s (4N
  // contiguous doubles) are free during the first phase and hold the slices.
  // Only the Hartree chain waits for them.  A single CTA, and the first CTA at
  // NG = 64 with several CTAs per column, sums them on all its threads;
  // otherwise the first CTA's kinetic warp (6) starts its transforms at once
  // and the other seven warps sum the slices.
  constexpr int NSUB = (kSmallThreads / N) < 4 ? (kSmallThreads / N) : 4;
  double* dslice = reinterpret_cast<double*>(F_s);  // [NSUB][N]
  auto density_slices = [&](int t0, int nthreads, int nsub) {
    const int per = (M + nsub - 1) / nsub;
    for (int slot = t0; slot < nsub * N; slot += nthreads) {
      const int ig = slot % N, j = slot / N;
      const int q1 = min(M, (j + 1) * per);
      double s = 0.0;
#pragma unroll 4
      for (int p = j * per; p < q1; ++p) {
        const int ik = p / a.nbocc, b = p % a.nbocc;
        const double2 z = a.u[((size_t)ik * a.nb + b) * N + ig];
        s = fma(z.y, z.y, fma(z.x, z.x, s));
      }
      dslice[j * N + ig] = s;
    }
  };
  // At NG = 64 with several CTAs per column the first CTA's Hartree (warps 0
  // and 1) and kinetic (warps 6 and 7) chains each run on two warps, one
  // point per lane (fft_lane), after all eight warps have summed the density
  // slices (the kinetic chain could start at once, but its FP64 issue would
  // slow the density down, and the Hartree chain waits for that).
  const bool two_warp = N == 64 && a.P > 1 && a.mode != 4;
  if (chunk == 0) {
    if (a.P == 1 || two_warp) {
      density_slices(tid, kSmallThreads, NSUB);
      __syncthreads();
    } else if (warp != kSmallWarps - 2) {
      const int dw = warp < kSmallWarps - 2 ? warp : warp - 1;
      density_slices(dw * 32 + lane, kSmallThreads - 32, NSUB);
      asm volatile("bar.sync 1, %0;" ::"n"(kSmallThreads - 32) : "memory");
    }
  }
  if constexpr (N == 64) {
    if (two_warp && chunk == 0 && warp >= kSmallWarps - 2) {
      // kinetic term T_A w of column c at the stage field (F:212-234), on
      // warps 6 and 7, one point per lane
      const int L = (warp - (kSmallWarps - 2)) * 32 + lane;
      const int rb = (int)(__brev((unsigned)L) >> 26);
      double2* kb = bufs + (size_t)((kSmallWarps - 2) * PW) * N;
      double2 x = fft_lane<N, -1>(wcol[rb], L, tw_s, kb, 3);
      const double A = afield_value(a.af);
      const double kAx = a.kx[kr] + A, kA2 = kAx * kAx;
      const double G = a.Gx[L];
      const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
      kb[L] = make_double2(m * x.x / (double)N, m * x.y / (double)N);
      asm volatile("bar.sync 3, %0;" ::"n"(N) : "memory");
      x = kb[rb];
      asm volatile("bar.sync 3, %0;" ::"n"(N) : "memory");
      K_s[L] = fft_lane<N, +1>(x, L, tw_s, kb, 3);
    } else if (two_warp && chunk == 0 && warp < 2) {
      // density (slices in order; lane L sums point bitrev(L), so rho_s's
      // entry, slice 2's, is read by this lane before it is overwritten, and
      // vh_s's, slice 3's, before the barriers inside fft_lane) and
      // vH (F:147-162) on warps 0 and 1, one point per lane
      const int L = warp * 32 + lane;
      const int rb = (int)(__brev((unsigned)L) >> 26);
      double s = dslice[rb];
#pragma unroll
      for (int j = 1; j < NSUB; ++j) s += dslice[j * N + rb];
      const double rho = a.occ * s;
      rho_s[rb] = rho;
      double2* hb = bufs;
      double2 x = fft_lane<N, -1>(make_double2(rho, 0.0), L, tw_s, hb, 2);
      const double g = a.vCG[L];
      hb[L] = make_double2(g * x.x, g * x.y);
      asm volatile("bar.sync 2, %0;" ::"n"(N) : "memory");
      x = hb[rb];
      asm volatile("bar.sync 2, %0;" ::"n"(N) : "memory");
      x = fft_lane<N, +1>(x, L, tw_s, hb, 2);
      const double vh = x.x / (double)N;
      vh_s[L] = vh;  // slice 3's entry L, read by lane bitrev(L) before the barriers above
      if (a.mode == 0 && c == 0) {
        a.obs_dens[rb] = rho;
        a.obs_dens[N + L] = vh;
      }
    }
  }
  if (two_warp && chunk == 0 && (warp < 2 || warp >= kSmallWarps - 2)) {
    // done above
  } else if (chunk == 0 && warp == kSmallWarps - 1) {
    {
      // density (slices in order; with 3 or more slices rho_s[ig] is slice
      // 2's entry for ig, read by this lane before it is overwritten) and vH
      for (int ig = lane; ig < N; ig += 32) {
        double s = dslice[ig];
#pragma unroll
        for (int j = 1; j < NSUB; ++j) s += dslice[j * N + ig];
        rho_s[ig] = a.occ * s;
      }
      __syncwarp();
      double2 x[E];
#pragma unroll
      for (int e = 0; e < E; ++e) x[e] = make_double2(rho_s[TM::pos(tl, e)], 0.0);
      fft_team<N, -1, kSmallPlan<N>>(x, buf, tw_s, tl);
      fft_team_in<N, +1, kSmallPlan<N>>(InScaled<N, kSmallPlan<N>>{x, a.vCG, tl}, x, buf, tw_s, tl);
      if (lane < T) {
#pragma unroll
        for (int e = 0; e < E; ++e) vh_s[TM::pos(tl, e)] = x[e].x / (double)N;
      }
      if (a.mode == 0 && c == 0) {
        // the density and vH of this stage input (the previous step's state)
        // for its observables, which stage 1 completes off this critical path
        __syncwarp();
        for (int ig = lane; ig < N; ig += 32) {
          a.obs_dens[ig] = rho_s[ig];
          a.obs_dens[N + ig] = vh_s[ig];
        }
      }
    }
  } else if (chunk == 0 && warp == kSmallWarps - 2) {
    {
      // kinetic term T_A w of column c at the stage field (F:212-234) and, for
      // stage 0 and the closing pass, Ekin and Je of the input column at the
      // previous step's field by Parseval on the same forward transform
      double2 x[E];
#pragma unroll
      for (int e = 0; e < E; ++e) x[e] = wcol[TM::pos(tl, e)];
      fft_team<N, -1, kSmallPlan<N>>(x, buf, tw_s, tl);
      if (obs && !(a.mode == 0 && a.P > 1)) {
        const int itn = *a.it;
        const double Ao = (itn >= 1 && a.Aobs) ? a.Aobs[itn - 1] : 0.0;
        const double kAx = a.kx[kr] + Ao, kA2 = kAx * kAx;
        double ek = 0.0, je = 0.0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const double G = a.Gx[TM::pos(tl, e)];
          const double m2 = x[e].x * x[e].x + x[e].y * x[e].y;
          ek += 0.5 * (G * G + 2.0 * G * kAx + kA2) * m2;
          je += (G + a.kx[kr] + Ao) * m2;
        }
        ek = team_sum<T>(ek) / (double)N;
        je = team_sum<T>(je) / (double)N;
        if (lane == 0) {
          a.colbuf[(size_t)c * 4] = ek;
          a.colbuf[(size_t)c * 4 + 1] = je;
        }
      }
      if (a.mode != 4) {
        const double A = afield_value(a.af);
        const double kAx = a.kx[kr] + A, kA2 = kAx * kAx;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const double G = a.Gx[TM::pos(tl, e)];
          const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
          x[e] = make_double2(m * x[e].x / (double)N, m * x[e].y / (double)N);
        }
        fft_team<N, +1, kSmallPlan<N>>(x, buf, tw_s, tl);
        if (lane < T) {
#pragma unroll
          for (int e = 0; e < E; ++e) K_s[TM::pos(tl, e)] = x[e];
        }
      }
    }
  } else if (chunk == 0 && a.P > 1 && warp == 3 && a.mode == 0) {
    // Ekin and Je of the input column at the previous step's field (Parseval
    // on its forward transform), beside warp 6's kinetic transforms
    double2 x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = wcol[TM::pos(tl, e)];
    fft_team<N, -1, kSmallPlan<N>>(x, buf, tw_s, tl);
    const int itn = *a.it;
    const double Ao = (itn >= 1 && a.Aobs) ? a.Aobs[itn - 1] : 0.0;
    const double kAx = a.kx[kr] + Ao, kA2 = kAx * kAx;
    double ek = 0.0, je = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const double G = a.Gx[TM::pos(tl, e)];
      const double m2 = x[e].x * x[e].x + x[e].y * x[e].y;
      ek += 0.5 * (G * G + 2.0 * G * kAx + kA2) * m2;
      je += (G + a.kx[kr] + Ao) * m2;
    }
    ek = team_sum<T>(ek) / (double)N;
    je = team_sum<T>(je) / (double)N;
    if (lane == 0) {
      a.colbuf[(size_t)c * 4] = ek;
      a.colbuf[(size_t)c * 4 + 1] = je;
    }
  } else if (warp < workers && a.hf && (a.mode != 4 || occupied)) {
    // this CTA's exchange pairs of column c, one pair per team per round
    double2 acc[E];
#pragma unroll
    for (int e = 0; e < E; ++e) acc[e] = make_double2(0.0, 0.0);
    // warp-uniform trip count: every team of a warp runs the same rounds
    for (int base = p0 + warp * PW; base < p1; base += worker_teams) {
      const int p = base + lane / T;
      const bool valid = p < p1;
      const int pp = valid ? p : p0;
      const int kc = pp / a.nbocc, bc = pp % a.nbocc;
      const double2* ucol = a.u + ((size_t)kc * a.nb + bc) * N;
      const double* kern = a.kern + (size_t)(kr - kc + a.nk - 1) * N;
      // the pair's kernel row, loaded while the forward transform runs
      double kf[E];
#pragma unroll
      for (int e = 0; e < E; ++e) kf[e] = __ldg(kern + TM::pos(tl, e));
      double2 x[E];
      fft_team_in<N, -1, kSmallPlan<N>>(InConjProduct<N, kSmallPlan<N>>{wcol, ucol, tl}, x, buf, tw_s, tl);
      fft_team_in<N, +1, kSmallPlan<N>>(InScaledRegs{x, kf}, x, buf, tw_s, tl);
      if (valid) {
#pragma unroll
        for (int e = 0; e < E; ++e) acc[e] = cfma(x[e], ucol[TM::pos(tl, e)], acc[e]);
      }
    }
    __syncwarp();
#pragma unroll
    for (int e = 0; e < E; ++e) buf[TM::pos(tl, e)] = acc[e];
  }
  // stage 1: the observables of the previous step's state, from the column
  // buffer and the density stage 0 left (stage 0 completed before this grid
  // passed griddepcontrol.wait), on an idle warp of column 0's first CTA
  if (a.mode == 1 && c == 0 && chunk == 0 && warp == (a.P > 1 ? 2 : kSmallWarps - 1))
    small_finalize(a, a.obs_dens, a.obs_dens + N, N);
  // The epilogue runs one real component per lane: lane slot idx = 2 e + cc
  // takes component cc of h = T_A w + v w + F at this CTA's element e and
  // writes the other component, dd = 1 - cc, of k = -i h and of the stage
  // output (k.x = h.y, k.y = -h.x).  A warp issues at most one FP64
  // instruction per ~64 cycles, so halving each lane's chain halves the
  // epilogue's time.  These are its inputs that no other CTA writes.
  constexpr int EPI = (2 * N + kSmallThreads - 1) / kSmallThreads;  // lane slots per thread
  const int per = (N + a.P - 1) / a.P;
  const double cdt = a.mode == 2 ? a.dt : 0.5 * a.dt;
  double wc[EPI], vi[EPI], ud[EPI], ks[EPI];
  // stage 0 and the closing pass: the w factors of this thread's components
  // in the partial sum below (component i = 2 q + cc of every point)
  double wt[EPI][2];
#pragma unroll
  for (int r = 0; r < EPI; ++r) {
    wt[r][0] = wt[r][1] = 0.0;
    const int i = tid + r * kSmallThreads;
    if (obs && i < 2 * N) {
      const double* w2 = reinterpret_cast<const double*>(wcol + (i >> 1));
      wt[r][0] = w2[i & 1];
      wt[r][1] = (i & 1) ? w2[0] : -w2[1];
    }
  }
#pragma unroll
  for (int r = 0; r < EPI; ++r) {
    wc[r] = vi[r] = ud[r] = ks[r] = 0.0;
    const int idx = tid + r * kSmallThreads, e = idx >> 1, cc = idx & 1, dd = 1 - cc;
    const int q = chunk * per + e;
    if (e < per && q < N) {
      const double* w2 = reinterpret_cast<const double*>(wcol + q);
      wc[r] = w2[cc];
      if (a.mode != 4) {
        const size_t od = 2 * ((size_t)c * N + q) + dd;
        vi[r] = a.vion[q];
        ud[r] = reinterpret_cast<const double*>(a.u0)[od];
        if (a.mode == 3) {
          // k0 + 2 k1 + 2 k2, formed before the barrier (the order of
          // ubk + (k1 + 2 k2 + 2 k3 + k4) * dt / 6, RT:165-170, is kept)
          const double k0 = reinterpret_cast<const double*>(a.kbuf[0])[od];
          const double k1 = reinterpret_cast<const double*>(a.kbuf[1])[od];
          const double k2 = reinterpret_cast<const double*>(a.kbuf[2])[od];
          ks[r] = fma(2.0, k2, fma(2.0, k1, k0));
        }
      }
    }
  }
  __syncthreads();
  if (ADJ && (a.store || ckpt_step()) && tid < per && chunk * per + tid < N) {
    asm volatile("cp.async.wait_all;" ::: "memory");
    const size_t elems = (size_t)ncols * N, o = (size_t)c * N + chunk * per + tid;
    const int t = *a.it;
    if (a.store) a.store[((size_t)(t - *a.seg0) * 4 + a.store_slot) * elems + o] = st_s[tid];
    if (ckpt_step()) a.ckpt[(size_t)((t + a.ckpt_phase) / a.ckpt_every) * elems + o] = st_s[tid];
  }
  // This CTA's partial (pair teams in order; a team past the CTA's pair count
  // holds none), one real component per thread, pushed into the shared memory
  // of the CTA that owns the point (distributed shared memory); the first CTA
  // also pushes vH and T_A w.  After the cluster barrier every CTA finds the
  // P partials of its points in its own shared memory and does h w and the
  // RK4 update for its share of the grid, with no remote reads.
  cg::cluster_group cluster = cg::this_cluster();
  asm volatile("barrier.cluster.wait;" ::: "memory");
  const int act = (a.hf && (a.mode != 4 || occupied)) ? min(worker_teams, p1 - p0) : 0;
  {
    const double* bd = reinterpret_cast<const double*>(bufs);
    // stage 0 and the closing pass: this CTA's share of <w|F> = sum over all
    // points of conj(w) F_chunk, one real component per thread (Re gets
    // w_cc F_cc, Im gets sg w_dd F_cc with sg = +1 for cc = 1, -1 for cc = 0)
    double exr = 0.0, exi = 0.0;
#pragma unroll
    for (int r = 0; r < EPI; ++r) {
      const int i = tid + r * kSmallThreads;
      if (i >= 2 * N) continue;
      double f = 0.0;
      if (act > 0) f = bd[i];
      for (int t2 = 1; t2 < act; ++t2) f += bd[(size_t)t2 * 2 * N + i];
      const int q = i >> 1, cc = i & 1, owner = q / per, e = q - owner * per;
      cluster.map_shared_rank(recvF, owner)[chunk * 2 * per + 2 * e + cc] = f;
      if (obs) {
        exr = fma(wt[r][0], f, exr);
        exi = fma(wt[r][1], f, exi);
      }
    }
    if (obs) {
      // warp tree, then warps in order, pushed to the first CTA's slot
      exr = small_warp_sum(exr);
      exi = small_warp_sum(exi);
      if (lane == 0) {
        red_s[0][warp] = exr;
        red_s[1][warp] = exi;
      }
      __syncthreads();
      if (tid == 0) {
        double sr = red_s[0][0], si = red_s[1][0];
        for (int w2 = 1; w2 < kSmallWarps; ++w2) {
          sr += red_s[0][w2];
          si += red_s[1][w2];
        }
        double* dst = cluster.map_shared_rank(&ex_s[0][0], 0) + 2 * chunk;
        dst[0] = sr;
        dst[1] = si;
      }
    }
    if (chunk == 0 && a.mode != 4) {
      for (int q = tid; q < N; q += kSmallThreads) {
        const int owner = q / per, e = q - owner * per;
        cluster.map_shared_rank(recvV, owner)[e] = vh_s[q];
        double* rk = cluster.map_shared_rank(recvK, owner);
        rk[2 * e] = K_s[q].x;
        rk[2 * e + 1] = K_s[q].y;
      }
    }
  }
  cluster.sync();
  if (obs && chunk == 0 && tid == 0 && occupied) {
    double sr = ex_s[0][0], si = ex_s[0][1];
    for (int r = 1; r < a.P; ++r) {
      sr += ex_s[r][0];
      si += ex_s[r][1];
    }
    a.colbuf[(size_t)c * 4 + 2] = sr;
    a.colbuf[(size_t)c * 4 + 3] = si;
  }
  bool bad = false;
  // F (the P partials in chunk order) and h, from this CTA's shared memory
  double hr[EPI];
#pragma unroll
  for (int r = 0; r < EPI; ++r) {
    hr[r] = 0.0;
    const int idx = tid + r * kSmallThreads, e = idx >> 1, cc = idx & 1;
    const int q = chunk * per + e;
    if (!(e < per && q < N)) continue;
    double f = recvF[2 * e + cc];
#pragma unroll
    for (int rr = 1; rr < kSmallMaxCtas; ++rr)
      if (rr < a.P) f += recvF[rr * 2 * per + 2 * e + cc];
    if (a.mode != 4) hr[r] = fma(recvV[e] + vi[r], wc[r], recvK[2 * e + cc]) + f;
  }
#pragma unroll
  for (int r = 0; r < EPI; ++r) {
    const int idx = tid + r * kSmallThreads, e = idx >> 1, cc = idx & 1, dd = 1 - cc;
    const int q = chunk * per + e;
    if (!(e < per && q < N)) continue;
    const double scdt = cc ? cdt : -cdt;  // k_dd = sg h_cc with sg = +1 (cc = 1) or -1 (cc = 0)
    if (a.mode != 4) {
      const double h = hr[r];
      const size_t od = 2 * ((size_t)c * N + q) + dd;
      double nx;
      if (a.mode < 3) {
        nx = fma(scdt, h, ud[r]);
        reinterpret_cast<double*>(a.kbuf[a.mode])[od] = cc ? h : -h;
        reinterpret_cast<double*>(a.out)[od] = nx;
      } else {
        const double kd = cc ? h : -h;
        nx = ud[r] + (ks[r] + kd) * a.dt / 6.0;
        reinterpret_cast<double*>(a.u0)[od] = nx;  // this component only, read above by this thread
      }
      bad = bad || !isfinite(nx);
    }
  }
  if (bad && a.nonfinite) *a.nonfinite = 1;
  // No CTA touches another's shared memory after the cluster barrier, so the
  // stage is done; in the closing pass the last column to finish
  // finalizes (nothing waits on another column)
  if (a.mode != 4 || chunk != 0) return;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned t = atomicAdd(a.ticket, 1u);
    last_s = (t == (unsigned)ncols - 1) ? 1 : 0;
  }
  __syncthreads();
  if (last_s && warp == 0) {
    __threadfence();
    small_finalize(a, rho_s, vh_s, N);
    if (lane == 0) *a.ticket = 0u;
  }
}

template <int N, bool ADJ>
static cudaError_t small_impl(const SmallStageArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nk * a.nb * a.P);
  cfg.blockDim = dim3(kSmallThreads);
  cfg.dynamicSmemBytes = ADJ ? SmallLayout<N>::bytes_adj : SmallLayout<N>::bytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;  // one cluster per output column
  attr[1].val.clusterDim.x = a.P;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_small_stage<N, ADJ>, a);
}

template <int N>
static cudaError_t small_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_small_stage<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)SmallLayout<N>::bytes_adj);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_small_stage<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)SmallLayout<N>::bytes);
}

bool small_stage_supported(int NG) { return NG >= 16 && NG <= 256 && (NG & (NG - 1)) == 0; }

int small_pair_teams(int NG) {
  switch (NG) {
    case 16: return SmallLayout<16>::PAIR_TEAMS;
    case 32: return SmallLayout<32>::PAIR_TEAMS;
    case 64: return SmallLayout<64>::PAIR_TEAMS;
    case 128: return SmallLayout<128>::PAIR_TEAMS;
    case 256: return SmallLayout<256>::PAIR_TEAMS;
    default: return 0;
  }
}

cudaError_t launch_small_stage(int NG, const SmallStageArgs& a, cudaStream_t s) {
  if (a.P < 1 || a.P > kSmallMaxCtas) return cudaErrorInvalidValue;
  const bool adj = a.store != nullptr || a.ckpt != nullptr;
  switch (NG) {
    case 16: return adj ? small_impl<16, true>(a, s) : small_impl<16, false>(a, s);
    case 32: return adj ? small_impl<32, true>(a, s) : small_impl<32, false>(a, s);
    case 64: return adj ? small_impl<64, true>(a, s) : small_impl<64, false>(a, s);
    case 128: return adj ? small_impl<128, true>(a, s) : small_impl<128, false>(a, s);
    case 256: return adj ? small_impl<256, true>(a, s) : small_impl<256, false>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t configure_small_kernels() {
  cudaError_t e;
  if ((e = small_configure<16>()) != cudaSuccess) return e;
  if ((e = small_configure<32>()) != cudaSuccess) return e;
  if ((e = small_configure<64>()) != cudaSuccess) return e;
  if ((e = small_configure<128>()) != cudaSuccess) return e;
  return small_configure<256>();
}

}  // namespace mattohf
