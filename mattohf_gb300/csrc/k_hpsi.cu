// Hamiltonian-apply kernels: density + Hartree, Fock pair transforms, and the
// per-column combine (kinetic + local + exchange + RK4 / observable epilogues).
//
// Reference: src/Functions.f90 ubkwbk_hwbk (F:187-209), ubk_tubk (F:212-234),
// ubk_dns (F:55-71), dns_vH (F:147-162), ubkwbk_vFwbk (F:237-261), ubk_Ekin
// (F:94-119), ubk_Ex (F:165-183), ubk_Je (F:289-318); RK4 stages from
// src/RT_calculation.f90:154-173.
#include "fft.cuh"
#include "internal.h"

namespace mattohf {

// Fixed xor-shuffle tree over the 32 lanes of a warp (deterministic order).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Density (F:55-71) and Hartree potential (F:147-162), one CTA.
// ---------------------------------------------------------------------------
// Stage 1: partial densities over a contiguous range of columns (one CTA per
// chunk, thread per grid point); the FP64 work is spread over many SMs.
__device__ __forceinline__ void dens_partial_body(const DensArgs& a, int N, int chunk) {
  const int ncol = a.nk * a.u.nb;
  const int per = (ncol + kDensChunks - 1) / kDensChunks;
  const int c0 = chunk * per, c1 = min(ncol, c0 + per);
  for (int ig = threadIdx.x; ig < N; ig += blockDim.x) {
    double s = 0.0;
    if (a.mu == nullptr) {
      for (int c = c0; c < c1; ++c) {   // ik outer, ib inner within the chunk (reference order)
        const int ik = c / a.u.nb, ib = c % a.u.nb;
        const double occ = ib < a.nbocc ? a.occ : 0.0;
        const double2 z = a.u.p[(size_t)ik * a.u.kstride + (size_t)ib * N + ig];
        s += fma(occ * z.x, z.x, (occ * z.y) * z.y);
      }
    } else {
      for (int c = c0; c < c1; ++c) {   // adjoint source: Im(conj(mu) u)
        const int ik = c / a.u.nb, ib = c % a.u.nb;
        const size_t o = (size_t)ik * a.u.kstride + (size_t)ib * N + ig;
        const double2 z = a.u.p[o], m = a.mu[o];
        s += fma(m.x, z.y, -(m.y * z.x));
      }
    }
    a.part[(size_t)chunk * N + ig] = s;
  }
}

__global__ void __launch_bounds__(256) k_dens_partial(DensArgs a, int N) { dens_partial_body(a, N, blockIdx.x); }

__global__ void __launch_bounds__(256) k_dens_partial_batch(const DensArgs* __restrict__ args, int N) {
  dens_partial_body(args[blockIdx.y], N, blockIdx.x);
}

// Stage 2 (one CTA): rho = ordered sum of the chunk partials, then the
// Hartree potential (F:147-162), vloc = vH + vion and the density scalars.
template <int N>
__device__ __forceinline__ void density_body(const DensArgs& a) {
  using TM = Team<N>;
  __shared__ double rho_s[N];
  __shared__ double vh_s[N];
  __shared__ double2 tw_s[N];
  __shared__ double2 buf_s[TM::PER_WARP][N];
  const int tid = threadIdx.x;
  for (int i = tid; i < N; i += blockDim.x) tw_s[i] = a.tw[i];
  for (int ig = tid; ig < N; ig += blockDim.x) {
    double s = a.part[ig];
    for (int ch = 1; ch < kDensChunks; ++ch) s += a.part[(size_t)ch * N + ig];
    rho_s[ig] = s;
    a.rho[ig] = s;
  }
  __syncthreads();
  if (tid < 32) {
    const int lane = tid, tl = lane % TM::T, team = lane / TM::T;
    double2 x[TM::E];
#pragma unroll
    for (int e = 0; e < TM::E; ++e) x[e] = make_double2(rho_s[TM::pos(tl, e)], 0.0);
    fft_team<N, -1>(x, buf_s[team], tw_s, tl);
#pragma unroll
    for (int e = 0; e < TM::E; ++e) {
      const double v = a.vCG[TM::pos(tl, e)];
      x[e] = make_double2(v * x[e].x, v * x[e].y);
    }
    fft_team<N, +1>(x, buf_s[team], tw_s, tl);
    if (team == 0) {
#pragma unroll
      for (int e = 0; e < TM::E; ++e) vh_s[TM::pos(tl, e)] = x[e].x / (double)N;
    }
  }
  __syncthreads();
  if (a.mu != nullptr) {
    for (int ig = tid; ig < N; ig += blockDim.x) {
      a.vloc[ig] = vh_s[ig];
      if (a.gvion) a.gvion[ig] += rho_s[ig];
    }
    return;
  }
  for (int ig = tid; ig < N; ig += blockDim.x) a.vloc[ig] = vh_s[ig] + a.vion[ig];
  if (tid < 32) {
    // Nele, Eion, EH: lane-strided partial sums, then a fixed shuffle tree
    double sn = 0.0, si = 0.0, sh = 0.0;
    for (int ig = tid; ig < N; ig += 32) {
      sn += rho_s[ig];
      si += a.vion[ig] * rho_s[ig];
      sh += vh_s[ig] * rho_s[ig];
    }
    sn = warp_sum(sn);
    si = warp_sum(si);
    sh = warp_sum(sh);
    if (tid == 0) {
      a.scal[0] = sn * a.dvcell;
      a.scal[1] = si * a.dvcell;
      a.scal[2] = 0.5 * sh * a.dvcell;
    }
  }
}

template <int N>
__global__ void __launch_bounds__(512) k_density(DensArgs a) { density_body<N>(a); }


// one CTA per run
template <int N>
__global__ void __launch_bounds__(512) k_density_batch(const DensArgs* __restrict__ args) {
  density_body<N>(args[blockIdx.x]);
}

// run owning work item `i` given exclusive prefix sums pre[0..nruns] (pre[0] = 0)
__device__ __forceinline__ int find_run(const int* __restrict__ pre, int nruns, int i) {
  int lo = 0, hi = nruns - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Fock exchange pair kernel (F:237-261).
//
// Work item = (output column (kr, ibr), chunk of source pairs (kc, ibc)).
// Each team streams its share of the chunk's pairs:
//   x = w(kr,ibr) * conj(u(kc,ibc));  X = FFT(x);  X *= -v(G+kx(kr)-kx(kc))/(NG NK);
//   x = IFFT(X);  acc += x * u(kc,ibc)
// with w, u, acc held in registers at the team's fixed FFT slot positions.
// Teams are reduced in a fixed order and the partial column is written to
// scratch[item]; the combine kernel sums the chunks in order.  No atomics,
// bitwise-reproducible.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(kThreads) k_fock(FockArgs a) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NWARP = kThreads / 32;
  constexpr int NTEAM = NWARP * PW;
  extern __shared__ double2 sm[];
  double2* tw_s = sm;                 // N
  double2* bufs = sm + N;             // NTEAM * N
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, tiw = lane / T, team = warp * PW + tiw;
  double2* buf = bufs + team * N;
  for (int i = tid; i < N; i += kThreads) tw_s[i] = a.tw[i];
  __syncthreads();

  const int item = blockIdx.x;
  const int col = item / a.nchunks, chunk = item % a.nchunks;
  const int kr = col / a.w.nb, ibr = col % a.w.nb;
  const double2* wcol = a.w.p + (size_t)kr * a.w.kstride + (size_t)ibr * N;
  // w and u columns are re-read (L1/L2) instead of held in registers
  double2 acc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) acc[e] = make_double2(0.0, 0.0);
  const int npairs = a.nk * a.nbocc;
  const int p0 = chunk * a.chunk;
  const int p1 = min(npairs, p0 + a.chunk);
  // warp-uniform trip count: every team of a warp runs the same rounds
  for (int base = p0 + warp * PW; base < p1; base += NTEAM) {
    const int p = base + tiw;
    const bool valid = p < p1;
    const int pp = valid ? p : p0;
    const int kc = pp / a.nbocc, ibc = pp % a.nbocc;
    const double2* ucol = a.u.p + (size_t)kc * a.u.kstride + (size_t)ibc * N;
    const double* kern = a.kern + (size_t)(kr - kc + a.nk - 1) * N;
    double2 x[E];
    fft_team_in<N, -1>(InConjProduct<N>{wcol, ucol, tl}, x, buf, tw_s, tl);
    fft_team_in<N, +1>(InScaled<N>{x, kern, tl}, x, buf, tw_s, tl);
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) acc[e] = cfma(x[e], ucol[TM::pos(tl, e)], acc[e]);
    }
  }
  // fixed-order reduction over teams
#pragma unroll
  for (int e = 0; e < E; ++e) buf[TM::pos(tl, e)] = acc[e];
  __syncthreads();
  double2* dst = a.scratch + (size_t)item * N;
  for (int i = tid; i < N; i += kThreads) {
    double2 s = bufs[i];
    for (int t = 1; t < NTEAM; ++t) s = cadd(s, bufs[t * N + i]);
    dst[i] = s;
  }
}


// ---------------------------------------------------------------------------
// Symmetric exchange for w == u over occupied pairs (same F:237-261 sum).
//
// For occupied orbitals a=(ka,ba), b=(kb,bb) the pair potentials obey
//   phi_ba(x_m) = conj(phi_ab(x_m)) + (kern_ba[N/2] - kern_ab[N/2]) conj(R_ab[N/2]) (-1)^m
// (the soft-Coulomb kernel is even; only the self-aliased Nyquist frequency
// breaks the conjugate symmetry, R_ab being FFT(u_a conj(u_b))).  One pair of
// transforms therefore yields both out(a) += phi_ab u_b and
// out(b) += phi_ba u_a.  A CTA handles a tile pair (i <= j) of S orbitals:
// team w owns row a = i*S + w (accumulated in registers) and in round r
// visits b = j*S + (w + r) % S, so within a round every column accumulator
// (shared memory) has exactly one writer.  Diagonal tiles visit each
// unordered pair once (rounds 0..S/2).
// ---------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void fock_sym_body(const FockSymArgs& a, const int tile) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  const int S = a.S;                          // tile size (runtime, <= teams per CTA)
  const int nteam = (blockDim.x >> 5) * PW;    // teams in this CTA (>= S)
  extern __shared__ double2 sm[];
  double2* tw_s = sm;                  // N
  double2* bufs = sm + N;              // nteam * N  (team FFT buffers)
  double2* cacc = bufs + nteam * N;    // S * N  (column accumulators)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, tw_ = warp * PW + lane / T;
  const int team_lane0 = (lane / T) * T;
  double2* buf = bufs + tw_ * N;
  for (int i = tid; i < N; i += blockDim.x) tw_s[i] = a.tw[i];
  for (int i = tid; i < S * N; i += blockDim.x) cacc[i] = make_double2(0.0, 0.0);
  // tile pair (ti, tj), ti <= tj, from the linear block index
  int ti = 0, rem = tile;
  while (rem >= a.T - ti) { rem -= a.T - ti; ++ti; }
  const int tj = ti + rem;
  const int M = a.nk * a.nbocc;
  const int ia = ti * S + tw_;
  const bool va = tw_ < S && ia < M;
  const int ka = (va ? ia : 0) / a.nbocc, ba = (va ? ia : 0) % a.nbocc;
  // orbitals are re-read from global memory (L1/L2-resident) where needed
  // rather than held in registers: the kernel is FP64-pipe bound, and this
  // keeps the largest grids free of register spills
  const double2* ucol_a = a.u.p + (size_t)ka * a.u.kstride + (size_t)ba * N;
  double2 racc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) racc[e] = make_double2(0.0, 0.0);
  __syncthreads();
  const bool diag = (ti == tj);
  const int nrounds = diag ? (S / 2 + 1) : S;
  for (int r = 0; r < nrounds; ++r) {
    const int lb = (tw_ + r) % S;
    const int ib = tj * S + lb;
    bool valid = va && ib < M;
    if (diag && (S % 2 == 0) && r == S / 2 && tw_ >= S / 2) valid = false;  // counted by the partner
    const bool self = diag && r == 0;
    const int kb = (ib < M ? ib : 0) / a.nbocc, bb = (ib < M ? ib : 0) % a.nbocc;
    const double2* ucol_b = a.u.p + (size_t)kb * a.u.kstride + (size_t)bb * N;
    double2 x[E];
    fft_team_in<N, -1>(InConjProduct<N>{ucol_a, ucol_b, tl}, x, buf, tw_s, tl);
    // Nyquist coefficient R_ab[N/2] lives in slot (p=0, r=R0/2) of the team's lane 0
    const double2 rn_own = x[TM::R0 / 2];
    const double rnx = __shfl_sync(0xffffffffu, rn_own.x, team_lane0);
    const double rny = __shfl_sync(0xffffffffu, rn_own.y, team_lane0);
    const int dab = ka - kb + a.nk - 1, dba = kb - ka + a.nk - 1;
    const double* kab = a.kern + (size_t)dab * N;
    fft_team_in<N, +1>(InScaled<N>{x, kab, tl}, x, buf, tw_s, tl);
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) racc[e] = cfma(x[e], ucol_b[TM::pos(tl, e)], racc[e]);
      if (!self) {
        const double dk = __ldg(a.kern + (size_t)dba * N + N / 2) - __ldg(kab + N / 2);
        const double cx = dk * rnx, cy = -dk * rny;  // dk * conj(R)
        double2* col = cacc + lb * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          const double sg = (q & 1) ? -1.0 : 1.0;
          const double2 pba = make_double2(fma(sg, cx, x[e].x), fma(sg, cy, -x[e].y));
          col[q] = cfma(pba, ucol_a[q], col[q]);
        }
      }
    }
    __syncthreads();
  }
  // write partials: rows from registers, columns from shared memory
  double2* dst = a.scratch + (size_t)tile * 2 * S * N;
  if (tw_ < S) {
#pragma unroll
    for (int e = 0; e < E; ++e) dst[(size_t)tw_ * N + TM::pos(tl, e)] = racc[e];
  }
  for (int i = tid; i < S * N; i += blockDim.x) dst[(size_t)S * N + i] = cacc[i];
}

template <int N>
__global__ void __launch_bounds__(kThreads) k_fock_sym(FockSymArgs a) { fock_sym_body<N>(a, blockIdx.x); }

template <int N>
__global__ void __launch_bounds__(kThreads) k_fock_sym_batch(const FockSymArgs* __restrict__ args,
                                                           const int* __restrict__ pre, int nruns) {
  const int r = find_run(pre, nruns, blockIdx.x);
  fock_sym_body<N>(args[r], blockIdx.x - pre[r]);
}

// Sum the tile-pair partials of every occupied output into F[o][q] (fixed
// order over tiles: column partials of earlier tiles, the diagonal tile's row
// and column partials, row partials of later tiles).
// Run c of the ordered partial sum of output element idx (see sym_term).
__device__ __forceinline__ double2 sym_run_sum(const double2* __restrict__ part, int S, int T, int N, int idx,
                                               int c) {
  const int o = idx / N, q = idx % N;
  const int i = o / S, l = o % S;
  int t0, t1;
  sym_run_bounds(T, c, &t0, &t1);
  double2 f = make_double2(0.0, 0.0);
#pragma unroll 4
  for (int t = t0; t < t1; ++t) f = cadd(f, part[sym_term(t, i, l, q, S, T, N)]);
  return f;
}

// kRedQ runs per element through shared memory, added in run order.
__device__ __forceinline__ void sym_reduce_finish(double2 f, bool valid, double2* __restrict__ out) {
  __shared__ double2 red[kRedQ][kRedE];
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  red[c][e] = f;
  __syncthreads();
  if (c == 0 && valid) {
    double2 s = red[0][e];
#pragma unroll
    for (int k = 1; k < kRedQ; ++k) s = cadd(s, red[k][e]);
    *out = s;
  }
}

__global__ void __launch_bounds__(kRedQ* kRedE) k_sym_reduce(const double2* __restrict__ part, int S, int T,
                                                             int M, int N, double2* __restrict__ F) {
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  const int idx = blockIdx.x * kRedE + e;
  const bool valid = idx < M * N;
  const double2 f = valid ? sym_run_sum(part, S, T, N, idx, c) : make_double2(0.0, 0.0);
  sym_reduce_finish(f, valid, F + (valid ? idx : 0));
}

// element prefix: pre[r] = sum over earlier runs of M_r * N
__global__ void __launch_bounds__(kRedQ* kRedE) k_sym_reduce_batch(const FockSymArgs* __restrict__ args,
                                                                   const int* __restrict__ pre, int nruns,
                                                                   int N) {
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  const int idx = blockIdx.x * kRedE + e;
  const bool valid = idx < pre[nruns];
  double2 f = make_double2(0.0, 0.0);
  double2* out = nullptr;
  if (valid) {
    const int r = find_run(pre, nruns, idx);
    const FockSymArgs& a = args[r];
    f = sym_run_sum(a.scratch, a.S, a.T, N, idx - pre[r], c);
    out = a.F + (idx - pre[r]);
  }
  sym_reduce_finish(f, valid, out);
}

// Exchange term of output column (ik, ib) at grid point q, summed over the
// partials in a fixed order.
__device__ __forceinline__ double2 exchange_at(const CombineArgs& a, int ik, int ib, int q, int N) {
  if (a.sym != nullptr && ib < a.nbocc) return a.sym[(size_t)(ik * a.nbocc + ib) * N + q];
  const int nbc = a.w.nb - a.chunk_b0;
  const int c = ik * nbc + (ib - a.chunk_b0);
  const double2* src = a.scratch + (size_t)c * a.nchunks * N + q;
  double2 f = src[0];
  for (int ch = 1; ch < a.nchunks; ++ch) f = cadd(f, src[(size_t)ch * N]);
  return f;
}

// ---------------------------------------------------------------------------
// Combine: kinetic (F:212-234) + local potential (F:199-203) + Fock partials,
// then the mode's epilogue (RK4 stages RT:166-170, observables F:94-119,
// F:165-183, F:289-318).  One team per output column.
// ---------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void combine_body(const CombineArgs& a, const int ncols, const int cta) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NTEAM = kCombineWarps * PW;
  __shared__ double2 tw_s[N];
  __shared__ double2 bufs[NTEAM][N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, team = warp * PW + lane / T;
  for (int i = tid; i < N; i += kCombineWarps * 32) tw_s[i] = a.tw[i];
  __syncthreads();
  const double A = afield_value(a.af);
  // warp-uniform: whole warps go idle together
  const int col0 = (cta * kCombineWarps + warp) * PW;
  if (col0 >= ncols) return;
  const int col = col0 + lane / T;
  const bool valid = col < ncols;
  const int c = valid ? col : col0;
  const int ik = c / a.w.nb, ib = c % a.w.nb;
  const double2* wcol = a.w.p + (size_t)ik * a.w.kstride + (size_t)ib * N;
  double2 wv[E], x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    wv[e] = wcol[TM::pos(tl, e)];
    x[e] = wv[e];
  }
  // split == 2: the kinetic and local-potential part was made by the split == 1
  // pass (beside the exchange); only the exchange and the epilogue remain
  const bool post = a.split == 2;
  if (!post) fft_team<N, -1>(x, bufs[team], tw_s, tl);
  const double kAx = a.kx[ik] + A;
  const double kA2 = kAx * kAx;
  if (a.mode == CM_OBS) {
    // Ekin and Je of this column by Parseval on FFT(u):
    //   sum_x conj(u) IFFT(f * FFT(u)) = sum_G f(G) |FFT(u)(G)|^2
    double ek = 0.0, je = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const double G = a.Gx[TM::pos(tl, e)];
      const double m2 = x[e].x * x[e].x + x[e].y * x[e].y;
      ek += 0.5 * (G * G + 2.0 * G * kAx + kA2) * m2;
      je += (G + a.kx[ik] + A) * m2;
    }
    ek = team_sum<T>(ek) / (double)N;
    je = team_sum<T>(je) / (double)N;
    double fr = 0.0, fi = 0.0;
    if ((a.scratch != nullptr || a.sym != nullptr) && ib < a.nbocc) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const double2 f = exchange_at(a, ik, ib, TM::pos(tl, e), N);
        fr += wv[e].x * f.x + wv[e].y * f.y;
        fi += wv[e].x * f.y - wv[e].y * f.x;
      }
    }
    fr = team_sum<T>(fr);
    fi = team_sum<T>(fi);
    if (valid && tl == 0) {
      double* cb = a.colbuf + (size_t)c * 4;
      cb[0] = ek;
      cb[1] = je;
      cb[2] = fr;
      cb[3] = fi;
    }
    return;
  }
  if (!post) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const double G = a.Gx[TM::pos(tl, e)];
      const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
      x[e] = make_double2(m * x[e].x / (double)N, m * x[e].y / (double)N);
    }
    fft_team<N, +1>(x, bufs[team], tw_s, tl);
  }
  const size_t ocol = (size_t)ik * a.w.nb * N + (size_t)ib * N;  // [NK][NB][NG]
  if (a.split == 1) {
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int q = TM::pos(tl, e);
        const double v = a.vloc[q];
        a.hpre[ocol + q] = make_double2(x[e].x + v * wv[e].x, x[e].y + v * wv[e].y);
      }
    }
    return;
  }
  // deferred exchange energy: <w|F> of occupied columns (stage 1 of an RK4 step)
  double exr = 0.0, exi = 0.0;
  bool bad = false;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int q = TM::pos(tl, e);
    double2 h;
    if (a.mode == CM_T) {
      h = x[e];
    } else {
      if (a.mode == CM_F) h = make_double2(0.0, 0.0);
      else if (post) h = a.hpre[ocol + q];
      else {
        const double v = a.vloc[q];
        h = make_double2(x[e].x + v * wv[e].x, x[e].y + v * wv[e].y);
      }
      if (a.scratch != nullptr || a.sym != nullptr) {
        const double2 f = exchange_at(a, ik, ib, q, N);
        if (a.ex_cols) {
          exr += wv[e].x * f.x + wv[e].y * f.y;
          exi += wv[e].x * f.y - wv[e].y * f.x;
        }
        h = cadd(h, f);
      }
    }
    if (!valid) continue;
    if (a.mode == CM_H || a.mode == CM_F || a.mode == CM_T) {
      a.out.p[(size_t)ik * a.out.kstride + (size_t)ib * N + q] = h;
      bad |= !(isfinite(h.x) && isfinite(h.y));
      continue;
    }
    // RK4: k = -i h
    const double2 k = make_double2(h.y, -h.x);
    const size_t o = (size_t)ik * a.w.nb * N + (size_t)ib * N + q;  // [NK][NB][NG]
    const double2 u0 = a.u0[o];
    double2 nx;
    if (a.mode == CM_RK0 || a.mode == CM_RK1 || a.mode == CM_RK2) {
      a.kbuf[a.mode - CM_RK0][o] = k;
      const double cdt = (a.mode == CM_RK2) ? a.dt : 0.5 * a.dt;
      nx = make_double2(u0.x + cdt * k.x, u0.y + cdt * k.y);
      a.out.p[(size_t)ik * a.out.kstride + (size_t)ib * N + q] = nx;
    } else {  // CM_RK3: ubk + (k1 + 2 k2 + 2 k3 + k4) * dt / 6
      const double2 k0 = a.kbuf[0][o], k1 = a.kbuf[1][o], k2 = a.kbuf[2][o];
      double sx = k0.x + 2.0 * k1.x, sy = k0.y + 2.0 * k1.y;
      sx = sx + 2.0 * k2.x;
      sy = sy + 2.0 * k2.y;
      sx = sx + k.x;
      sy = sy + k.y;
      sx = sx * a.dt / 6.0;
      sy = sy * a.dt / 6.0;
      nx = make_double2(u0.x + sx, u0.y + sy);
      a.u0[o] = nx;
    }
    bad |= !(isfinite(nx.x) && isfinite(nx.y));
  }
  if (a.ex_cols) {
    exr = team_sum<T>(exr);
    exi = team_sum<T>(exi);
    if (valid && tl == 0) {
      a.colbuf[(size_t)c * 4 + 2] = exr;
      a.colbuf[(size_t)c * 4 + 3] = exi;
    }
  }
  if (bad && a.nonfinite) *a.nonfinite = 1;
}

template <int N>
__global__ void __launch_bounds__(kCombineWarps * 32) k_combine(CombineArgs a, int ncols) {
  combine_body<N>(a, ncols, blockIdx.x);
}

// CTA prefix: pre[r] = sum over earlier runs of ceil(ncols_r / columns per CTA)
template <int N>
__global__ void __launch_bounds__(kCombineWarps * 32) k_combine_batch(const CombineArgs* __restrict__ args,
                                                          const int* __restrict__ pre, int nruns) {
  const int r = find_run(pre, nruns, blockIdx.x);
  const CombineArgs& a = args[r];
  combine_body<N>(a, a.nk * a.w.nb, blockIdx.x - pre[r]);
}

// Deferred exchange energy Ex = 0.5 sum_occ occ <u|F u> dvcell (F:165-183),
// added to the Etot of the step whose orbitals produced F.
__device__ __forceinline__ void ex_finalize_body(const ExArgs& a, int lane) {
  int idx = a.idx;
  if (idx < 0) idx = *a.it - 1;
  if (idx < 0) return;
  double ex = 0.0;
  const int ncol = a.nk * a.nbocc;
  for (int o = lane; o < ncol; o += 32) {
    const int ik = o / a.nbocc, ib = o % a.nbocc;
    ex += a.occ * a.colbuf[(size_t)(ik * a.nb + ib) * 4 + 2] * a.dvcell;
  }
  ex = 0.5 * warp_sum(ex);
  if (lane != 0) return;
  if (a.series_E) a.series_E[idx] = a.series_E[idx] + ex;
  if (a.out) {
    a.out[0] = a.out[0] + ex;
    a.out[4] = ex;
  }
}

__global__ void k_ex_finalize(ExArgs a) {
  if (blockIdx.x == 0 && threadIdx.x < 32) ex_finalize_body(a, threadIdx.x);
}

__global__ void k_ex_finalize_batch(const ExArgs* __restrict__ args, int nruns) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r < nruns) ex_finalize_body(args[r], threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// Observable reduction (F:74-91, F:165-183, F:289-318) in reference order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void obs_reduce_body(const ObsReduceArgs& a, int lane) {
  double ekin = 0.0, jre = 0.0, exr = 0.0;
  const int ncol = a.nk * a.nb;
  for (int c = lane; c < ncol; c += 32) {
    const int ib = c % a.nb;
    const double occ = ib < a.nbocc ? a.occ : 0.0;
    const double* cb = a.colbuf + (size_t)c * 4;
    ekin += occ * cb[0] * a.dvcell;
    jre += occ * cb[1];
    if (ib < a.nbocc && !a.defer_ex) exr += occ * cb[2] * a.dvcell;
  }
  ekin = warp_sum(ekin);
  jre = warp_sum(jre);
  exr = warp_sum(exr);
  if (lane != 0) return;
  const double Ex = (a.hf && !a.defer_ex) ? 0.5 * exr : 0.0;
  const double Eion = a.scal[1], EH = a.scal[2], Nele = a.scal[0];
  const double Etot = a.defer_ex ? (ekin + Eion + EH) : (ekin + Eion + EH + Ex);
  const double Je = -(jre * a.dvcell / a.vcell);
  a.out[0] = Etot;
  a.out[1] = ekin;
  a.out[2] = Eion;
  a.out[3] = EH;
  a.out[4] = Ex;
  a.out[5] = Je;
  a.out[6] = Nele;
  if (a.advance) {
    const int it = *a.it;
    if (a.series_E) a.series_E[it] = Etot;
    if (a.series_J) a.series_J[it] = Je;
    if (a.series_N) a.series_N[it] = Nele;
    if (!(isfinite(Etot) && isfinite(Je) && isfinite(Nele)) && a.nonfinite) *a.nonfinite = 1;
    if (a.advance == 1) *a.it = it + 1;
  }
}

__global__ void k_obs_reduce(ObsReduceArgs a) {
  if (blockIdx.x == 0 && threadIdx.x < 32) obs_reduce_body(a, threadIdx.x);
}

// one warp per run; the step counter is advanced by k_step_advance afterwards
__global__ void k_obs_reduce_batch(const ObsReduceArgs* __restrict__ args, int nruns) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r < nruns) obs_reduce_body(args[r], threadIdx.x & 31);
}

__global__ void k_step_advance(int* it) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *it = *it + 1;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <int N>
static cudaError_t fock_impl(const FockArgs& a, int ncols, cudaStream_t s) {
  constexpr int NTEAM = (kThreads / 32) * Team<N>::PER_WARP;
  const size_t smem = sizeof(double2) * (size_t)N * (1 + NTEAM);
  static_assert(sizeof(double2) * N * (1 + NTEAM) <= 48 * 1024, "fits the default dynamic smem limit");
  const int items = ncols * a.nchunks;
  if (items == 0) return cudaSuccess;
  k_fock<N><<<items, kThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
static constexpr int sym_teams() { return (kThreads / 32) * Team<N>::PER_WARP; }

template <int N>
static size_t sym_smem() { return sizeof(double2) * (size_t)N * (1 + 2 * sym_teams<N>()); }

// threads and dynamic shared memory of a symmetric-exchange CTA with tile size S
template <int N>
static void sym_launch_shape(int S, int* threads, size_t* smem) {
  constexpr int PW = Team<N>::PER_WARP;
  const int warps = (S + PW - 1) / PW;
  *threads = 32 * warps;
  *smem = sizeof(double2) * (size_t)N * (1 + warps * PW + S);
}

template <int N>
static cudaError_t fock_sym_impl(const FockSymArgs& a, cudaStream_t s) {
  const int tiles = a.T * (a.T + 1) / 2;
  if (tiles == 0) return cudaSuccess;
  int threads;
  size_t smem;
  sym_launch_shape<N>(a.S, &threads, &smem);
  k_fock_sym<N><<<tiles, threads, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int M = a.nk * a.nbocc;
  k_sym_reduce<<<(M * N + kRedE - 1) / kRedE, kRedQ * kRedE, 0, s>>>(a.scratch, a.S, a.T, M, N, a.F);
  return cudaGetLastError();
}

template <int N>
static cudaError_t configure_impl() {
  // the single-run and the batched symmetric exchange (above 48 KB at NG = 512)
  const cudaError_t e =
      cudaFuncSetAttribute(k_fock_sym<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem<N>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_fock_sym_batch<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem<N>());
}

template <int N>
static cudaError_t combine_impl(const CombineArgs& a, int ncols, cudaStream_t s) {
  constexpr int PER_CTA = kCombineWarps * Team<N>::PER_WARP;
  const int blocks = (ncols + PER_CTA - 1) / PER_CTA;
  if (blocks == 0) return cudaSuccess;
  k_combine<N><<<blocks, kCombineWarps * 32, 0, s>>>(a, ncols);
  return cudaGetLastError();
}

#define MATTOHF_DISPATCH(NG, CALL)                 \
  switch (NG) {                                    \
    case 16: return CALL(16);                      \
    case 32: return CALL(32);                      \
    case 64: return CALL(64);                      \
    case 128: return CALL(128);                    \
    case 256: return CALL(256);                    \
    case 512: return CALL(512);                    \
    default: return cudaErrorInvalidValue;         \
  }

cudaError_t launch_density(int NG, const DensArgs& a, cudaStream_t s) {
  k_dens_partial<<<kDensChunks, 256, 0, s>>>(a, NG);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
#define CALL(n) (k_density<n><<<1, (n) < 64 ? 64 : (n), 0, s>>>(a), cudaGetLastError())
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_fock(int NG, const FockArgs& a, int ncols, cudaStream_t s) {
#define CALL(n) fock_impl<n>(a, ncols, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_fock_sym(int NG, const FockSymArgs& a, cudaStream_t s) {
#define CALL(n) fock_sym_impl<n>(a, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

// Largest tile size (a power of two up to the teams of a full CTA) that still
// yields enough tile pairs to occupy every one of the device's nsm SMs four
// times; small systems fall back to small tiles so their few pairs spread over
// many SMs.
int choose_sym_tile(int NG, int M, int nsm) {
  int S = fock_sym_teams(NG);
  const int want = 4 * (nsm > 0 ? nsm : 1);
  while (S > 1) {
    const int T = (M + S - 1) / S;
    if (T * (T + 1) / 2 >= want) break;
    S >>= 1;
  }
  return S;
}

cudaError_t sym_launch_params(int NG, int S, int* threads, size_t* smem) {
  switch (NG) {
    case 16: sym_launch_shape<16>(S, threads, smem); break;
    case 32: sym_launch_shape<32>(S, threads, smem); break;
    case 64: sym_launch_shape<64>(S, threads, smem); break;
    case 128: sym_launch_shape<128>(S, threads, smem); break;
    case 256: sym_launch_shape<256>(S, threads, smem); break;
    case 512: sym_launch_shape<512>(S, threads, smem); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

int fock_sym_teams(int NG) {
  switch (NG) {
    case 16: return sym_teams<16>();
    case 32: return sym_teams<32>();
    case 64: return sym_teams<64>();
    case 128: return sym_teams<128>();
    case 256: return sym_teams<256>();
    case 512: return sym_teams<512>();
    default: return 0;
  }
}

// Per-device kernel attributes (larger dynamic shared memory); call with the
// device current.
cudaError_t configure_kernels() {
  cudaError_t e;
  if ((e = configure_impl<16>()) != cudaSuccess) return e;
  if ((e = configure_impl<32>()) != cudaSuccess) return e;
  if ((e = configure_impl<64>()) != cudaSuccess) return e;
  if ((e = configure_impl<128>()) != cudaSuccess) return e;
  if ((e = configure_impl<256>()) != cudaSuccess) return e;
  return configure_impl<512>();
}

cudaError_t launch_ex_finalize(const ExArgs& a, cudaStream_t s) {
  k_ex_finalize<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_combine(int NG, const CombineArgs& a, int ncols, cudaStream_t s) {
#define CALL(n) combine_impl<n>(a, ncols, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

// ---- batched launchers (many independent runs per launch) ----
cudaError_t launch_density_batch(int NG, const DensArgs* d_args, int nruns, cudaStream_t s) {
  k_dens_partial_batch<<<dim3(kDensChunks, nruns), 256, 0, s>>>(d_args, NG);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
#define CALL(n) (k_density_batch<n><<<nruns, (n) < 64 ? 64 : (n), 0, s>>>(d_args), cudaGetLastError())
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

template <int N>
static cudaError_t fock_sym_batch_impl(const FockSymArgs* d_args, const int* d_tile_pre, int nruns,
                                       int total_tiles, const int* d_elem_pre, int total_elems,
                                       cudaStream_t s) {
  if (total_tiles <= 0) return cudaSuccess;
  k_fock_sym_batch<N><<<total_tiles, kThreads, sym_smem<N>(), s>>>(d_args, d_tile_pre, nruns);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_sym_reduce_batch<<<(total_elems + kRedE - 1) / kRedE, kRedQ * kRedE, 0, s>>>(d_args, d_elem_pre, nruns, N);
  return cudaGetLastError();
}

cudaError_t launch_fock_sym_batch(int NG, const FockSymArgs* d_args, const int* d_tile_pre, int nruns,
                                  int total_tiles, const int* d_elem_pre, int total_elems,
                                  cudaStream_t s) {
#define CALL(n) fock_sym_batch_impl<n>(d_args, d_tile_pre, nruns, total_tiles, d_elem_pre, total_elems, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

int combine_cols_per_cta(int NG) {
  switch (NG) {
    case 16: return kCombineWarps * Team<16>::PER_WARP;
    case 32: return kCombineWarps * Team<32>::PER_WARP;
    case 64: return kCombineWarps * Team<64>::PER_WARP;
    case 128: return kCombineWarps * Team<128>::PER_WARP;
    case 256: return kCombineWarps * Team<256>::PER_WARP;
    case 512: return kCombineWarps * Team<512>::PER_WARP;
    default: return 0;
  }
}

cudaError_t launch_combine_batch(int NG, const CombineArgs* d_args, const int* d_cta_pre, int nruns,
                                 int total_ctas, cudaStream_t s) {
  if (total_ctas <= 0) return cudaSuccess;
#define CALL(n) (k_combine_batch<n><<<total_ctas, kCombineWarps * 32, 0, s>>>(d_args, d_cta_pre, nruns), cudaGetLastError())
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_obs_reduce_batch(const ObsReduceArgs* d_args, int nruns, cudaStream_t s) {
  k_obs_reduce_batch<<<(nruns + 3) / 4, 128, 0, s>>>(d_args, nruns);
  return cudaGetLastError();
}

cudaError_t launch_ex_finalize_batch(const ExArgs* d_args, int nruns, cudaStream_t s) {
  k_ex_finalize_batch<<<(nruns + 3) / 4, 128, 0, s>>>(d_args, nruns);
  return cudaGetLastError();
}

cudaError_t launch_step_advance(int* it, cudaStream_t s) {
  k_step_advance<<<1, 32, 0, s>>>(it);
  return cudaGetLastError();
}

cudaError_t launch_sym_reduce(const double2* part, int S, int T, int M, int N, double2* F, cudaStream_t s) {
  k_sym_reduce<<<(M * N + kRedE - 1) / kRedE, kRedQ * kRedE, 0, s>>>(part, S, T, M, N, F);
  return cudaGetLastError();
}

cudaError_t launch_obs_reduce(const ObsReduceArgs& a, cudaStream_t s) {
  k_obs_reduce<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mattohf
