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

// ---------------------------------------------------------------------------
// Density (F:55-71) and Hartree potential (F:147-162), one CTA.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(256) k_density(DensArgs a) {
  using TM = Team<N>;
  __shared__ double rho_s[N];
  __shared__ double vh_s[N];
  __shared__ double2 tw_s[N];
  __shared__ double2 buf_s[TM::PER_WARP][N];
  const int tid = threadIdx.x;
  for (int i = tid; i < N; i += blockDim.x) tw_s[i] = a.tw[i];
  // rho(ig) = sum_ik sum_ib occ*|u|^2, ik outer, ib inner (reference order)
  for (int ig = tid; ig < N; ig += blockDim.x) {
    double s = 0.0;
    for (int ik = 0; ik < a.nk; ++ik) {
      const double2* col = a.u.p + (size_t)ik * a.u.kstride + ig;
      for (int ib = 0; ib < a.u.nb; ++ib) {
        const double occ = ib < a.nbocc ? a.occ : 0.0;
        const double2 z = col[(size_t)ib * N];
        s += fma(occ * z.x, z.x, (occ * z.y) * z.y);
      }
    }
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
  for (int ig = tid; ig < N; ig += blockDim.x) a.vloc[ig] = vh_s[ig] + a.vion[ig];
  if (tid == 0) {
    // sequential sums, as the Fortran SUM intrinsic evaluates them
    double sn = 0.0, si = 0.0, sh = 0.0;
    for (int ig = 0; ig < N; ++ig) {
      sn += rho_s[ig];
      si += a.vion[ig] * rho_s[ig];
      sh += vh_s[ig] * rho_s[ig];
    }
    a.scal[0] = sn * a.dvcell;
    a.scal[1] = si * a.dvcell;
    a.scal[2] = 0.5 * sh * a.dvcell;
  }
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
  double2 wv[E], acc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    wv[e] = wcol[TM::pos(tl, e)];
    acc[e] = make_double2(0.0, 0.0);
  }
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
    double2 uv[E], x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      uv[e] = ucol[TM::pos(tl, e)];
      x[e] = cmulc(wv[e], uv[e]);
    }
    fft_team<N, -1>(x, buf, tw_s, tl);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const double v = __ldg(kern + TM::pos(tl, e));
      x[e] = make_double2(v * x[e].x, v * x[e].y);
    }
    fft_team<N, +1>(x, buf, tw_s, tl);
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) acc[e] = cfma(x[e], uv[e], acc[e]);
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
__global__ void __launch_bounds__(kThreads) k_fock_sym(FockSymArgs a) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int S = (kThreads / 32) * PW;
  extern __shared__ double2 sm[];
  double2* tw_s = sm;                  // N
  double2* bufs = sm + N;              // S * N  (team FFT buffers)
  double2* cacc = bufs + S * N;        // S * N  (column accumulators)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, tw_ = warp * PW + lane / T;
  const int team_lane0 = (lane / T) * T;
  double2* buf = bufs + tw_ * N;
  for (int i = tid; i < N; i += kThreads) tw_s[i] = a.tw[i];
  for (int i = tid; i < S * N; i += kThreads) cacc[i] = make_double2(0.0, 0.0);
  // tile pair (ti, tj), ti <= tj, from the linear block index
  int ti = 0, rem = blockIdx.x;
  while (rem >= a.T - ti) { rem -= a.T - ti; ++ti; }
  const int tj = ti + rem;
  const int M = a.nk * a.nbocc;
  const int ia = ti * S + tw_;
  const bool va = ia < M;
  const int ka = (va ? ia : 0) / a.nbocc, ba = (va ? ia : 0) % a.nbocc;
  const double2* ucol_a = a.u.p + (size_t)ka * a.u.kstride + (size_t)ba * N;
  double2 ua[E], racc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    ua[e] = ucol_a[TM::pos(tl, e)];
    racc[e] = make_double2(0.0, 0.0);
  }
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
    double2 ub[E], x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      ub[e] = ucol_b[TM::pos(tl, e)];
      x[e] = cmulc(ua[e], ub[e]);
    }
    fft_team<N, -1>(x, buf, tw_s, tl);
    // Nyquist coefficient R_ab[N/2] lives in slot (p=0, r=R0/2) of the team's lane 0
    const double2 rn_own = x[TM::R0 / 2];
    const double rnx = __shfl_sync(0xffffffffu, rn_own.x, team_lane0);
    const double rny = __shfl_sync(0xffffffffu, rn_own.y, team_lane0);
    const int dab = ka - kb + a.nk - 1, dba = kb - ka + a.nk - 1;
    const double* kab = a.kern + (size_t)dab * N;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const double v = __ldg(kab + TM::pos(tl, e));
      x[e] = make_double2(v * x[e].x, v * x[e].y);
    }
    fft_team<N, +1>(x, buf, tw_s, tl);
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) racc[e] = cfma(x[e], ub[e], racc[e]);
      if (!self) {
        const double dk = __ldg(a.kern + (size_t)dba * N + N / 2) - __ldg(kab + N / 2);
        const double cx = dk * rnx, cy = -dk * rny;  // dk * conj(R)
        double2* col = cacc + lb * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          const double sg = (q & 1) ? -1.0 : 1.0;
          const double2 pba = make_double2(fma(sg, cx, x[e].x), fma(sg, cy, -x[e].y));
          col[q] = cfma(pba, ua[e], col[q]);
        }
      }
    }
    __syncthreads();
  }
  // write partials: rows from registers, columns from shared memory
  double2* dst = a.scratch + (size_t)blockIdx.x * 2 * S * N;
#pragma unroll
  for (int e = 0; e < E; ++e) dst[(size_t)tw_ * N + TM::pos(tl, e)] = racc[e];
  for (int i = tid; i < S * N; i += kThreads) dst[(size_t)S * N + i] = cacc[i];
}

// Exchange term of output column (ik, ib) at grid point q, summed over the
// partials in a fixed order.
__device__ __forceinline__ double2 exchange_at(const CombineArgs& a, int ik, int ib, int q, int N) {
  if (a.sym != nullptr && ib < a.nbocc) {
    const int S = a.sym_S, T = a.sym_T;
    const int o = ik * a.nbocc + ib;
    const int i = o / S, l = o % S;
    double2 f = make_double2(0.0, 0.0);
    for (int j = 0; j < T; ++j) {
      if (j < i) {
        f = cadd(f, a.sym[((size_t)sym_tp(j, i, T) * 2 + 1) * S * N + (size_t)l * N + q]);
      } else if (j == i) {
        const size_t b = (size_t)sym_tp(i, i, T) * 2 * S * N + (size_t)l * N + q;
        f = cadd(f, a.sym[b]);
        f = cadd(f, a.sym[b + (size_t)S * N]);
      } else {
        f = cadd(f, a.sym[(size_t)sym_tp(i, j, T) * 2 * S * N + (size_t)l * N + q]);
      }
    }
    return f;
  }
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
__global__ void __launch_bounds__(kThreads) k_combine(CombineArgs a, int ncols) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NTEAM = (kThreads / 32) * PW;
  __shared__ double2 tw_s[N];
  __shared__ double2 bufs[NTEAM][N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, team = warp * PW + lane / T;
  for (int i = tid; i < N; i += kThreads) tw_s[i] = a.tw[i];
  __syncthreads();
  const double A = afield_value(a.af);
  // warp-uniform: whole warps go idle together
  const int col0 = (blockIdx.x * (kThreads / 32) + warp) * PW;
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
  fft_team<N, -1>(x, bufs[team], tw_s, tl);
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
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const double G = a.Gx[TM::pos(tl, e)];
    const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
    x[e] = make_double2(m * x[e].x / (double)N, m * x[e].y / (double)N);
  }
  fft_team<N, +1>(x, bufs[team], tw_s, tl);
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

// Deferred exchange energy Ex = 0.5 sum_occ occ <u|F u> dvcell (F:165-183),
// added to the Etot of the step whose orbitals produced F.
__global__ void k_ex_finalize(ExArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int idx = a.idx;
  if (idx < 0) idx = *a.it - 1;
  if (idx < 0) return;
  double ex = 0.0;
  for (int ik = 0; ik < a.nk; ++ik)
    for (int ib = 0; ib < a.nbocc; ++ib) ex += a.occ * a.colbuf[(size_t)(ik * a.nb + ib) * 4 + 2] * a.dvcell;
  ex = 0.5 * ex;
  if (a.series_E) a.series_E[idx] = a.series_E[idx] + ex;
  if (a.out) {
    a.out[0] = a.out[0] + ex;
    a.out[4] = ex;
  }
}

// ---------------------------------------------------------------------------
// Observable reduction (F:74-91, F:165-183, F:289-318) in reference order.
// ---------------------------------------------------------------------------
__global__ void k_obs_reduce(ObsReduceArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ekin = 0.0, jre = 0.0, exr = 0.0;
  for (int ik = 0; ik < a.nk; ++ik) {
    for (int ib = 0; ib < a.nb; ++ib) {
      const double occ = ib < a.nbocc ? a.occ : 0.0;
      const double* cb = a.colbuf + (size_t)(ik * a.nb + ib) * 4;
      ekin += occ * cb[0] * a.dvcell;
      jre += occ * cb[1];
      if (ib < a.nbocc && !a.defer_ex) exr += occ * cb[2] * a.dvcell;
    }
  }
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
    *a.it = it + 1;
  }
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

template <int N>
static cudaError_t fock_sym_impl(const FockSymArgs& a, cudaStream_t s) {
  const int tiles = a.T * (a.T + 1) / 2;
  if (tiles == 0) return cudaSuccess;
  k_fock_sym<N><<<tiles, kThreads, sym_smem<N>(), s>>>(a);
  return cudaGetLastError();
}

template <int N>
static cudaError_t configure_impl() {
  return cudaFuncSetAttribute(k_fock_sym<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem<N>());
}

template <int N>
static cudaError_t combine_impl(const CombineArgs& a, int ncols, cudaStream_t s) {
  constexpr int PER_CTA = (kThreads / 32) * Team<N>::PER_WARP;
  const int blocks = (ncols + PER_CTA - 1) / PER_CTA;
  if (blocks == 0) return cudaSuccess;
  k_combine<N><<<blocks, kThreads, 0, s>>>(a, ncols);
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
#define CALL(n) (k_density<n><<<1, 256, 0, s>>>(a), cudaGetLastError())
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

cudaError_t launch_obs_reduce(const ObsReduceArgs& a, cudaStream_t s) {
  k_obs_reduce<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mattohf
