// Fused reverse RK4 stage for small problems.
//
// One launch does what one stage of the backward step does as separate
// launches (stage copy, two densities and Hartree solves, the adjoint
// exchange and its reduction, the combine and the field-gradient sum; the
// adjoint of src/RT_calculation.f90:154-173 for the energy and current
// objectives).  All bands are occupied (the adjoint requires it), so the
// columns a = (k, b) are also the exchange orbitals.  Output column a is
// served by P CTAs (a, chunk):
//   * the column's first CTA sums rho(v) = occ sum |v|^2 and
//     sigma = sum Im(conj(mu) v) over slices of the orbitals with all its
//     threads; warp 6 then solves both Hartree problems with one transform
//     pair (vCG is real and even, so IFFT(vCG FFT(rho + i sigma)) is
//     vH[rho] + i vH[sigma]), giving vloc = vH[rho] + vion and psi = vH[sigma];
//     warp 7 forms the kinetic term T_A mu_a and the field-gradient partial
//     sum_G (G+k+A) Im(conj(FFT mu_a) FFT v_a) / N;
//   * the CTA's worker warps (all eight, or warps 0..5 in the column's first
//     CTA, which therefore takes half the others' share of orbitals) apply
//     the adjoint exchange of column a against the CTA's orbitals b in
//     ordered form.  A work unit is (a warp's group of orbitals b, pass);
//     units are dealt round-robin over the worker warps:
//       pass A: out_a += i (phi_ab + (-1)^m dk_ab R_ab) mu_b,
//         phi_ab = Phi_ab[v_a conj(v_b)], R_ab its Nyquist coefficient,
//         dk_ab = kern_ba[N/2] - kern_ab[N/2];
//       pass B: out_a += i v_b (Phi_ab[mu_a conj(v_b) - v_a conj(mu_b)]
//                              - dk_ab Nyq(v_a conj(mu_b)) (-1)^m),
//         the second part being the Nyquist term of the transposed pair
//         operator (see k_adjoint.cu), Nyq(f) = sum_m (-1)^m f(m);
//     these are the row-a terms of the symmetric adjoint exchange (k_fock_adj)
//     with the column terms written as the rows of the reversed pairs.  The
//     transforms use the 32-lane latency plans, so a unit is one team;
//   * the column's last CTA (per-column ticket) adds the P partials in chunk
//     order and does the stage bookkeeping element by element:
//       lu = i (T_A + vloc) mu + Fa + 2 occ psi v,  lam_u += lu,
//       lam_prev += cprev lu  (stage 0: lam = lam_u);
//   * the last column (global ticket) adds the field-gradient partials in
//     column order into gstage[n][slot]; stage 0 then steps n back.
// Nothing waits on another CTA.
#include "fft.cuh"
#include "internal.h"

namespace mattohf {

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjWarps = kAdjThreads / 32;

__device__ __forceinline__ double2 times_i(double2 a) { return make_double2(-a.y, a.x); }

// acc += i a b (4 FMA)
__device__ __forceinline__ double2 cfma_i(double2 a, double2 b, double2 acc) {
  acc.x = fma(-a.x, b.y, acc.x);
  acc.x = fma(-a.y, b.x, acc.x);
  acc.y = fma(a.x, b.x, acc.y);
  acc.y = fma(-a.y, b.y, acc.y);
  return acc;
}

// 32-lane latency transforms: the (orbital, pass) work units are one warp's
// team each, fine enough to balance over the CTA's warps
constexpr int kAdjPlan = 1;

template <int N>
struct SmallAdjLayout {
  static constexpr int PW = Team<N, kAdjPlan>::PER_WARP;
  static constexpr int NTEAM = kAdjWarps * PW;
  static constexpr int PASS_TEAMS = 3 * PW;    // orbitals b per round of warps 0..5 (host estimate)
  static constexpr int NSUB = (kAdjThreads / N) < 4 ? (kAdjThreads / N) : 4;
  // tw[N], bufs[NTEAM][N], F[N] (double2); vloc[N], psi[N], slices[2][NSUB][N] (double)
  static constexpr size_t bytes =
      sizeof(double2) * (size_t)N * (2 + NTEAM) + sizeof(double) * (size_t)N * (2 + 2 * NSUB);
};

template <int N>
__global__ void __launch_bounds__(kAdjThreads) k_small_adj(SmallAdjArgs a) {
  using TM = Team<N, kAdjPlan>;
  using L = SmallAdjLayout<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NSUB = L::NSUB;
  extern __shared__ double2 sm3[];
  double2* tw_s = sm3;
  double2* bufs = tw_s + N;
  double2* F_s = bufs + L::NTEAM * N;
  double* vl_s = reinterpret_cast<double*>(F_s + N);
  double* ps_s = vl_s + N;
  double* dsl = ps_s + N;                  // [2][NSUB][N]: rho slices, then sigma slices
  __shared__ int last_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, team = warp * PW + lane / T;
  const int team_lane0 = (lane / T) * T;
  double2* buf = bufs + team * N;
  const int ncols = a.nk * a.nb;
  const int c = blockIdx.x / a.P;          // output column a = (ka, ba)
  const int chunk = blockIdx.x % a.P;
  const int ka = c / a.nb;
  const int M = ncols;
  // orbitals b of this CTA, in groups of PW (a warp's teams).  The column's
  // first CTA keeps warps 6 and 7 for the Hartree and kinetic work, so it takes
  // half the share of the others.
  const int G = (M + PW - 1) / PW;
  const int wsum = 1 + 2 * (a.P - 1);
  const int g0 = chunk == 0 ? 0 : (G * (2 * chunk - 1)) / wsum;
  const int g1 = chunk + 1 == a.P ? G : (G * (2 * chunk + 1)) / wsum;
  const int b0 = g0 * PW, b1 = min(M, g1 * PW);
  const int workers = chunk == 0 ? kAdjWarps - 2 : kAdjWarps;
  double2* rv_g = a.part + (size_t)ncols * a.P * N + (size_t)c * N;         // (vloc, psi)
  double2* kin_g = a.part + (size_t)ncols * (a.P + 1) * N + (size_t)c * N;  // T_A mu_a

  for (int i = tid; i < N; i += kAdjThreads) tw_s[i] = a.tw[i];
  // programmatic dependent launch: only constant tables above this line
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;");
  const size_t elems = (size_t)ncols * N;
  const double2* v = a.store + ((size_t)(*a.n - *a.seg0) * 4 + a.slot) * elems;
  const double2* vA = v + (size_t)c * N;
  const double2* mA = a.mu + (size_t)c * N;
  if (chunk == 0 && tid < NSUB * N) {
    // density slices (ik -> ib order within a slice): rho without the uniform
    // occupation, and sigma
    const int ig = tid % N, j = tid / N;
    const int per = (M + NSUB - 1) / NSUB;
    const int q1 = min(M, (j + 1) * per);
    double sr = 0.0, ss = 0.0;
#pragma unroll 4
    for (int p = j * per; p < q1; ++p) {
      const double2 z = v[(size_t)p * N + ig], m = a.mu[(size_t)p * N + ig];
      sr = fma(z.y, z.y, fma(z.x, z.x, sr));
      ss = fma(m.x, z.y, fma(-m.y, z.x, ss));
    }
    dsl[j * N + ig] = sr;
    dsl[(NSUB + j) * N + ig] = ss;
  }
  __syncthreads();
  if (warp == kAdjWarps - 2) {
    if (chunk == 0) {
      double2 x[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int q = TM::pos(tl, e);
        double r = dsl[q], s = dsl[NSUB * N + q];
#pragma unroll
        for (int j = 1; j < NSUB; ++j) {
          r += dsl[j * N + q];
          s += dsl[(NSUB + j) * N + q];
        }
        x[e] = make_double2(a.occ * r, s);
        if (c == 0 && lane < T) a.gvion[q] += s;  // once per stage
      }
      fft_team<N, -1, kAdjPlan>(x, buf, tw_s, tl);
      fft_team_in<N, +1, kAdjPlan>(InScaled<N, kAdjPlan>{x, a.vCG, tl}, x, buf, tw_s, tl);
      if (lane < T) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          vl_s[q] = x[e].x / (double)N + a.vion[q];
          ps_s[q] = x[e].y / (double)N;
        }
      }
    }
  } else if (warp == kAdjWarps - 1) {
    if (chunk == 0) {
      double2 x[E], vf[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        x[e] = mA[TM::pos(tl, e)];
        vf[e] = vA[TM::pos(tl, e)];
      }
      fft_team<N, -1, kAdjPlan>(x, buf, tw_s, tl);
      fft_team<N, -1, kAdjPlan>(vf, buf, tw_s, tl);
      const double A = afield_value(a.af);
      const double kAx = a.kx[ka] + A, kA2 = kAx * kAx;
      double gp = 0.0;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const double G = a.Gx[TM::pos(tl, e)];
        gp += (G + a.kx[ka] + A) * (x[e].x * vf[e].y - x[e].y * vf[e].x);
        const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
        x[e] = make_double2(m * x[e].x / (double)N, m * x[e].y / (double)N);
      }
      gp = team_sum<T>(gp) / (double)N;
      fft_team<N, +1, kAdjPlan>(x, buf, tw_s, tl);
      if (lane < T) {
#pragma unroll
        for (int e = 0; e < E; ++e) kin_g[TM::pos(tl, e)] = x[e];
      }
      if (lane == 0) a.gcol[c] = gp;
    }
  }
  if (warp < workers) {
    // adjoint exchange of column a: unit u = (group u/2 of PW orbitals b,
    // pass u%2), dealt round-robin over the worker warps; the pass is uniform
    // over a warp in each round
    double2 acc[E];
#pragma unroll
    for (int e = 0; e < E; ++e) acc[e] = make_double2(0.0, 0.0);
    const int units = 2 * (g1 - g0);
    for (int u = warp; u < units; u += workers) {
      const bool passB = (u & 1) != 0;
      const int b = b0 + (u >> 1) * PW + lane / T;
      const bool valid = b < b1;
      const int bb = valid ? b : b0;
      const int kb = bb / a.nb;
      const double2* vB = v + (size_t)bb * N;
      const double2* mB = a.mu + (size_t)bb * N;
      const double* kab = a.kern + (size_t)(ka - kb + a.nk - 1) * N;
      double2 x[E];
      double n2x = 0.0, n2y = 0.0;   // pass B: Nyq(v_a conj(mu_b))
      if (!passB) {
        fft_team_in<N, -1, kAdjPlan>(InConjProduct<N, kAdjPlan>{vA, vB, tl}, x, buf, tw_s, tl);
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          const double sg = (q & 1) ? -1.0 : 1.0;
          // mu_a conj(v_b) - v_a conj(mu_b)
          const double2 t = cmulc(mA[q], vB[q]), t2 = cmulc(vA[q], mB[q]);
          x[e] = csub(t, t2);
          n2x = fma(sg, t2.x, n2x);
          n2y = fma(sg, t2.y, n2y);
        }
        n2x = team_sum<T>(n2x);
        n2y = team_sum<T>(n2y);
        fft_team<N, -1, kAdjPlan>(x, buf, tw_s, tl);
      }
      // Nyquist coefficient (pass A) in slot (p=0, r=R0/2) of the team's lane 0
      const double rnx = __shfl_sync(0xffffffffu, x[TM::R0 / 2].x, team_lane0);
      const double rny = __shfl_sync(0xffffffffu, x[TM::R0 / 2].y, team_lane0);
      fft_team_in<N, +1, kAdjPlan>(InScaled<N, kAdjPlan>{x, kab, tl}, x, buf, tw_s, tl);
      if (valid) {
        if (!passB) {
          const double dk = __ldg(a.kern + (size_t)(kb - ka + a.nk - 1) * N + N / 2) - __ldg(kab + N / 2);
          const double cx = dk * rnx, cy = dk * rny;
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int q = TM::pos(tl, e);
            const double sg = (q & 1) ? -1.0 : 1.0;
            const double2 pr = make_double2(fma(sg, cx, x[e].x), fma(sg, cy, x[e].y));
            acc[e] = cfma_i(pr, mB[q], acc[e]);
          }
        } else {
          const double dk = __ldg(a.kern + (size_t)(kb - ka + a.nk - 1) * N + N / 2) - __ldg(kab + N / 2);
          const double cx = dk * n2x, cy = dk * n2y;
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int q = TM::pos(tl, e);
            const double sg = (q & 1) ? -1.0 : 1.0;
            const double2 y = make_double2(fma(-sg, cx, x[e].x), fma(-sg, cy, x[e].y));
            acc[e] = cfma_i(vB[q], y, acc[e]);
          }
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int e = 0; e < E; ++e) buf[TM::pos(tl, e)] = acc[e];
  }
  __syncthreads();
  // this CTA's partial (pair teams in order) -> part[c][chunk]; the first CTA
  // also publishes (vloc, psi)
  double2* mine = a.part + ((size_t)c * a.P + chunk) * N;
  const int pair_teams = workers * PW;
  for (int i = tid; i < N; i += kAdjThreads) {
    double2 f = bufs[i];
    for (int t2 = 1; t2 < pair_teams; ++t2) f = cadd(f, bufs[(size_t)t2 * N + i]);
    mine[i] = f;
    if (chunk == 0) rv_g[i] = make_double2(vl_s[i], ps_s[i]);
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned t = atomicAdd(a.ticket + 1 + c, 1u);
    last_s = (t == (unsigned)a.P - 1) ? 1 : 0;
    if (last_s) {
      __threadfence();      // acquire: the other CTAs' partials, read below through L2
      a.ticket[1 + c] = 0u;
    }
  }
  __syncthreads();
  if (!last_s) return;
  // ---- the last CTA of column a: ordered sum of the P partials, bookkeeping
  const double2* cp = a.part + (size_t)c * a.P * N;
  for (int q = tid; q < N; q += kAdjThreads) {
    double2 f = __ldcg(cp + q);
    for (int ch = 1; ch < a.P; ++ch) f = cadd(f, __ldcg(cp + (size_t)ch * N + q));
    const double2 rv = __ldcg(rv_g + q);     // written by the column's first CTA
    const double2 kin = __ldcg(kin_g + q);
    const size_t o = (size_t)c * N + q;
    const double2 mu = mA[q], vv = vA[q];
    double2 lu = times_i(make_double2(kin.x + rv.x * mu.x, kin.y + rv.x * mu.y));
    lu = cadd(lu, f);
    const double ps = 2.0 * a.occ * rv.y;
    lu = make_double2(fma(ps, vv.x, lu.x), fma(ps, vv.y, lu.y));
    const double2 nu = cadd(a.lam_u[o], lu);
    a.lam_u[o] = nu;
    if (a.lam_prev) {
      const double2 p = a.lam_prev[o];
      a.lam_prev[o] = make_double2(fma(a.cprev, lu.x, p.x), fma(a.cprev, lu.y, p.y));
    }
    if (a.slot == 0) a.lam[o] = nu;
  }
  // ---- the last column: ordered field-gradient sum (the partials were
  // published before each column's ticket)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned t = atomicAdd(a.ticket, 1u);
    if (t == (unsigned)ncols - 1) {
      __threadfence();
      double g = 0.0;
      for (int i = 0; i < ncols; ++i) g += __ldcg(a.gcol + i);
      const int n = *a.n;
      a.gstage[(size_t)n * 4 + a.slot] = g;
      if (a.slot == 0) *a.n = n - 1;
      *a.ticket = 0u;
    }
  }
}

template <int N>
cudaError_t small_adj_impl(const SmallAdjArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nk * a.nb * a.P);
  cfg.blockDim = dim3(kAdjThreads);
  cfg.dynamicSmemBytes = SmallAdjLayout<N>::bytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_small_adj<N>, a);
}

template <int N>
cudaError_t small_adj_configure() {
  return cudaFuncSetAttribute(k_small_adj<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)SmallAdjLayout<N>::bytes);
}

}  // namespace

int small_adj_pair_warps_teams(int NG) {
  switch (NG) {
    case 16: return SmallAdjLayout<16>::PASS_TEAMS;
    case 32: return SmallAdjLayout<32>::PASS_TEAMS;
    case 64: return SmallAdjLayout<64>::PASS_TEAMS;
    case 128: return SmallAdjLayout<128>::PASS_TEAMS;
    case 256: return SmallAdjLayout<256>::PASS_TEAMS;
    default: return 0;
  }
}

cudaError_t launch_small_adj(int NG, const SmallAdjArgs& a, cudaStream_t s) {
  if (a.P < 1) return cudaErrorInvalidValue;
  switch (NG) {
    case 16: return small_adj_impl<16>(a, s);
    case 32: return small_adj_impl<32>(a, s);
    case 64: return small_adj_impl<64>(a, s);
    case 128: return small_adj_impl<128>(a, s);
    case 256: return small_adj_impl<256>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t configure_small_adj_kernels() {
  cudaError_t e;
  if ((e = small_adj_configure<16>()) != cudaSuccess) return e;
  if ((e = small_adj_configure<32>()) != cudaSuccess) return e;
  if ((e = small_adj_configure<64>()) != cudaSuccess) return e;
  if ((e = small_adj_configure<128>()) != cudaSuccess) return e;
  return small_adj_configure<256>();
}

}  // namespace mattohf
