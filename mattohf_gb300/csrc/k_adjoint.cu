// Adjoint (reverse-mode) kernels of the RK4 real-time loop.
//
// No counterpart in the reference: the gradient of the absorbed energy or of
// the final current with respect to every sample of the vector potential.
// For the RK4 right-hand side f(v) = -i h[v](a) v of src/RT_calculation.f90:166-169
// (h from src/Functions.f90:187-209) the transposed Jacobian, for the real
// inner product <x,y> = Re sum conj(x) y, is (all bands occupied)
//   J^T mu = i h[v](a) mu                                  kinetic, local, exchange at fixed v
//          + 2 occ vH[sigma] v,  sigma = sum Im(conj(mu) v)  Hartree response
//          + i sum_j conj(phi_ji) mu_j                      exchange: dependence through the source orbital
//          + i sum_j v_j (Phi_ij[mu_i conj(v_j)] - Phi~_ji[v_i conj(mu_j)])   (the i VF mu term folded in)
// with phi_ij = Phi_ij[v_i conj(v_j)] the pair potentials of the forward step.
// Phi~_ji, the transpose of dv_j -> Phi_ij[v_i conj(dv_j)], has the multiplier
// kern_ji(-G): that is kern_ij(G) (v is even) except at the self-aliased
// Nyquist index N/2, where it stays kern_ji.  So
//   Phi~_ji[f] = Phi_ij[f] + dk_ij Nyq(f) (-1)^m,  dk_ij = kern_ji[N/2] - kern_ij[N/2],
// Nyq(f) = sum_m (-1)^m f(m) the Nyquist coefficient of the forward transform.
// k_fock_adj evaluates the two exchange sums over unordered occupied pairs
// with two transform pairs per pair (pair densities v_i conj(v_j) and
// mu_i conj(v_j) - v_i conj(mu_j)), using the same conjugate-plus-Nyquist
// relation as the forward symmetric kernel.
#include "fft.cuh"
#include "internal.h"

namespace mattohf {

__device__ __forceinline__ double2 mul_i(double2 a) { return make_double2(-a.y, a.x); }

template <int N>
__global__ void __launch_bounds__(kThreads) k_fock_adj(AdjFockArgs a) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  const int S = a.S;
  const int nteam = (blockDim.x >> 5) * PW;
  extern __shared__ double2 sm[];
  double2* tw_s = sm;
  double2* bufs = sm + N;
  double2* cacc = bufs + nteam * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, tw_ = warp * PW + lane / T;
  const int team_lane0 = (lane / T) * T;
  double2* buf = bufs + tw_ * N;
  for (int i = tid; i < N; i += blockDim.x) tw_s[i] = a.tw[i];
  for (int i = tid; i < S * N; i += blockDim.x) cacc[i] = make_double2(0.0, 0.0);
  int ti = 0, rem = blockIdx.x;
  while (rem >= a.T - ti) { rem -= a.T - ti; ++ti; }
  const int tj = ti + rem;
  const int M = a.nk * a.nbocc;
  const int ia = ti * S + tw_;
  const bool va = tw_ < S && ia < M;
  const int ka = (va ? ia : 0) / a.nbocc, ba = (va ? ia : 0) % a.nbocc;
  const size_t oa = (size_t)ka * a.kstride + (size_t)ba * N;
  // orbitals and adjoints are re-read (L1/L2) where needed instead of held in
  // registers (the kernel is FP64-pipe bound; this avoids spills at NG=512)
  const double2* vA = a.v + oa;
  const double2* mA = a.mu + oa;
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
    if (diag && (S % 2 == 0) && r == S / 2 && tw_ >= S / 2) valid = false;
    const bool self = diag && r == 0;
    const int kb = (ib < M ? ib : 0) / a.nbocc, bb = (ib < M ? ib : 0) % a.nbocc;
    const size_t ob = (size_t)kb * a.kstride + (size_t)bb * N;
    const int dab = ka - kb + a.nk - 1, dba = kb - ka + a.nk - 1;
    const double* kab = a.kern + (size_t)dab * N;
    const double dk = __ldg(a.kern + (size_t)dba * N + N / 2) - __ldg(kab + N / 2);
    const double2* vB = a.v + ob;
    const double2* mB = a.mu + ob;
    double2 x[E];
    // ---- pass A: phi_ab = Phi_ab[v_a conj(v_b)]
    fft_team_in<N, -1>(InConjProduct<N>{vA, vB, tl}, x, buf, tw_s, tl);
    const double rnx = __shfl_sync(0xffffffffu, x[TM::R0 / 2].x, team_lane0);
    const double rny = __shfl_sync(0xffffffffu, x[TM::R0 / 2].y, team_lane0);
    fft_team_in<N, +1>(InScaled<N>{x, kab, tl}, x, buf, tw_s, tl);
    if (valid) {
      if (self) {
        // out_a += i conj(phi_aa) mu_a
#pragma unroll
        for (int e = 0; e < E; ++e)
          racc[e] = cadd(racc[e], mul_i(cmul(make_double2(x[e].x, -x[e].y), mA[TM::pos(tl, e)])));
      } else {
        // c = dk * conj(R); out_a += i (phi_ab + conj(c)(-1)^m) mu_b ; out_b += i conj(phi_ab) mu_a
        const double cx = dk * rnx, cy = -dk * rny;
        double2* col = cacc + lb * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          const double sg = (q & 1) ? -1.0 : 1.0;
          const double2 pr = make_double2(fma(sg, cx, x[e].x), fma(-sg, cy, x[e].y));
          racc[e] = cadd(racc[e], mul_i(cmul(pr, mB[q])));
          col[q] = cadd(col[q], mul_i(cmul(make_double2(x[e].x, -x[e].y), mA[q])));
        }
      }
    }
    // ---- pass B: phi'_ab = Phi_ab[mu_a conj(v_b) - v_a conj(mu_b)], and
    //      n2 = Nyq(v_a conj(mu_b)) for the transposed operator's Nyquist term
    double n2x = 0.0, n2y = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int q = TM::pos(tl, e);
      const double sg = (q & 1) ? -1.0 : 1.0;
      const double2 t2 = cmulc(vA[q], mB[q]);
      x[e] = csub(cmulc(mA[q], vB[q]), t2);
      n2x = fma(sg, t2.x, n2x);
      n2y = fma(sg, t2.y, n2y);
    }
    n2x = team_sum<T>(n2x);
    n2y = team_sum<T>(n2y);
    fft_team<N, -1>(x, buf, tw_s, tl);
    fft_team_in<N, +1>(InScaled<N>{x, kab, tl}, x, buf, tw_s, tl);
    if (valid) {
      // y = Phi_ab[mu_a conj(v_b)] - Phi~_ba[v_a conj(mu_b)] = phi'_ab - dk n2 (-1)^m;
      // out_a += i v_b y.  The pair's reversed term is its mirror image:
      // Phi_ba[mu_b conj(v_a)] - Phi~_ab[v_b conj(mu_a)] = -conj(y), so
      // out_b += i v_a (-conj(y)).  (dk = 0 on the diagonal.)
      const double cx = dk * n2x, cy = dk * n2y;
      double2* col = cacc + lb * N;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int q = TM::pos(tl, e);
        const double sg = (q & 1) ? -1.0 : 1.0;
        const double2 y = make_double2(fma(-sg, cx, x[e].x), fma(-sg, cy, x[e].y));
        racc[e] = cadd(racc[e], mul_i(cmul(vB[q], y)));
        if (!self) col[q] = cadd(col[q], mul_i(cmul(vA[q], make_double2(-y.x, y.y))));
      }
    }
    __syncthreads();
  }
  double2* dst = a.scratch + (size_t)blockIdx.x * 2 * S * N;
  if (tw_ < S) {
#pragma unroll
    for (int e = 0; e < E; ++e) dst[(size_t)tw_ * N + TM::pos(tl, e)] = racc[e];
  }
  for (int i = tid; i < S * N; i += blockDim.x) dst[(size_t)S * N + i] = cacc[i];
}

// Adjoint combine of one RK4 stage, one team per column:
//   lu   = i (T_a + vloc) mu + Fa + 2 occ psi v
//   g_a += sum_G (G+k+a) Im(conj(FFT mu) FFT v) / N     (field gradient partial)
//   lam_u += lu ; lam_prev += c_prev * lu               (RK4 stage bookkeeping)
template <int N>
__global__ void __launch_bounds__(kThreads) k_adj_combine(AdjCombineArgs a, int ncols) {
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
  const int col0 = (blockIdx.x * (kThreads / 32) + warp) * PW;
  if (col0 >= ncols) return;
  const int col = col0 + lane / T;
  const bool valid = col < ncols;
  const int c = valid ? col : col0;
  const int ik = c / a.nb;
  const size_t o = (size_t)c * N;
  if (a.split == 2) {
    if (!valid) return;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int q = TM::pos(tl, e);
      double2 lu = cadd(a.lpre[o + q], a.Fa[o + q]);
      const double ps = 2.0 * a.occ * a.psi[q];
      const double2 vv = a.v[o + q];
      lu = make_double2(fma(ps, vv.x, lu.x), fma(ps, vv.y, lu.y));
      a.lam_u[o + q] = cadd(a.lam_u[o + q], lu);
      if (a.lam_prev) {
        const double2 p = a.lam_prev[o + q];
        a.lam_prev[o + q] = make_double2(fma(a.cprev, lu.x, p.x), fma(a.cprev, lu.y, p.y));
      }
    }
    return;
  }
  double2 mu[E], v[E], x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int q = TM::pos(tl, e);
    mu[e] = a.mu[o + q];
    v[e] = a.v[o + q];
    x[e] = mu[e];
  }
  fft_team<N, -1>(x, bufs[team], tw_s, tl);
  // field-gradient partial needs FFT(v) too
  double2 vf[E];
#pragma unroll
  for (int e = 0; e < E; ++e) vf[e] = v[e];
  fft_team<N, -1>(vf, bufs[team], tw_s, tl);
  const double kAx = a.kx[ik] + A, kA2 = kAx * kAx;
  double gp = 0.0;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const double G = a.Gx[TM::pos(tl, e)];
    gp += (G + a.kx[ik] + A) * (x[e].x * vf[e].y - x[e].y * vf[e].x);
    const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
    x[e] = make_double2(m * x[e].x / (double)N, m * x[e].y / (double)N);
  }
  gp = team_sum<T>(gp) / (double)N;
  fft_team<N, +1>(x, bufs[team], tw_s, tl);
  if (valid && tl == 0) a.gcol[c] = gp;
  if (!valid) return;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int q = TM::pos(tl, e);
    const double vl = a.vloc[q];
    double2 lu = mul_i(make_double2(x[e].x + vl * mu[e].x, x[e].y + vl * mu[e].y));
    if (a.split == 1) {
      a.lpre[o + q] = lu;
      continue;
    }
    lu = cadd(lu, a.Fa[o + q]);
    const double ps = 2.0 * a.occ * a.psi[q];
    lu = make_double2(fma(ps, v[e].x, lu.x), fma(ps, v[e].y, lu.y));
    a.lam_u[o + q] = cadd(a.lam_u[o + q], lu);
    if (a.lam_prev) {
      const double2 p = a.lam_prev[o + q];
      a.lam_prev[o + q] = make_double2(fma(a.cprev, lu.x, p.x), fma(a.cprev, lu.y, p.y));
    }
  }
}

// Ordered sum of the per-column field-gradient partials into g[slot].
__global__ void k_adj_gsum(const double* __restrict__ gcol, int ncols, double* g, const int* n, int s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = 0.0;
  for (int i = 0; i < ncols; ++i) acc += gcol[i];
  g[(size_t)(*n) * 4 + s] = acc;
}

// lam_k[s] = w_s lam (w = dt/6, dt/3, dt/3, dt/6); lam_u = lam.
__global__ void k_adj_init(const double2* __restrict__ lam, double2* lam_u, double2* k0, double2* k1,
                           double2* k2, double2* k3, double dt, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 l = lam[i];
  const double w6 = dt / 6.0, w3 = dt / 3.0;
  lam_u[i] = l;
  k0[i] = make_double2(w6 * l.x, w6 * l.y);
  k1[i] = make_double2(w3 * l.x, w3 * l.y);
  k2[i] = make_double2(w3 * l.x, w3 * l.y);
  k3[i] = make_double2(w6 * l.x, w6 * l.y);
}

// dst = store[(n - seg0) * 4 + slot]  (or the reverse with `to_store`)
__global__ void k_stage_copy(double2* dst, const double2* src, double2* store, const int* n,
                             const int* seg0, int slot, size_t elems, int to_store) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= elems) return;
  const size_t base = ((size_t)(*n - *seg0) * 4 + slot) * elems;
  if (to_store) store[base + i] = src[i];
  else dst[i] = store[base + i];
}

// checkpoint u every `every` steps: ckpt[it / every] = u when it % every == 0
// Checkpoint j holds the state at the start of segment j; segments start at
// step 0 and at every t with (t + phase) % every == 0.
__global__ void k_checkpoint(double2* ckpt, const double2* u, const int* it, int every, int phase, size_t elems) {
  const int t = *it;
  if (t != 0 && (t + phase) % every != 0) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < elems) ckpt[(size_t)((t + phase) / every) * elems + i] = u[i];
}

__global__ void k_counter_add(int* p, int d) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p += d;
}

// out = scale * P_A u, P_A = IFFT((G+k+A) FFT(.)/N)  (the operator of ubk_Je, F:306-310)
template <int N>
__global__ void __launch_bounds__(kThreads) k_velocity(const double2* __restrict__ u, double2* out,
                                                       const double2* __restrict__ tw,
                                                       const double* __restrict__ Gx,
                                                       const double* __restrict__ kx, int nb, double A,
                                                       double scale, int ncols) {
  using TM = Team<N>;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  constexpr int NTEAM = (kThreads / 32) * PW;
  __shared__ double2 tw_s[N];
  __shared__ double2 bufs[NTEAM][N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, team = warp * PW + lane / T;
  for (int i = tid; i < N; i += kThreads) tw_s[i] = tw[i];
  __syncthreads();
  const int col0 = (blockIdx.x * (kThreads / 32) + warp) * PW;
  if (col0 >= ncols) return;
  const int col = col0 + lane / T;
  const bool valid = col < ncols;
  const int c = valid ? col : col0;
  const int ik = c / nb;
  double2 x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) x[e] = u[(size_t)c * N + TM::pos(tl, e)];
  fft_team<N, -1>(x, bufs[team], tw_s, tl);
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const double g = Gx[TM::pos(tl, e)] + kx[ik] + A;
    x[e] = make_double2(g * (x[e].x / (double)N), g * (x[e].y / (double)N));
  }
  fft_team<N, +1>(x, bufs[team], tw_s, tl);
  if (!valid) return;
#pragma unroll
  for (int e = 0; e < E; ++e)
    out[(size_t)c * N + TM::pos(tl, e)] = make_double2(scale * x[e].x, scale * x[e].y);
}

__global__ void k_scale2(double2* x, double s, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = make_double2(s * x[i].x, s * x[i].y);
}

// ---------------------------------------------------------------------------
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

template <int N>
static size_t adj_smem() { return sizeof(double2) * (size_t)N * (1 + 2 * (kThreads / 32) * Team<N>::PER_WARP); }

template <int N>
static cudaError_t fock_adj_impl(const AdjFockArgs& a, cudaStream_t s) {
  const int tiles = a.T * (a.T + 1) / 2;
  if (tiles == 0) return cudaSuccess;
  int threads;
  size_t smem;
  cudaError_t e = sym_launch_params(N, a.S, &threads, &smem);
  if (e != cudaSuccess) return e;
  k_fock_adj<N><<<tiles, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
static cudaError_t configure_adj_impl() {
  return cudaFuncSetAttribute(k_fock_adj<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_smem<N>());
}

cudaError_t configure_adjoint_kernels() {
  cudaError_t e;
  if ((e = configure_adj_impl<16>()) != cudaSuccess) return e;
  if ((e = configure_adj_impl<32>()) != cudaSuccess) return e;
  if ((e = configure_adj_impl<64>()) != cudaSuccess) return e;
  if ((e = configure_adj_impl<128>()) != cudaSuccess) return e;
  if ((e = configure_adj_impl<256>()) != cudaSuccess) return e;
  return configure_adj_impl<512>();
}

cudaError_t launch_fock_adj(int NG, const AdjFockArgs& a, cudaStream_t s) {
#define CALL(n) fock_adj_impl<n>(a, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

template <int N>
static cudaError_t adj_combine_impl(const AdjCombineArgs& a, int ncols, cudaStream_t s) {
  constexpr int PER_CTA = (kThreads / 32) * Team<N>::PER_WARP;
  k_adj_combine<N><<<(ncols + PER_CTA - 1) / PER_CTA, kThreads, 0, s>>>(a, ncols);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || a.split == 2) return e;  // the field-gradient partials come from the other passes
  k_adj_gsum<<<1, 32, 0, s>>>(a.gcol, ncols, a.gstage, a.n, a.slot);
  return cudaGetLastError();
}

cudaError_t launch_adj_combine(int NG, const AdjCombineArgs& a, int ncols, cudaStream_t s) {
#define CALL(n) adj_combine_impl<n>(a, ncols, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_adj_init(const double2* lam, double2* lam_u, double2* const* lamk, double dt, size_t n,
                            cudaStream_t s) {
  k_adj_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lam, lam_u, lamk[0], lamk[1], lamk[2], lamk[3], dt, n);
  return cudaGetLastError();
}

cudaError_t launch_stage_copy(double2* dst, const double2* src, double2* store, const int* n, const int* seg0,
                              int slot, size_t elems, int to_store, cudaStream_t s) {
  k_stage_copy<<<(unsigned)((elems + 255) / 256), 256, 0, s>>>(dst, src, store, n, seg0, slot, elems, to_store);
  return cudaGetLastError();
}

cudaError_t launch_checkpoint(double2* ckpt, const double2* u, const int* it, int every, int phase, size_t elems,
                              cudaStream_t s) {
  k_checkpoint<<<(unsigned)((elems + 255) / 256), 256, 0, s>>>(ckpt, u, it, every, phase, elems);
  return cudaGetLastError();
}

cudaError_t launch_counter_add(int* p, int d, cudaStream_t s) {
  k_counter_add<<<1, 32, 0, s>>>(p, d);
  return cudaGetLastError();
}

template <int N>
static cudaError_t velocity_impl(const double2* u, double2* out, const double2* tw, const double* Gx,
                                 const double* kx, int nb, double A, double scale, int ncols, cudaStream_t s) {
  constexpr int PER_CTA = (kThreads / 32) * Team<N>::PER_WARP;
  k_velocity<N><<<(ncols + PER_CTA - 1) / PER_CTA, kThreads, 0, s>>>(u, out, tw, Gx, kx, nb, A, scale, ncols);
  return cudaGetLastError();
}

cudaError_t launch_velocity(int NG, const double2* u, double2* out, const double2* tw, const double* Gx,
                            const double* kx, int nb, double A, double scale, int ncols, cudaStream_t s) {
#define CALL(n) velocity_impl<n>(u, out, tw, Gx, kx, nb, A, scale, ncols, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_scale2(double2* x, double sc, size_t n, cudaStream_t s) {
  k_scale2<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, sc, n);
  return cudaGetLastError();
}

// Nyquist term of the exchange-energy gradient.  Ex = 1/2 occ dvcell
// sum_ij <p_ij, Phi_ij p_ij>, p_ij = u_i conj(u_j) (src/Functions.f90:165-183).
// Varying the conj(u_j) factor brings in conj(Phi_ij[p_ij]), which equals
// Phi_ji[p_ji] except at the self-aliased Nyquist index; so the gradient is
// 2 occ dvcell h[u] u plus, for column i,
//   g_i += sc sum_j (kern_ji - kern_ij)[N/2] Nyq(p_ij) (-1)^m u_j,
// Nyq(p) = sum_m (-1)^m p(m), sc = occ dvcell.  One CTA per column i; the
// orbitals j are visited in order, each dot product reduced in a fixed order.
constexpr int kNyqThreads = 256;
__global__ void __launch_bounds__(kNyqThreads) k_energy_grad_nyquist(const double2* __restrict__ u, double2* g,
                                                                      const double* __restrict__ kern, int N,
                                                                      int nk, int nb, double sc) {
  __shared__ double2 red[kNyqThreads / 32];
  const int i = blockIdx.x, ki = i / nb;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const double2* ui = u + (size_t)i * N;
  const int M = nk * nb;
  constexpr int kMaxPer = 512 / kNyqThreads;    // N <= 512
  double2 acc[kMaxPer];
#pragma unroll
  for (int r = 0; r < kMaxPer; ++r) acc[r] = make_double2(0.0, 0.0);
  for (int j = 0; j < M; ++j) {
    const int kj = j / nb;
    if (kj == ki) continue;   // the two multipliers coincide
    const double d = kern[(size_t)(kj - ki + nk - 1) * N + N / 2] - kern[(size_t)(ki - kj + nk - 1) * N + N / 2];
    const double2* uj = u + (size_t)j * N;
    double px = 0.0, py = 0.0;
    for (int m = tid; m < N; m += kNyqThreads) {
      const double sg = (m & 1) ? -1.0 : 1.0;
      const double2 t = cmulc(ui[m], uj[m]);
      px = fma(sg, t.x, px);
      py = fma(sg, t.y, py);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      px += __shfl_xor_sync(0xffffffffu, px, o);
      py += __shfl_xor_sync(0xffffffffu, py, o);
    }
    if (lane == 0) red[warp] = make_double2(px, py);
    __syncthreads();
    double2 c = red[0];
    for (int w = 1; w < kNyqThreads / 32; ++w) c = cadd(c, red[w]);
    __syncthreads();
    const double2 f = make_double2(sc * d * c.x, sc * d * c.y);
#pragma unroll
    for (int r = 0; r < kMaxPer; ++r) {
      const int m = tid + r * kNyqThreads;
      if (m < N) {
        const double sg = (m & 1) ? -1.0 : 1.0;
        const double2 t = cmul(f, uj[m]);
        acc[r] = make_double2(fma(sg, t.x, acc[r].x), fma(sg, t.y, acc[r].y));
      }
    }
  }
  double2* gi = g + (size_t)i * N;
#pragma unroll
  for (int r = 0; r < kMaxPer; ++r) {
    const int m = tid + r * kNyqThreads;
    if (m < N) gi[m] = cadd(gi[m], acc[r]);
  }
}

cudaError_t launch_energy_grad_nyquist(const double2* u, double2* g, const double* kern, int NG, int nk, int nb,
                                       double sc, cudaStream_t s) {
  if (NG > 512) return cudaErrorInvalidValue;
  k_energy_grad_nyquist<<<nk * nb, kNyqThreads, 0, s>>>(u, g, kern, NG, nk, nb, sc);
  return cudaGetLastError();
}

}  // namespace mattohf

namespace mattohf {

// Taylor-propagator update (RT:86-88, RT:110-117): w = -i c (h0 [+ h1]) / iorder ; acc += w
__global__ void k_te_update(double2* __restrict__ w, const double2* __restrict__ h0,
                            const double2* __restrict__ h1, double c, double iorder,
                            double2* __restrict__ acc, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 s = h0[i];
  if (h1) s = make_double2(s.x + h1[i].x, s.y + h1[i].y);
  const double2 v = make_double2((c * s.y) / iorder, (-c * s.x) / iorder);
  w[i] = v;
  const double2 a = acc[i];
  acc[i] = make_double2(a.x + v.x, a.y + v.y);
}

// out = 0.5 * (a + b)
__global__ void k_half_sum(double2* __restrict__ out, const double2* __restrict__ a,
                           const double2* __restrict__ b, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double2(0.5 * (a[i].x + b[i].x), 0.5 * (a[i].y + b[i].y));
}

cudaError_t launch_te_update(double2* w, const double2* h0, const double2* h1, double c, double iorder,
                             double2* acc, size_t n, cudaStream_t s) {
  k_te_update<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, h0, h1, c, iorder, acc, n);
  return cudaGetLastError();
}

cudaError_t launch_half_sum(double2* out, const double2* a, const double2* b, size_t n, cudaStream_t s) {
  k_half_sum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, a, b, n);
  return cudaGetLastError();
}

}  // namespace mattohf
