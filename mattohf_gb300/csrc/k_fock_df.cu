// Symmetric exchange (src/Functions.f90:237-261, w == u) with the pair
// transforms in double-float arithmetic (fft_df.cuh).
//
// Same tile-pair decomposition, Nyquist correction and partial-sum layout as
// k_fock_sym in k_hpsi.cu; only the arithmetic of the pair chain (pair
// density, forward transform, kernel, inverse transform, the two
// accumulations) runs on the FP32 pipe as unevaluated hi+lo pairs.  Inputs are
// converted from FP64 once per apply, the partial sums back to FP64 on the way
// out, so everything outside this kernel stays complex128.
#include "fft_df.cuh"
#include "internal.h"

namespace mattohf {

template <int N>
__device__ __forceinline__ void fock_sym_df_body(const FockSymDfArgs& a, const int tile) {
  using TM = Team<N>;
  using df::cdf;
  constexpr int E = TM::E, T = TM::T, PW = TM::PER_WARP;
  const int S = a.S;
  const int nteam = (blockDim.x >> 5) * PW;
  extern __shared__ float4 smf[];
  cdf* tw_s = reinterpret_cast<cdf*>(smf);        // N
  cdf* bufs = tw_s + N;                           // nteam * N
  cdf* cacc = bufs + nteam * N;                   // S * N
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tl = lane % T, tw_ = warp * PW + lane / T;
  const int team_lane0 = (lane / T) * T;
  cdf* buf = bufs + tw_ * N;
  for (int i = tid; i < N; i += blockDim.x) tw_s[i] = df::load(a.tw + i);
  for (int i = tid; i < S * N; i += blockDim.x) {
    cdf z;
    z.re = make_float2(0.f, 0.f);
    z.im = make_float2(0.f, 0.f);
    cacc[i] = z;
  }
  int ti = 0, rem = tile;
  while (rem >= a.T - ti) { rem -= a.T - ti; ++ti; }
  const int tj = ti + rem;
  const int M = a.nk * a.nbocc;
  const int ia = ti * S + tw_;
  const bool va = tw_ < S && ia < M;
  const int oa = va ? ia : 0;
  const int ka = oa / a.nbocc;
  // the row orbital is re-read from the (L1-resident) df copy where needed
  // instead of being held in registers, to keep three CTAs per SM
  const float4* ua_p = a.u + (size_t)oa * N;
  cdf racc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    racc[e].re = make_float2(0.f, 0.f);
    racc[e].im = make_float2(0.f, 0.f);
  }
  __syncthreads();
  const bool diag = (ti == tj);
  const int nrounds = diag ? (S / 2 + 1) : S;
  for (int r = 0; r < nrounds; ++r) {
    const int lb = (tw_ + r) % S;
    const int ib = tj * S + lb;
    bool valid = va && ib < M;
    if (diag && (S % 2 == 0) && r == S / 2 && tw_ >= S / 2) valid = false;
    const bool self = diag && r == 0;
    const int ob = ib < M ? ib : 0;
    const int kb = ob / a.nbocc;
    const int dab = ka - kb + a.nk - 1, dba = kb - ka + a.nk - 1;
    const float2* kab = a.kern + (size_t)dab * N;
    const float4* ub_p = a.u + (size_t)ob * N;
    cdf x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int q = TM::pos(tl, e);
      x[e] = df::cmulc(df::load(ua_p + q), df::load(ub_p + q));
    }
    // Both transforms run through ONE copy of the forward FFT code (the
    // kernel is instruction-cache bound): IFFT(y) = conj(FFT(conj(y))), so
    // after the second pass x = conj(phi_ab).
    cdf rn;
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      df::fft_team_compact<N>(x, buf, tw_s, tl);
      if (pass == 0) {
        const cdf rn_own = x[TM::R0 / 2];
        rn.re.x = __shfl_sync(0xffffffffu, rn_own.re.x, team_lane0);
        rn.re.y = __shfl_sync(0xffffffffu, rn_own.re.y, team_lane0);
        rn.im.x = __shfl_sync(0xffffffffu, rn_own.im.x, team_lane0);
        rn.im.y = __shfl_sync(0xffffffffu, rn_own.im.y, team_lane0);
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = df::conj(df::scale(x[e], kab[TM::pos(tl, e)]));
      }
    }
    if (valid) {
      // row: out_a += phi_ab u_b with phi_ab = conj(x)
#pragma unroll
      for (int e = 0; e < E; ++e)
        racc[e] = df::cadd(racc[e], df::cmul(df::conj(x[e]), df::load(ub_p + TM::pos(tl, e))));
      if (!self) {
        const float2 dk = df::sub(a.kern[(size_t)dba * N + N / 2], kab[N / 2]);
        // c = dk conj(R); phi_ba = conj(phi_ab) + c (-1)^m = x + c (-1)^m
        const float2 cx = df::mul(dk, rn.re), cy = df::neg(df::mul(dk, rn.im));
        cdf* col = cacc + lb * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int q = TM::pos(tl, e);
          const bool odd = q & 1;
          const cdf pba = df::make(df::add(x[e].re, odd ? df::neg(cx) : cx),
                                   df::add(x[e].im, odd ? df::neg(cy) : cy));
          col[q] = df::cadd(col[q], df::cmul(pba, df::load(ua_p + q)));
        }
      }
    }
    __syncthreads();
  }
  // partials stay double-float; k_sym_reduce_df sums them and converts once
  float4* dst = a.scratch + (size_t)tile * 2 * S * N;
  if (tw_ < S) {
#pragma unroll
    for (int e = 0; e < E; ++e) df::store(dst + (size_t)tw_ * N + TM::pos(tl, e), racc[e]);
  }
  for (int i = tid; i < S * N; i += blockDim.x) df::store(dst + (size_t)S * N + i, cacc[i]);
}

template <int N>
__global__ void __launch_bounds__(kThreads) k_fock_sym_df(FockSymDfArgs a) { fock_sym_df_body<N>(a, blockIdx.x); }

__device__ __forceinline__ int df_find_run(const int* __restrict__ pre, int nruns, int i) {
  int lo = 0, hi = nruns - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// many runs per launch: tile pairs of all runs, mapped through a prefix array
template <int N>
__global__ void __launch_bounds__(kThreads) k_fock_sym_df_batch(const FockSymDfArgs* __restrict__ args,
                                                              const int* __restrict__ pre, int nruns) {
  const int r = df_find_run(pre, nruns, blockIdx.x);
  fock_sym_df_body<N>(args[r], blockIdx.x - pre[r]);
}

// Ordered double-float sum of the tile partials of every occupied output,
// converted to FP64 once (same term order and runs as k_sym_reduce).
__device__ __forceinline__ df::cdf sym_run_sum_df(const float4* __restrict__ part, int S, int T, int N, int idx,
                                                  int c) {
  const int o = idx / N, q = idx % N;
  const int i = o / S, l = o % S;
  int t0, t1;
  sym_run_bounds(T, c, &t0, &t1);
  df::cdf f;
  f.re = make_float2(0.f, 0.f);
  f.im = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int t = t0; t < t1; ++t) f = df::cadd(f, df::load(part + sym_term(t, i, l, q, S, T, N)));
  return f;
}

__device__ __forceinline__ void sym_reduce_finish_df(const df::cdf& f, bool valid, double2* __restrict__ out) {
  __shared__ df::cdf red[kRedQ][kRedE];
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  red[c][e] = f;
  __syncthreads();
  if (c == 0 && valid) {
    df::cdf s = red[0][e];
#pragma unroll
    for (int k = 1; k < kRedQ; ++k) s = df::cadd(s, red[k][e]);
    *out = df::to_double2(s);
  }
}

__global__ void __launch_bounds__(kRedQ* kRedE) k_sym_reduce_df(const float4* __restrict__ part, int S, int T,
                                                                int M, int N, double2* __restrict__ F) {
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  const int idx = blockIdx.x * kRedE + e;
  const bool valid = idx < M * N;
  df::cdf f;
  f.re = make_float2(0.f, 0.f);
  f.im = make_float2(0.f, 0.f);
  if (valid) f = sym_run_sum_df(part, S, T, N, idx, c);
  sym_reduce_finish_df(f, valid, F + (valid ? idx : 0));
}

__global__ void __launch_bounds__(kRedQ* kRedE) k_sym_reduce_df_batch(const FockSymDfArgs* __restrict__ args,
                                                                      const int* __restrict__ pre, int nruns,
                                                                      int N) {
  const int e = threadIdx.x % kRedE, c = threadIdx.x / kRedE;
  const int idx = blockIdx.x * kRedE + e;
  const bool valid = idx < pre[nruns];
  df::cdf f;
  f.re = make_float2(0.f, 0.f);
  f.im = make_float2(0.f, 0.f);
  double2* out = nullptr;
  if (valid) {
    const int r = df_find_run(pre, nruns, idx);
    const FockSymDfArgs& a = args[r];
    f = sym_run_sum_df(a.scratch, a.S, a.T, N, idx - pre[r], c);
    out = a.F + (idx - pre[r]);
  }
  sym_reduce_finish_df(f, valid, out);
}

// df copies of every run's occupied orbitals (element prefix as for the reduction)
__global__ void k_orb_to_df_batch(const FockSymArgs* __restrict__ src, const FockSymDfArgs* __restrict__ dst,
                                  const int* __restrict__ pre, int nruns, int N) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= pre[nruns]) return;
  const int r = df_find_run(pre, nruns, idx);
  const int i = idx - pre[r];
  const FockSymArgs& s = src[r];
  const int o = i / N, g = i % N;
  const int k = o / s.nbocc, b = o % s.nbocc;
  df::store(const_cast<float4*>(dst[r].u) + i, df::from_double2(s.u.p[(size_t)k * s.u.kstride + (size_t)b * N + g]));
}

// occupied orbitals (FP64, [NK][NB][NG]) -> df copy [NK*NBocc][NG]
__global__ void k_orb_to_df(const double2* __restrict__ u, int kstride, int nbocc, int N, int total,
                            float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int o = i / N, g = i % N;
  const int k = o / nbocc, b = o % nbocc;
  df::store(out + i, df::from_double2(u[(size_t)k * kstride + (size_t)b * N + g]));
}

__global__ void k_real_to_df(const double* __restrict__ x, int n, float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = df::from_double(x[i]);
}

__global__ void k_cplx_to_df(const double2* __restrict__ x, int n, float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) df::store(out + i, df::from_double2(x[i]));
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

template <int N>
static cudaError_t fock_df_impl(const FockSymDfArgs& a, const double2* u, int kstride, float4* udf,
                                cudaStream_t s) {
  const int M = a.nk * a.nbocc;
  const int total = M * N;
  k_orb_to_df<<<(total + 255) / 256, 256, 0, s>>>(u, kstride, a.nbocc, N, total, udf);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int tiles = a.T * (a.T + 1) / 2;
  if (tiles == 0) return cudaSuccess;
  int threads;
  size_t smem;
  if ((e = sym_launch_params(N, a.S, &threads, &smem)) != cudaSuccess) return e;
  k_fock_sym_df<N><<<tiles, threads, smem, s>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_sym_reduce_df<<<(M * N + kRedE - 1) / kRedE, kRedQ * kRedE, 0, s>>>(a.scratch, a.S, a.T, M, N, a.F);
  return cudaGetLastError();
}

template <int N>
static cudaError_t fock_df_batch_impl(const FockSymArgs* d_src, const FockSymDfArgs* d_args, const int* d_tile_pre,
                                      int nruns, int total_tiles, const int* d_elem_pre, int total_elems,
                                      cudaStream_t s) {
  k_orb_to_df_batch<<<(total_elems + 255) / 256, 256, 0, s>>>(d_src, d_args, d_elem_pre, nruns, N);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || total_tiles <= 0) return e;
  constexpr int NTEAM = (kThreads / 32) * Team<N>::PER_WARP;
  const size_t smem = sizeof(float4) * (size_t)N * (1 + 2 * NTEAM);
  k_fock_sym_df_batch<N><<<total_tiles, kThreads, smem, s>>>(d_args, d_tile_pre, nruns);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_sym_reduce_df_batch<<<(total_elems + kRedE - 1) / kRedE, kRedQ * kRedE, 0, s>>>(d_args, d_elem_pre, nruns,
                                                                                     N);
  return cudaGetLastError();
}

cudaError_t launch_fock_sym_df_batch(int NG, const FockSymArgs* d_src, const FockSymDfArgs* d_args,
                                     const int* d_tile_pre, int nruns, int total_tiles, const int* d_elem_pre,
                                     int total_elems, cudaStream_t s) {
#define CALL(n) fock_df_batch_impl<n>(d_src, d_args, d_tile_pre, nruns, total_tiles, d_elem_pre, total_elems, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

cudaError_t launch_fock_sym_df(int NG, const FockSymDfArgs& a, const double2* u, int kstride, float4* udf,
                               cudaStream_t s) {
#define CALL(n) fock_df_impl<n>(a, u, kstride, udf, s)
  MATTOHF_DISPATCH(NG, CALL)
#undef CALL
}

template <int N>
static cudaError_t configure_df_impl() {
  constexpr int NTEAM = (kThreads / 32) * Team<N>::PER_WARP;
  const size_t smem = sizeof(float4) * (size_t)N * (1 + 2 * NTEAM);
  cudaError_t e = cudaFuncSetAttribute(k_fock_sym_df<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_fock_sym_df_batch<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t configure_df_kernels() {
  cudaError_t e;
  if ((e = configure_df_impl<16>()) != cudaSuccess) return e;
  if ((e = configure_df_impl<32>()) != cudaSuccess) return e;
  if ((e = configure_df_impl<64>()) != cudaSuccess) return e;
  if ((e = configure_df_impl<128>()) != cudaSuccess) return e;
  if ((e = configure_df_impl<256>()) != cudaSuccess) return e;
  return configure_df_impl<512>();
}

cudaError_t launch_to_df_tables(const double* kern, int nkern, float2* kern_df, const double2* tw, int ntw,
                                float4* tw_df, cudaStream_t s) {
  k_real_to_df<<<(nkern + 255) / 256, 256, 0, s>>>(kern, nkern, kern_df);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cplx_to_df<<<(ntw + 255) / 256, 256, 0, s>>>(tw, ntw, tw_df);
  return cudaGetLastError();
}

}  // namespace mattohf
