// Ground-state kernels: Gram-Schmidt (src/mATTOHF.f90:134-157), Krylov block
// orthonormalisation (replaces ZGESVD('O','N') of src/GS_calculation.f90:161-166),
// projected matrices (GS:175-181, GS:218-224), a Jacobi Hermitian eigensolver
// (replaces ZHEEV('V','U') of GS:183, GS:226), the subspace rotation
// (GS:184-190, GS:227-231) and Ritz values / residuals (src/Functions.f90:321-358).
//
// All reductions run in a fixed order so results are bitwise reproducible.
#include "internal.h"
#include <cfloat>

namespace mattohf {

constexpr int kGsThreads = 256;

// Fixed-order CTA sum of a complex value (kGsThreads threads), times `scale`.
// Two barriers: every thread stores its partial, warp 0 adds the eight warp
// partials of its lane (a fixed pairwise tree) and then its 32 lanes (a
// shuffle tree), and lane 0 publishes the scaled result.  On this part an SM
// issues about one FP64 warp instruction per 19 cycles in all, so the tree
// runs in one warp and only once, not redundantly in every thread.  `red` and `res` are safe to reuse on the next call without a
// third barrier: warp 0 reads `red` before the second barrier, and every
// thread reads `res` before it reaches the next call's first barrier.
__device__ double2 block_sum2(double2 v, double scale, double2* red, double2* res) {
  static_assert(kGsThreads == 256, "eight warp partials per lane");
  red[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    double2 p[8];
#pragma unroll
    for (int w = 0; w < 8; ++w) p[w] = red[w * 32 + l];
#pragma unroll
    for (int h = 4; h > 0; h >>= 1)
#pragma unroll
      for (int w = 0; w < h; ++w) {
        p[w].x += p[w + h].x;
        p[w].y += p[w + h].y;
      }
    double sx = p[0].x, sy = p[0].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (l == 0) *res = make_double2(sx * scale, sy * scale);
  }
  __syncthreads();
  return *res;
}

// Gram-Schmidt of nb columns per k with weight `weight`.
//   passes == 1: modified Gram-Schmidt, the reference's Gram_Schmidt.
//   passes == 2: the orthonormal basis of the Krylov block, by classical
//     Gram-Schmidt applied twice ("twice is enough": Giraud, Langou and
//     Rozloznik, 2005).  Each pass projects a column on all earlier columns at
//     once; the dot products are summed eight at a time, one per warp, so the
//     reductions run side by side instead of serialising in one warp (a warp
//     issues at most one FP64 instruction per ~64 cycles).
// Thread t owns the grid points t, t + kGsThreads, ... of every column, so
// between reductions no thread reads what another wrote and only the
// reductions synchronise.  STAGE: the k-point's nb columns are held in shared
// memory for the sweep (loaded and stored by their owners), so each projection
// waits on shared-memory rather than L2 latency.
constexpr int kCgsChunk = kGsThreads / 32;  // dot products reduced per round
constexpr int kCgsMaxCols = 64;
template <bool STAGE, int PASSES>
__global__ void __launch_bounds__(kGsThreads) k_mgs(double2* u, int kstride, int nb, int NG,
                                                    double weight, int* flag) {
  constexpr int passes = PASSES;
  // the classical pass's buffers exist only in its instantiation (32 KB)
  constexpr int kPartRows = PASSES == 2 ? kCgsChunk : 1, kPartCols = PASSES == 2 ? kGsThreads : 1;
  extern __shared__ double2 cols[];  // STAGE: nb * NG
  __shared__ double2 red[kGsThreads];
  __shared__ double2 res;
  __shared__ double2 part[kPartRows][kPartCols];               // passes == 2: per-thread partial dots
  __shared__ double2 zc[PASSES == 2 ? kCgsMaxCols : 1];        // passes == 2: projections of the pass
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double2* gbase = u + (size_t)blockIdx.x * kstride;
  double2* base = STAGE ? cols : gbase;
  if (STAGE)
    for (int ib = 0; ib < nb; ++ib)
      for (int i = threadIdx.x; i < NG; i += kGsThreads) cols[(size_t)ib * NG + i] = gbase[(size_t)ib * NG + i];
  for (int ib = 0; ib < nb; ++ib) {
    double2* ub = base + (size_t)ib * NG;
    for (int pass = 0; passes == 2 && pass < 2 && ib > 0; ++pass) {
      // zc[t] = weight * <u_t|u_ib> for all t < ib, from the column as it
      // stands at the start of the pass, kCgsChunk at a time
      for (int t0 = 0; t0 < ib; t0 += kCgsChunk) {
        const int nt = min(kCgsChunk, ib - t0);
        double2 acc[kCgsChunk];
#pragma unroll
        for (int c = 0; c < kCgsChunk; ++c) acc[c] = make_double2(0.0, 0.0);
        for (int i = threadIdx.x; i < NG; i += kGsThreads) {
          const double2 b = ub[i];
#pragma unroll
          for (int c = 0; c < kCgsChunk; ++c)
            if (c < nt) {
              const double2 a = base[(size_t)(t0 + c) * NG + i];
              acc[c].x = fma(a.y, b.y, fma(a.x, b.x, acc[c].x));   // conj(a)*b
              acc[c].y = fma(-a.y, b.x, fma(a.x, b.y, acc[c].y));
            }
        }
#pragma unroll
        for (int c = 0; c < kCgsChunk; ++c) part[c][threadIdx.x] = acc[c];
        __syncthreads();
        if (warp < nt) {  // warp c sums dot product t0 + c in a fixed order
          double2 p[kGsThreads / 32];
#pragma unroll
          for (int w = 0; w < kGsThreads / 32; ++w) p[w] = part[warp][w * 32 + lane];
#pragma unroll
          for (int h = kGsThreads / 64; h > 0; h >>= 1)
#pragma unroll
            for (int w = 0; w < h; ++w) {
              p[w].x += p[w + h].x;
              p[w].y += p[w + h].y;
            }
          double sx = p[0].x, sy = p[0].y;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
          }
          if (lane == 0) zc[t0 + warp] = make_double2(sx * weight, sy * weight);
        }
        __syncthreads();
      }
      // u_ib -= sum_t zc[t] u_t, t ascending
      for (int i = threadIdx.x; i < NG; i += kGsThreads) {
        double2 b = ub[i];
        for (int t = 0; t < ib; ++t) {
          const double2 a = base[(size_t)t * NG + i], z = zc[t];
          b.x = fma(a.y, z.y, fma(-a.x, z.x, b.x));
          b.y = fma(-a.y, z.x, fma(-a.x, z.y, b.y));
        }
        ub[i] = b;
      }
    }
    for (int pass = 0; passes == 1 && pass < 1; ++pass) {
      for (int ibt = 0; ibt < ib; ++ibt) {
        const double2* ut = base + (size_t)ibt * NG;
        double2 s = make_double2(0.0, 0.0);
        // FMA chains: 2 FP64 instructions per real component (dot and update)
        for (int i = threadIdx.x; i < NG; i += kGsThreads) {
          const double2 a = ut[i], b = ub[i];
          s.x = fma(a.y, b.y, fma(a.x, b.x, s.x));   // conj(a)*b
          s.y = fma(-a.y, b.x, fma(a.x, b.y, s.y));
        }
        const double2 zov = block_sum2(s, weight, red, &res);
        for (int i = threadIdx.x; i < NG; i += kGsThreads) {
          const double2 a = ut[i];
          double2 b = ub[i];
          b.x = fma(a.y, zov.y, fma(-a.x, zov.x, b.x));   // b - a*zov
          b.y = fma(-a.y, zov.x, fma(-a.x, zov.y, b.y));
          ub[i] = b;
        }
      }
    }
    double2 s = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < NG; i += kGsThreads) {
      const double2 b = ub[i];
      s.x = fma(b.y, b.y, fma(b.x, b.x, s.x));
    }
    const double nrm = block_sum2(s, weight, red, &res).x;
    if (!(nrm > 0.0) || !isfinite(nrm)) {
      if (threadIdx.x == 0 && flag) *flag = 1;
      continue;
    }
    const double sq = sqrt(nrm);
    for (int i = threadIdx.x; i < NG; i += kGsThreads) {
      double2 b = ub[i];
      b.x = b.x / sq;
      b.y = b.y / sq;
      ub[i] = b;
    }
  }
  if (STAGE)
    for (int ib = 0; ib < nb; ++ib)
      for (int i = threadIdx.x; i < NG; i += kGsThreads) gbase[(size_t)ib * NG + i] = cols[(size_t)ib * NG + i];
}

// k_mgs with the columns staged in shared memory when they fit
constexpr size_t kMgsStageMax = 160 * 1024;
static cudaError_t launch_mgs(double2* u, int kstride, int nb, int NG, double weight, int passes, int nk,
                              int* flag, cudaStream_t s) {
  if ((passes != 1 && passes != 2) || (passes == 2 && nb > kCgsMaxCols)) return cudaErrorInvalidValue;
  const size_t bytes = sizeof(double2) * (size_t)nb * NG;
  const bool stage = bytes <= kMgsStageMax;
  // the static buffers take about 37 KB with two passes, so even small
  // stagings can pass the 48 KB default: always raise the dynamic limit to
  // what this launch needs
  auto go = [&](auto kern) {
    if (stage) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
      if (e != cudaSuccess) return e;
    }
    kern<<<nk, kGsThreads, stage ? bytes : 0, s>>>(u, kstride, nb, NG, weight, flag);
    return cudaGetLastError();
  };
  if (passes == 2) return stage ? go(k_mgs<true, 2>) : go(k_mgs<false, 2>);
  return stage ? go(k_mgs<true, 1>) : go(k_mgs<false, 1>);
}

// M[k][i][j] = sum_x conj(x_i) y_j * weight for i >= j, one warp per (k, i, j):
// the eigensolver reads only the strictly lower triangle and the real part of
// the diagonal (the reference's whw/ubhub assembly), so the upper triangle is
// neither computed nor written.
__global__ void k_project(const double2* __restrict__ x, const double2* __restrict__ y, int kstride,
                          int m, int NG, double weight, double2* __restrict__ M, int total) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= total) return;
  const int ntri = m * (m + 1) / 2;
  const int k = wid / ntri, t = wid % ntri;
  int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);  // row of lower-triangle entry t
  while (i * (i + 1) / 2 > t) --i;
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  const int j = t - i * (i + 1) / 2;
  const double2* xi = x + (size_t)k * kstride + (size_t)i * NG;
  const double2* yj = y + (size_t)k * kstride + (size_t)j * NG;
  double sr = 0.0, si = 0.0;
  for (int g = lane; g < NG; g += 32) {
    const double2 a = xi[g], b = yj[g];
    sr = fma(a.y, b.y, fma(a.x, b.x, sr));
    si = fma(-a.y, b.x, fma(a.x, b.y, si));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) M[((size_t)k * m + i) * m + j] = make_double2(sr * weight, si * weight);
}

// Parallel (round-robin ordered) Jacobi for a complex Hermitian m x m matrix,
// one CTA per k.  The matrix is built from the lower triangle of M (i > j)
// with a real diagonal, like the reference's whw/ubhub assembly.  Each sweep
// is m'-1 rounds (m' = m rounded up to even) of m'/2 disjoint rotations
// applied together (A <- J^H A J with J a product of commuting plane
// rotations), so a sweep costs O(m) barriers instead of O(m^2).  Converged
// when the off-diagonal Frobenius norm is below 1e-15 of the full norm, or
// after 60 sweeps (flag set).  Eigenvalues ascending; vectors in columns of V.
constexpr int kJacMax = 64;
constexpr int kJacThreads = 128;
__global__ void __launch_bounds__(kJacThreads) k_jacobi(const double2* __restrict__ Min, int m,
                                               double* __restrict__ evals,
                                               double2* __restrict__ evecs, int* flag) {
  extern __shared__ double2 jsm[];
  const int mp = m + (m & 1);  // even size; a padded index has no coupling
  // Row stride mp + 1: the column pass reads A[r][p] and V[r][p] for 16
  // consecutive r per half-warp, which a stride of mp (a multiple of 256 B
  // when mp is a multiple of 16) would put in one shared-memory bank group.
  const int ld = mp + 1;
  double2* A = jsm;            // mp rows of ld, A[i*ld+j]
  double2* V = jsm + mp * ld;  // the same
  __shared__ double2 red[kJacThreads];
  __shared__ double2 norms;
  __shared__ int order[kJacMax + 1];
  __shared__ int pp[kJacMax / 2 + 1], qq[kJacMax / 2 + 1];
  // per pair: c, s / mag (only its being nonzero is used) and s e^{i phi}, the
  // products formed once rather than per element
  __shared__ double rc[kJacMax / 2 + 1], rs[kJacMax / 2 + 1], rsr[kJacMax / 2 + 1], rsi[kJacMax / 2 + 1];
  const int k = blockIdx.x;
  const double2* Mk = Min + (size_t)k * m * m;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < mp * mp; idx += blockDim.x) {
    const int i = idx / mp, j = idx % mp;
    double2 v = make_double2(0.0, 0.0);
    if (i < m && j < m) {
      if (i > j) v = Mk[i * m + j];
      else if (i < j) { v = Mk[j * m + i]; v.y = -v.y; }
      else v = make_double2(Mk[i * m + i].x, 0.0);
    }
    A[i * ld + j] = v;
    V[i * ld + j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  const int np = mp / 2;
  bool converged = false;
  for (int sweep = 0; sweep < 60 && !converged; ++sweep) {
    // off-diagonal and total squared norms in one fixed-order reduction
    // (four warp partials per lane, then the lanes of warp 0)
    double off = 0.0, tot = 0.0;
    for (int idx = tid; idx < mp * mp; idx += kJacThreads) {
      const double2 v = A[(idx / mp) * ld + idx % mp];
      const double a2 = v.x * v.x + v.y * v.y;
      tot += a2;
      if (idx / mp != idx % mp) off += a2;
    }
    red[tid] = make_double2(off, tot);
    __syncthreads();
    if (tid < 32) {
      const double2 r0 = red[tid], r1 = red[32 + tid], r2 = red[64 + tid], r3 = red[96 + tid];
      double so = (r0.x + r1.x) + (r2.x + r3.x), st = (r0.y + r1.y) + (r2.y + r3.y);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        so += __shfl_xor_sync(0xffffffffu, so, o);
        st += __shfl_xor_sync(0xffffffffu, st, o);
      }
      if (tid == 0) norms = make_double2(so, st);
    }
    __syncthreads();
    off = norms.x;
    tot = norms.y;
    if (off <= 1e-30 * tot || off == 0.0) { converged = true; break; }
    for (int round = 0; round < mp - 1; ++round) {
      // circle-method pairing: player mp-1 is fixed
      if (tid < np) {
        int p, q;
        if (tid == 0) { p = mp - 1; q = round; }
        else { p = (round + tid) % (mp - 1); q = (round - tid + mp - 1) % (mp - 1); }
        if (p > q) { const int t = p; p = q; q = t; }
        pp[tid] = p;
        qq[tid] = q;
        const double2 apq = A[p * ld + q];
        if (fabs(apq.x) + fabs(apq.y) <= 1e-150) {
          rc[tid] = 1.0; rs[tid] = 0.0; rsr[tid] = 0.0; rsi[tid] = 0.0;
        } else {
          // zero A[p][q] with J = [[c, s e^{i phi}], [-s e^{-i phi}, c]], apq = mag e^{i phi}.
          // With d = A_qq - A_pp the angle obeys tan(2 theta) = 2 mag / |d| (the smaller
          // solution), so with r = 1/sqrt(4 mag^2 + d^2): sin(2 theta) = 2 mag r,
          // cos(2 theta) = |d| r, c^2 = (1 + cos(2 theta)) / 2 and
          // s e^{i phi} = sign(d) sin(2 theta) / (2c) * apq / mag = sign(d) (r / c) apq.
          // Two reciprocal square roots and no division keep the serial chain of
          // this single-warp step short; c^2 + s^2 = 1 to rounding.
          const double d = A[q * ld + q].x - A[p * ld + p].x;
          const double r = rsqrt(fma(d, d, 4.0 * (apq.x * apq.x + apq.y * apq.y)));
          const double c2 = fma(0.5 * fabs(d), r, 0.5);
          const double rcp_c = rsqrt(c2);
          const double k = (d >= 0.0 ? r : -r) * rcp_c;  // s / mag with its sign
          rc[tid] = c2 * rcp_c;
          rs[tid] = k;  // nonzero exactly when the rotation is applied
          rsr[tid] = k * apq.x;
          rsi[tid] = k * apq.y;
        }
      }
      __syncthreads();
      // columns p, q of A and V
      for (int w = tid; w < np * mp; w += kJacThreads) {
        const int pr = w / mp, r = w % mp;
        const int p = pp[pr], q = qq[pr];
        const double c = rc[pr], sr = rsr[pr], si = rsi[pr];  // (sr, si) = s e^{i phi}
        const double2 xp = A[r * ld + p], xq = A[r * ld + q];
        A[r * ld + p] = make_double2(c * xp.x - (sr * xq.x + si * xq.y), c * xp.y - (sr * xq.y - si * xq.x));
        A[r * ld + q] = make_double2(c * xq.x + (sr * xp.x - si * xp.y), c * xq.y + (sr * xp.y + si * xp.x));
        const double2 vp = V[r * ld + p], vq = V[r * ld + q];
        V[r * ld + p] = make_double2(c * vp.x - (sr * vq.x + si * vq.y), c * vp.y - (sr * vq.y - si * vq.x));
        V[r * ld + q] = make_double2(c * vq.x + (sr * vp.x - si * vp.y), c * vq.y + (sr * vp.y + si * vp.x));
      }
      __syncthreads();
      // rows p, q (conjugate transpose); the rotated pair's coupling is set to
      // exactly zero and its diagonal to exactly real here
      for (int w = tid; w < np * mp; w += kJacThreads) {
        const int pr = w / mp, r = w % mp;
        const int p = pp[pr], q = qq[pr];
        const double c = rc[pr], sr = rsr[pr], si = rsi[pr];
        const double2 xp = A[p * ld + r], xq = A[q * ld + r];
        double2 np_ = make_double2(c * xp.x - (sr * xq.x - si * xq.y), c * xp.y - (sr * xq.y + si * xq.x));
        double2 nq_ = make_double2(c * xq.x + (sr * xp.x + si * xp.y), c * xq.y + (sr * xp.y - si * xp.x));
        if (rs[pr] != 0.0) {
          if (r == q) { np_ = make_double2(0.0, 0.0); nq_.y = 0.0; }       // A[p][q], A[q][q]
          else if (r == p) { np_.y = 0.0; nq_ = make_double2(0.0, 0.0); }  // A[p][p], A[q][p]
        }
        A[p * ld + r] = np_;
        A[q * ld + r] = nq_;
      }
      __syncthreads();
    }
  }
  if (!converged && tid == 0 && flag) *flag = 2;
  // ascending order over the m real indices (stable on ties)
  if (tid == 0) {
    for (int i = 0; i < m; ++i) order[i] = i;
    for (int i = 1; i < m; ++i) {
      const int oi = order[i];
      const double v = A[oi * ld + oi].x;
      int j = i - 1;
      while (j >= 0 && A[order[j] * ld + order[j]].x > v) { order[j + 1] = order[j]; --j; }
      order[j + 1] = oi;
    }
  }
  __syncthreads();
  for (int i = tid; i < m; i += blockDim.x) evals[(size_t)k * m + i] = A[order[i] * ld + order[i]].x;
  for (int idx = tid; idx < m * m; idx += blockDim.x) {
    const int r = idx / m, cidx = idx % m;
    evecs[(size_t)k * m * m + idx] = V[r * ld + order[cidx]];  // [row][col]
  }
}

// out[k][b][g] = sum_c x[k][c][g] * C[k][c][b], c ascending (GS:184-190).
__global__ void k_rotate(const double2* __restrict__ x, int xkstride, int m,
                         const double2* __restrict__ C, int nout, double2* __restrict__ out,
                         int okstride, int NG, int nk) {
  const size_t total = (size_t)nk * nout * NG;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int g = (int)(i % NG);
  const int b = (int)((i / NG) % nout);
  const int k = (int)(i / ((size_t)NG * nout));
  const double2* xk = x + (size_t)k * xkstride + g;
  const double2* Ck = C + (size_t)k * m * m;
  double2 s = make_double2(0.0, 0.0);
  for (int c = 0; c < m; ++c) {
    const double2 a = xk[(size_t)c * NG], w = Ck[c * m + b];
    s.x += a.x * w.x - a.y * w.y;
    s.y += a.x * w.y + a.y * w.x;
  }
  out[(size_t)k * okstride + (size_t)b * NG + g] = s;
}

// Ritz value and residual per column, one warp per (k, b) (F:321-358).
__global__ void k_eps(const double2* __restrict__ u, const double2* __restrict__ hu, int kstride,
                      int nb, int NG, double w, double* __restrict__ eps, double* __restrict__ err,
                      int total) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= total) return;
  const int k = wid / nb, b = wid % nb;
  const double2* uc = u + (size_t)k * kstride + (size_t)b * NG;
  const double2* hc = hu + (size_t)k * kstride + (size_t)b * NG;
  double sr = 0.0;
  for (int g = lane; g < NG; g += 32) sr += uc[g].x * hc[g].x + uc[g].y * hc[g].y;
  for (int o = 16; o > 0; o >>= 1) sr += __shfl_xor_sync(0xffffffffu, sr, o);
  const double e = sr * w;
  double sa = 0.0;
  for (int g = lane; g < NG; g += 32) {
    const double rx = hc[g].x - e * uc[g].x, ry = hc[g].y - e * uc[g].y;
    sa += hypot(rx, ry);  // abs, not abs^2 (F:353)
  }
  for (int o = 16; o > 0; o >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, o);
  if (lane == 0) {
    eps[wid] = e;
    err[wid] = sqrt(sa * w);
  }
}

cudaError_t launch_gram_schmidt(int NG, const GsArgs& a, int nk, cudaStream_t s) {
  return launch_mgs(a.u, a.kstride, a.nb, NG, a.weight, 1, nk, a.flag, s);
}

cudaError_t launch_block_orth(int NG, double2* x, int kstride, int m, double weight, int nk,
                              int* flag, cudaStream_t s) {
  return launch_mgs(x, kstride, m, NG, weight, 2, nk, flag, s);
}

cudaError_t launch_project(int NG, const double2* x, const double2* y, int kstride, int m,
                           double weight, double2* M, int nk, cudaStream_t s) {
  const int total = nk * (m * (m + 1) / 2);
  const int warps_per_block = 8;
  k_project<<<(total + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, s>>>(
      x, y, kstride, m, NG, weight, M, total);
  return cudaGetLastError();
}

cudaError_t launch_jacobi(const double2* M, int m, double* evals, double2* evecs, int nk,
                          int* flag, cudaStream_t s) {
  if (m > kJacMax) return cudaErrorInvalidValue;
  const int mp = m + (m & 1);
  const size_t smem = sizeof(double2) * 2 * (size_t)mp * (mp + 1);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_jacobi<<<nk, kJacThreads, smem, s>>>(M, m, evals, evecs, flag);
  return cudaGetLastError();
}

cudaError_t launch_rotate(int NG, const double2* x, int xkstride, int m, const double2* C,
                          int nout, double2* out, int okstride, int nk, cudaStream_t s) {
  const size_t total = (size_t)nk * nout * NG;
  k_rotate<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(x, xkstride, m, C, nout, out, okstride,
                                                           NG, nk);
  return cudaGetLastError();
}

cudaError_t launch_eps(int NG, const double2* u, const double2* hu, int kstride, int nb, double w,
                       double* eps, double* err, int nk, cudaStream_t s) {
  const int total = nk * nb;
  k_eps<<<(total + 7) / 8, 256, 0, s>>>(u, hu, kstride, nb, NG, w, eps, err, total);
  return cudaGetLastError();
}

}  // namespace mattohf
