// Soft-Coulomb kernel transform table (src/Functions.f90:33-52, used by
// src/Initialization.f90:130-146).
//
// vCk(k) = 2*dx*sum_{ix=0}^{n-1} 0.5*(f(ix*dx) + f((ix+1)*dx)),
// f(x) = cos(k*x)/sqrt(x*x + 1), dx = acell/NG/20, n = trip count of
// `Do While (ix*dx < NK*acell)`.  The trapezoid sum is the same as
// 0.5 f_0 + f_1 + ... + f_{n-1} + 0.5 f_n.  g(x) = 1/sqrt(x*x + 1) does not
// depend on k and is tabulated once (k_vck_g).  One CTA per k value; thread t
// takes the points t, t + 256, t + 512, ... and advances cos(k x) and sin(k x)
// between them by a rotation through the angle 256 k dx (angle addition),
// recomputing both from x with sincos every kReseed points so that the
// recurrence's rounding never builds up over more than kReseed steps.  The
// CTA then reduces the per-thread sums in a fixed tree order.
#include "internal.h"

namespace mattohf {

constexpr int kTableThreads = 256;
constexpr int kReseed = 32;

__global__ void k_vck_g(double dx, long long n, double* __restrict__ g) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const double x = (double)i * dx;
  g[i] = 1.0 / sqrt(x * x + 1.0);
}

__global__ void __launch_bounds__(kTableThreads) k_vck(const double* __restrict__ q, double dx,
                                                       long long n, const double* __restrict__ g,
                                                       double* __restrict__ out) {
  __shared__ double red[kTableThreads];
  const double k = q[blockIdx.x];
  double wc, ws;  // rotation by kTableThreads points
  sincos(k * ((double)kTableThreads * dx), &ws, &wc);
  double s = 0.0, c = 0.0, sn = 0.0;
  int since = kReseed;
  for (long long i = threadIdx.x; n > 0 && i <= n; i += kTableThreads) {
    if (since == kReseed) {
      sincos(k * ((double)i * dx), &sn, &c);
      since = 0;
    } else {
      const double c2 = fma(c, wc, -(sn * ws));
      sn = fma(sn, wc, c * ws);
      c = c2;
    }
    ++since;
    const double f = c * g[i];
    s += (i == 0 || i == n) ? 0.5 * f : f;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = kTableThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = 2.0 * red[0] * dx;
}

__global__ void k_make_kern(const double* __restrict__ vcq, double* __restrict__ kern, int total,
                            double ng, double nk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) kern[i] = (-vcq[i] / ng) / nk;
}

// Trip count of the reference loop, evaluated with the same floating-point
// comparisons (ix converted to double, times dx, against NK*acell).
static long long vck_count(double acell, int NG, int NK, double* dx_out) {
  const double dx = acell / (double)NG / 20.0;
  const double lim = (double)NK * acell;
  long long n = (long long)(lim / dx) - 2;
  if (n < 0) n = 0;
  while ((double)n * dx < lim) ++n;
  while (n > 0 && (double)(n - 1) * dx >= lim) --n;
  *dx_out = dx;
  return n;
}

long long vck_points(double acell, int NG, int NK) {
  double dx;
  return vck_count(acell, NG, NK, &dx) + 1;
}

cudaError_t launch_vck_table(int NG, int NK, double acell, const double* d_q, int nq, double* d_g,
                             double* d_out, cudaStream_t s) {
  double dx;
  const long long n = vck_count(acell, NG, NK, &dx);
  if (nq <= 0) return cudaSuccess;
  k_vck_g<<<(unsigned)((n + 1 + 255) / 256), 256, 0, s>>>(dx, n, d_g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_vck<<<nq, kTableThreads, 0, s>>>(d_q, dx, n, d_g, d_out);
  return cudaGetLastError();
}

cudaError_t launch_make_kern(int NG, int NK, const double* vcq, double* kern, cudaStream_t s) {
  const int total = (2 * NK - 1) * NG;
  k_make_kern<<<(total + 255) / 256, 256, 0, s>>>(vcq, kern, total, (double)NG, (double)NK);
  return cudaGetLastError();
}

}  // namespace mattohf
