// Soft-Coulomb kernel transform table (src/Functions.f90:33-52, used by
// src/Initialization.f90:130-146).
//
// vCk(k) = 2*dx*sum_{ix=0}^{n-1} 0.5*(f(ix*dx) + f((ix+1)*dx)),
// f(x) = cos(k*x)/sqrt(x*x + 1), dx = acell/NG/20, n = trip count of
// `Do While (ix*dx < NK*acell)`.  One CTA per k value; each thread walks a
// contiguous ix range in order (reusing f at the shared end point), then the
// CTA reduces the per-thread sums in a fixed tree order.  cos/sqrt are CUDA's
// library functions.
#include "internal.h"

namespace mattohf {

constexpr int kTableThreads = 256;

__global__ void __launch_bounds__(kTableThreads) k_vck(const double* __restrict__ q, double dx,
                                                       long long n, double* __restrict__ out) {
  __shared__ double red[kTableThreads];
  const double k = q[blockIdx.x];
  const long long per = (n + kTableThreads - 1) / kTableThreads;
  const long long i0 = (long long)threadIdx.x * per;
  const long long i1 = min(n, i0 + per);
  double s = 0.0;
  if (i0 < i1) {
    double x = (double)i0 * dx;
    double f0 = cos(k * x) / sqrt(x * x + 1.0);
    for (long long i = i0; i < i1; ++i) {
      const double x1 = (double)(i + 1) * dx;
      const double f1 = cos(k * x1) / sqrt(x1 * x1 + 1.0);
      s += 0.5 * (f0 + f1);
      f0 = f1;
    }
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

cudaError_t launch_vck_table(int NG, int NK, double acell, const double* d_q, int nq,
                             double* d_out, cudaStream_t s) {
  double dx;
  const long long n = vck_count(acell, NG, NK, &dx);
  if (nq <= 0) return cudaSuccess;
  k_vck<<<nq, kTableThreads, 0, s>>>(d_q, dx, n, d_out);
  return cudaGetLastError();
}

cudaError_t launch_make_kern(int NG, int NK, const double* vcq, double* kern, cudaStream_t s) {
  const int total = (2 * NK - 1) * NG;
  k_make_kern<<<(total + 255) / 256, 256, 0, s>>>(vcq, kern, total, (double)NG, (double)NK);
  return cudaGetLastError();
}

}  // namespace mattohf
