// Filtered Fourier transforms of the real-time series (src/RT_calculation.f90:246-351).
//
// For each frequency omega_i = i/Nomega * omegaM (i = 1..Nomega):
//   JF = sum_t exp(i omega t) filter(t) (J(t) - J0) dt
//   EF = sum_t exp(i omega t) filter(t) E(t) dt
//   AF = sum_t exp(i omega t) filter(t) A(t) dt
// The time sum is split into chunks (grid y) so that the Nomega x NT terms
// fill the GPU: a CTA takes 128 frequencies and one chunk of times, whose
// filtered samples it stages in shared memory once.  The chunk partials are
// added in chunk order by a second kernel (a fixed order; the reference's SUM
// runs through t in one pass, so the rounding differs at the 1e-15 level).
// On a uniform time grid exp(i omega t) is advanced by the rotation
// exp(i omega dt) (angle addition, 4 FP64 operations) and recomputed with
// sincos every 32 points, so the recurrence error stays near 1e-15; on any
// other grid every term takes its own sincos.
#include "internal.h"
#include "../../include/mattohf.h"

#include <cmath>
#include <vector>

namespace {

constexpr int kFtThreads = 128;   // frequencies per CTA
constexpr int kFtChunk = 512;     // time points per chunk (staged in shared memory)
constexpr int kFtReseed = 32;     // rotation steps between sincos evaluations

template <bool UNIFORM>
__global__ void __launch_bounds__(kFtThreads) k_fourier(int nt, const double* __restrict__ t,
                                                       const double* __restrict__ J, double J0,
                                                       const double* __restrict__ E,
                                                       const double* __restrict__ A,
                                                       const double* __restrict__ filt, int nomega,
                                                       double omegaM, double step, double* __restrict__ part) {
  __shared__ double sj[kFtChunk], se[kFtChunk], sa[kFtChunk], st[kFtChunk];
  const int chunk = blockIdx.y;
  const int k0 = chunk * kFtChunk, k1 = min(nt, k0 + kFtChunk), n = k1 - k0;
  for (int k = threadIdx.x; k < n; k += kFtThreads) {
    const double f = filt[k0 + k];
    sj[k] = f * (J[k0 + k] - J0);
    se[k] = f * E[k0 + k];
    sa[k] = f * A[k0 + k];
    st[k] = t[k0 + k];
  }
  __syncthreads();
  const int i = blockIdx.x * kFtThreads + threadIdx.x;
  if (i >= nomega) return;
  const double w = (double)(i + 1) / (double)nomega * omegaM;
  double jr = 0, ji = 0, er = 0, ei = 0, ar = 0, ai = 0;
  double rs = 0.0, rc = 1.0;  // exp(i w step)
  if (UNIFORM) sincos(w * step, &rs, &rc);
  double s = 0.0, c = 1.0;
  for (int k = 0; k < n; ++k) {
    if (!UNIFORM || k % kFtReseed == 0) {
      sincos(w * st[k], &s, &c);
    } else {
      const double cn = fma(c, rc, -(s * rs));
      s = fma(s, rc, c * rs);
      c = cn;
    }
    jr = fma(c, sj[k], jr);
    ji = fma(s, sj[k], ji);
    er = fma(c, se[k], er);
    ei = fma(s, se[k], ei);
    ar = fma(c, sa[k], ar);
    ai = fma(s, sa[k], ai);
  }
  double* o = part + ((size_t)chunk * nomega + i) * 6;
  o[0] = jr;
  o[1] = ji;
  o[2] = er;
  o[3] = ei;
  o[4] = ar;
  o[5] = ai;
}

// out[i] = (omega_i, the six sums times dt), chunks added in order
__global__ void k_fourier_sum(const double* __restrict__ part, int nchunks, int nomega, double omegaM,
                              double dt, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nomega) return;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int ch = 0; ch < nchunks; ++ch) {
    const double* p = part + ((size_t)ch * nomega + i) * 6;
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] += p[q];
  }
  double* o = out + (size_t)i * 7;
  o[0] = (double)(i + 1) / (double)nomega * omegaM;
#pragma unroll
  for (int q = 0; q < 6; ++q) o[q + 1] = acc[q] * dt;
}

}  // namespace

extern "C" int mattohf_fourier(int device, int nt, const double* time, const double* J, double J0,
                               const double* E, const double* A, const double* filter, int nomega,
                               double omegaM, double dt, double* out) {
  if (nt < 1 || nomega < 1 || !time || !J || !E || !A || !filter || !out) return MATTOHF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  // a uniform grid t_k = t_0 + k * step (to rounding) takes the rotation path
  const double step = nt > 1 ? (time[nt - 1] - time[0]) / (double)(nt - 1) : 0.0;
  bool uniform = nt > 1 && std::isfinite(step);
  for (int k = 0; k < nt && uniform; ++k) {
    const double tk = time[0] + step * (double)k;
    if (!(std::fabs(time[k] - tk) <= 4e-15 * (std::fabs(time[k]) + std::fabs(step)))) uniform = false;
  }
  const int nchunks = (nt + kFtChunk - 1) / kFtChunk;
  const size_t nin = 5 * (size_t)nt, npart = (size_t)nchunks * nomega * 6;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (nin + npart + 7 * (size_t)nomega)) != cudaSuccess) return MATTOHF_ERR_ALLOC;
  int rc = MATTOHF_OK;
  const double* src[5] = {time, J, E, A, filter};
  for (int k = 0; k < 5 && rc == MATTOHF_OK; ++k)
    if (cudaMemcpy(d + (size_t)k * nt, src[k], sizeof(double) * nt, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = MATTOHF_ERR_CUDA;
  if (rc == MATTOHF_OK) {
    double* part = d + nin;
    double* dout = part + npart;
    const dim3 grid((nomega + kFtThreads - 1) / kFtThreads, nchunks);
    if (uniform)
      k_fourier<true><<<grid, kFtThreads>>>(nt, d, d + nt, J0, d + 2 * (size_t)nt, d + 3 * (size_t)nt,
                                            d + 4 * (size_t)nt, nomega, omegaM, step, part);
    else
      k_fourier<false><<<grid, kFtThreads>>>(nt, d, d + nt, J0, d + 2 * (size_t)nt, d + 3 * (size_t)nt,
                                             d + 4 * (size_t)nt, nomega, omegaM, step, part);
    k_fourier_sum<<<(nomega + 127) / 128, 128>>>(part, nchunks, nomega, omegaM, dt, dout);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(out, dout, sizeof(double) * 7 * nomega, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MATTOHF_ERR_CUDA;
  }
  cudaFree(d);
  return rc;
}
