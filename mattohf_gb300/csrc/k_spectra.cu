// Filtered Fourier transforms of the real-time series (src/RT_calculation.f90:246-351).
//
// For each frequency omega_i = i/Nomega * omegaM (i = 1..Nomega):
//   JF = sum_t exp(i omega t) filter(t) (J(t) - J0) dt
//   EF = sum_t exp(i omega t) filter(t) E(t) dt
//   AF = sum_t exp(i omega t) filter(t) A(t) dt
// One thread per frequency, time summed in order like the Fortran SUM;
// exp(i omega t) through CUDA's sincos.
#include "internal.h"
#include "../../include/mattohf.h"

#include <vector>

namespace {

__global__ void k_fourier(int nt, const double* __restrict__ t, const double* __restrict__ J, double J0,
                          const double* __restrict__ E, const double* __restrict__ A,
                          const double* __restrict__ filt, int nomega, double omegaM, double dt,
                          double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nomega) return;
  const double w = (double)(i + 1) / (double)nomega * omegaM;
  double jr = 0, ji = 0, er = 0, ei = 0, ar = 0, ai = 0;
  for (int k = 0; k < nt; ++k) {
    double s, c;
    sincos(w * t[k], &s, &c);
    const double jt = filt[k] * (J[k] - J0);
    const double et = filt[k] * E[k];
    const double at = filt[k] * A[k];
    jr += c * jt;
    ji += s * jt;
    er += c * et;
    ei += s * et;
    ar += c * at;
    ai += s * at;
  }
  double* o = out + (size_t)i * 7;
  o[0] = w;
  o[1] = jr * dt;
  o[2] = ji * dt;
  o[3] = er * dt;
  o[4] = ei * dt;
  o[5] = ar * dt;
  o[6] = ai * dt;
}

}  // namespace

extern "C" int mattohf_fourier(int device, int nt, const double* time, const double* J, double J0,
                               const double* E, const double* A, const double* filter, int nomega,
                               double omegaM, double dt, double* out) {
  if (nt < 1 || nomega < 1 || !time || !J || !E || !A || !filter || !out) return MATTOHF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  double* d = nullptr;
  const size_t nin = 5 * (size_t)nt;
  if (cudaMalloc(&d, sizeof(double) * (nin + 7 * (size_t)nomega)) != cudaSuccess) return MATTOHF_ERR_ALLOC;
  int rc = MATTOHF_OK;
  const double* src[5] = {time, J, E, A, filter};
  for (int k = 0; k < 5 && rc == MATTOHF_OK; ++k)
    if (cudaMemcpy(d + (size_t)k * nt, src[k], sizeof(double) * nt, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = MATTOHF_ERR_CUDA;
  if (rc == MATTOHF_OK) {
    k_fourier<<<(nomega + 127) / 128, 128>>>(nt, d, d + nt, J0, d + 2 * (size_t)nt, d + 3 * (size_t)nt,
                                             d + 4 * (size_t)nt, nomega, omegaM, dt, d + nin);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(out, d + nin, sizeof(double) * 7 * nomega, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MATTOHF_ERR_CUDA;
  }
  cudaFree(d);
  return rc;
}
