// Allocation-free exchange apply (mattohf_fock_noalloc).
//
// Some callers cannot allocate device memory at the point where they need the
// exchange term: a host code that owns a fixed device arena and forbids
// allocation after start-up, a caller that must not disturb a memory pool
// shared with other work, or a time-stepping loop that must not take the
// allocator's locks or synchronisation.  They pass their own device buffers
// for inputs and outputs; the Fock pair kernel's scratch (twiddles, the
// scaled soft-Coulomb table and the chunk partial sums) comes from one
// file-scope device array of fixed size instead of cudaMalloc.
//
// The array (kNoAllocScratchBytes) is part of the library's device image:
// every GPU that loads the library holds it until the process exits.  All
// calls share it and it keeps the previous call's contents; everything a call
// reads is written earlier in the same call.  Calls whose work overlaps on the
// GPU (different streams, or different host threads without ordering) race on
// it and must be serialised by the caller.
#include "fft.cuh"
#include "internal.h"
#include "../../include/mattohf.h"

#include <mutex>

using namespace mattohf;

namespace {

constexpr size_t kNoAllocScratchBytes = 16ull << 20;  // 16 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Per device, resolved once with that device current: the device address of
// g_noalloc_scratch (the host symbol itself is only a stand-in, not a device
// address) and the device's multiprocessor count (the pair-chunking target).
// The cache belongs to the CUDA runtime's primary context of each device: a
// caller that resets a device (cudaDeviceReset) or makes another driver
// context current invalidates it and must not call this entry point again in
// that process.
void* g_scratch_addr[kMaxDevices] = {nullptr};
int g_scratch_nsm[kMaxDevices] = {0};
std::mutex g_scratch_mu;

__global__ void k_noalloc_prep(double2* tw, int NG, const double* vcq, double* kern, int total,
                               double ng, double nk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NG) {
    double s, c;
    sincospi(-2.0 * (double)i / (double)NG, &s, &c);
    tw[i] = make_double2(c, s);
  }
  if (i < total) kern[i] = (-vcq[i] / ng) / nk;
}

// vF[col][g] = sum_ch partial[col][ch][g], chunks in ascending order.
__global__ void k_noalloc_sum(const double2* __restrict__ part, int nchunks, int NG, int total,
                              double2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int col = i / NG, g = i % NG;
  const double2* src = part + (size_t)col * nchunks * NG + g;
  double2 f = src[0];
  for (int ch = 1; ch < nchunks; ++ch) f = cadd(f, src[(size_t)ch * NG]);
  out[i] = f;
}

// Device address of the scratch array and the multiprocessor count of the
// current device; set up once per device with that device current.
int scratch_setup(void** out, int* nsm) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MATTOHF_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MATTOHF_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    int n = 0;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return MATTOHF_ERR_CUDA;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
      return MATTOHF_ERR_CUDA;
    g_scratch_nsm[dev] = n;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  *nsm = g_scratch_nsm[dev];
  return MATTOHF_OK;
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

}  // namespace

extern "C" int mattohf_fock_noalloc(int NG, int NK, int NB, int NBocc, int nbw, const double* d_vCq,
                                    const double* d_ubk, const double* d_wbk, double* d_vFwbk,
                                    void* stream) {
  if (!(NG == 16 || NG == 32 || NG == 64 || NG == 128 || NG == 256 || NG == 512)) return MATTOHF_ERR_ARG;
  if (NK < 1 || NB < 1 || NBocc < 1 || NBocc > NB || nbw < 1) return MATTOHF_ERR_ARG;
  if (!d_vCq || !d_ubk || !d_wbk || !d_vFwbk) return MATTOHF_ERR_ARG;
  const size_t ncols = (size_t)NK * nbw;
  const size_t tw_bytes = align256(sizeof(double2) * NG);
  const size_t kern_bytes = align256(sizeof(double) * (size_t)(2 * NK - 1) * NG);
  const size_t col_bytes = sizeof(double2) * ncols * NG;  // one chunk of partials
  if (tw_bytes + kern_bytes + col_bytes > kNoAllocScratchBytes) return MATTOHF_ERR_TOO_LARGE;
  void* base = nullptr;
  int nsm = 0;
  const int rc = scratch_setup(&base, &nsm);
  if (rc != MATTOHF_OK) return rc;
  // same pair chunking as the context path, capped by the scratch budget
  const int npairs = NK * NBocc;
  int nch = (nsm * 8 + (int)ncols - 1) / (int)ncols;
  const int fit = (int)((kNoAllocScratchBytes - tw_bytes - kern_bytes) / col_bytes);
  nch = nch < fit ? nch : fit;
  nch = nch < npairs ? nch : npairs;
  if (nch < 1) nch = 1;
  const int chunk = (npairs + nch - 1) / nch;
  nch = (npairs + chunk - 1) / chunk;

  unsigned char* b = static_cast<unsigned char*>(base);
  double2* tw = reinterpret_cast<double2*>(b);
  double* kern = reinterpret_cast<double*>(b + tw_bytes);
  double2* part = reinterpret_cast<double2*>(b + tw_bytes + kern_bytes);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  const int total_k = (2 * NK - 1) * NG;
  const int n_prep = total_k > NG ? total_k : NG;
  k_noalloc_prep<<<(n_prep + 255) / 256, 256, 0, st>>>(tw, NG, d_vCq, kern, total_k, (double)NG,
                                                       (double)NK);
  if (cudaGetLastError() != cudaSuccess) return MATTOHF_ERR_CUDA;
  FockArgs a;
  a.u.p = reinterpret_cast<const double2*>(d_ubk);
  a.u.kstride = NB * NG;
  a.u.nb = NB;
  a.w.p = reinterpret_cast<const double2*>(d_wbk);
  a.w.kstride = nbw * NG;
  a.w.nb = nbw;
  a.nk = NK;
  a.nbocc = NBocc;
  a.kern = kern;
  a.tw = tw;
  a.scratch = part;
  a.nchunks = nch;
  a.chunk = chunk;
  if (launch_fock(NG, a, (int)ncols, st) != cudaSuccess) return MATTOHF_ERR_CUDA;
  const int total = (int)(ncols * NG);
  k_noalloc_sum<<<(total + 255) / 256, 256, 0, st>>>(part, nch, NG, total,
                                                     reinterpret_cast<double2*>(d_vFwbk));
  if (cudaGetLastError() != cudaSuccess) return MATTOHF_ERR_CUDA;
  return MATTOHF_OK;
}
