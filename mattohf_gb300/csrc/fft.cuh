// Team-level complex128 FFT for the short periodic grids of the 1D HF problem.
//
// One "team" of T lanes (T divides 32) transforms one length-N sequence.  The
// transform is a Stockham autosort FFT whose first and last passes share the
// same radix, so a lane's INPUT positions equal its OUTPUT positions:
//     pos(p, r) = (tl + T*p) + r * (N / R),   p < N/(T*R), r < R.
// Input and output therefore stay in registers, and only the middle passes
// exchange data through the team's shared-memory buffer (N double2).  This lets
// the Fock chain pair -> FFT -> kernel -> IFFT -> accumulate run without any
// shared-memory round trip between the forward and the inverse transform.
//
// Conventions match FFTW's dfftw_plan_dft_1d as the reference uses it
// (src/Initialization.f90:271-272): forward = exp(-2*pi*i*n*k/N), backward =
// exp(+2*pi*i*n*k/N), both unnormalised.
//
// The FP64 pipe bounds this code on GB300, so the butterflies are written to
// minimise DADD/DMUL/DFMA count (radix-8/4 with FMA-folded sqrt(1/2) terms,
// first-pass twiddles skipped); index arithmetic and shared-memory traffic are
// off the critical pipe.
#pragma once
#include <cuda_runtime.h>

namespace mattohf {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// a * w (4 FP64 instructions with FMA)
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.x, w.y, a.y * w.x));
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -(a.x * b.y)));
}
// acc += a * b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}

// Multiply by the primitive 4th root of unity of the transform direction:
// forward (DIR<0): -i ; backward (DIR>0): +i.  Free of FP64 arithmetic.
template <int DIR>
__device__ __forceinline__ double2 rot4(double2 a) {
  return DIR < 0 ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

template <int R, int DIR> struct Dft;

template <int DIR> struct Dft<2, DIR> {
  __device__ __forceinline__ static void run(double2* x) {
    double2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};

template <int DIR> struct Dft<4, DIR> {
  __device__ __forceinline__ static void run(double2* x) {
    double2 e0 = cadd(x[0], x[2]), e1 = csub(x[0], x[2]);
    double2 e2 = cadd(x[1], x[3]), e3 = rot4<DIR>(csub(x[1], x[3]));
    x[0] = cadd(e0, e2);
    x[2] = csub(e0, e2);
    x[1] = cadd(e1, e3);
    x[3] = csub(e1, e3);
  }
};

template <int DIR> struct Dft<8, DIR> {
  __device__ __forceinline__ static void run(double2* x) {
    constexpr double c = 0.70710678118654752440084436210485;
    // even / odd halves as two 4-point DFTs
    double2 a0 = cadd(x[0], x[4]), a1 = csub(x[0], x[4]);
    double2 a2 = cadd(x[2], x[6]), a3 = rot4<DIR>(csub(x[2], x[6]));
    double2 a4 = cadd(x[1], x[5]), a5 = csub(x[1], x[5]);
    double2 a6 = cadd(x[3], x[7]), a7 = rot4<DIR>(csub(x[3], x[7]));
    double2 b0 = cadd(a0, a2), b2 = csub(a0, a2);
    double2 b1 = cadd(a1, a3), b3 = csub(a1, a3);
    double2 b4 = cadd(a4, a6), b6 = rot4<DIR>(csub(a4, a6));
    double2 b5 = cadd(a5, a7), b7 = csub(a5, a7);
    x[0] = cadd(b0, b4);
    x[4] = csub(b0, b4);
    x[2] = cadd(b2, b6);
    x[6] = csub(b2, b6);
    // b5 * W8^1 and b7 * W8^3, folded into the final butterflies with FMA
    double s5, t5, s7, t7;
    if (DIR < 0) {            // W8 = (1-i)/sqrt2, W8^3 = (-1-i)/sqrt2
      s5 = b5.x + b5.y;  t5 = b5.y - b5.x;
      s7 = b7.y - b7.x;  t7 = -(b7.x + b7.y);
    } else {                  // W8 = (1+i)/sqrt2, W8^3 = (-1+i)/sqrt2
      s5 = b5.x - b5.y;  t5 = b5.x + b5.y;
      s7 = -(b7.x + b7.y); t7 = b7.x - b7.y;
    }
    x[1] = make_double2(fma(c, s5, b1.x), fma(c, t5, b1.y));
    x[5] = make_double2(fma(-c, s5, b1.x), fma(-c, t5, b1.y));
    x[3] = make_double2(fma(c, s7, b3.x), fma(c, t7, b3.y));
    x[7] = make_double2(fma(-c, s7, b3.x), fma(-c, t7, b3.y));
  }
};

// Pass plans: radices with equal first and last radix.
template <int N> struct FftPlan;
template <> struct FftPlan<16>  { static constexpr int NP = 2; static constexpr int R[4] = {4, 4, 0, 0}; };
template <> struct FftPlan<32>  { static constexpr int NP = 3; static constexpr int R[4] = {4, 2, 4, 0}; };
template <> struct FftPlan<64>  { static constexpr int NP = 2; static constexpr int R[4] = {8, 8, 0, 0}; };
template <> struct FftPlan<128> { static constexpr int NP = 3; static constexpr int R[4] = {4, 8, 4, 0}; };
template <> struct FftPlan<256> { static constexpr int NP = 3; static constexpr int R[4] = {8, 4, 8, 0}; };
template <> struct FftPlan<512> { static constexpr int NP = 3; static constexpr int R[4] = {8, 8, 8, 0}; };

template <int N> struct Team {
  static constexpr int R0 = FftPlan<N>::R[0];
  static constexpr int RMAX = FftPlan<N>::R[1] > R0 ? FftPlan<N>::R[1] : R0;
  // lanes per transform: every lane owns >= 1 butterfly in every pass
  static constexpr int T = (N / RMAX) < 32 ? (N / RMAX) : 32;
  static constexpr int PER = (N / R0) / T;     // butterflies per lane, first/last pass
  static constexpr int E = PER * R0;           // complex values per lane
  static constexpr int PER_WARP = 32 / T;      // transforms per warp
  static constexpr int STRIDE = N / R0;        // distance between r-slots
  // natural-order position of register slot (p, r) for team lane tl
  __device__ __forceinline__ static int pos(int tl, int p, int r) { return tl + T * p + r * STRIDE; }
  __device__ __forceinline__ static int pos(int tl, int e) { return pos(tl, e / R0, e % R0); }
};

// One Stockham pass reading and writing the team buffer.
template <int N, int R, int NS, int DIR, int T>
__device__ __forceinline__ void fft_mid_pass(double2* buf, const double2* __restrict__ tw, int tl) {
  constexpr int NBF = N / R;
  constexpr int PER = NBF / T;
  static_assert(NBF % T == 0, "team size must divide the butterfly count");
  double2 v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = tl + T * p;
    const int k = j % NS;
#pragma unroll
    for (int r = 0; r < R; ++r) v[p][r] = buf[j + r * NBF];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      double2 w = tw[(r * k) * (N / (NS * R))];
      if (DIR > 0) w.y = -w.y;
      v[p][r] = cmul(v[p][r], w);
    }
    Dft<R, DIR>::run(v[p]);
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = tl + T * p;
    const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
    for (int r = 0; r < R; ++r) buf[base + r * NS] = v[p][r];
  }
  __syncwarp();
}

// Transform x (register slots at Team<N>::pos) in place.  buf: N double2 of
// team-private shared memory; tw: N forward twiddles exp(-2 pi i m / N).
template <int N, int DIR>
__device__ __forceinline__ void fft_team(double2 (&x)[Team<N>::E], double2* buf,
                                         const double2* __restrict__ tw, int tl) {
  using TM = Team<N>;
  constexpr int R0 = FftPlan<N>::R[0];
  constexpr int NP = FftPlan<N>::NP;
  constexpr int T = TM::T;
  // first pass (NS = 1, no twiddles), from registers to the buffer
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    Dft<R0, DIR>::run(&x[p * R0]);
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
#pragma unroll
    for (int r = 0; r < R0; ++r) buf[j * R0 + r] = x[p * R0 + r];
  }
  __syncwarp();
  // middle passes
  if constexpr (NP == 3) {
    constexpr int R1 = FftPlan<N>::R[1];
    fft_mid_pass<N, R1, R0, DIR, T>(buf, tw, tl);
  }
  // last pass: NS = N / RL, outputs land at j + r*N/RL = register slot positions
  constexpr int RL = FftPlan<N>::R[NP - 1];
  static_assert(RL == R0, "plan must be symmetric");
  constexpr int NS = N / RL;
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
    const int k = j;  // j < NS
#pragma unroll
    for (int r = 0; r < RL; ++r) x[p * RL + r] = buf[j + r * NS];
#pragma unroll
    for (int r = 1; r < RL; ++r) {
      double2 w = tw[r * k];  // N/(NS*RL) == 1
      if (DIR > 0) w.y = -w.y;
      x[p * RL + r] = cmul(x[p * RL + r], w);
    }
    Dft<RL, DIR>::run(&x[p * RL]);
  }
  __syncwarp();
}

// Team-wide sum of one double; team lanes are contiguous within a warp.
template <int T>
__device__ __forceinline__ double team_sum(double v) {
#pragma unroll
  for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace mattohf
