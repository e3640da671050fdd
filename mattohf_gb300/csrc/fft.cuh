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
// minimise DADD/DMUL/DFMA count: radix-8/4 with FMA-folded sqrt(1/2) terms,
// first-pass twiddles skipped, and every multiplication in front of a
// butterfly (twiddles, a G-space kernel, a pair product) folded into its first
// level with FMA.  Index arithmetic and shared-memory traffic are off the
// critical pipe.
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
// a + b * w, accumulated into a (4 FMA)
__device__ __forceinline__ double2 cmadd(double2 b, double2 w, double2 a) {
  return make_double2(fma(-b.y, w.y, fma(b.x, w.x, a.x)), fma(b.y, w.x, fma(b.x, w.y, a.y)));
}
// a + b * conj(c), accumulated into a (4 FMA)
__device__ __forceinline__ double2 cmaddc(double2 b, double2 c, double2 a) {
  return make_double2(fma(b.y, c.y, fma(b.x, c.x, a.x)), fma(-b.x, c.y, fma(b.y, c.x, a.y)));
}
// 2a - s.  For s = a + t this is the partner output a - t of a butterfly, in
// 2 FMA instead of the 4 that recomputing a - t from a and t's factors costs.
// The extra rounding is that of s, the size of the butterfly's own rounding.
__device__ __forceinline__ double2 cmirror(double2 a, double2 s) {
  return make_double2(fma(2.0, a.x, -s.x), fma(2.0, a.y, -s.y));
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

// Inputs of a butterfly's first level.  pair(i, j, s, d) forms s = X_i + X_j
// and d = X_i - X_j, where X is what the butterfly transforms: a register
// slot as is, or a slot times a twiddle, a real scale or a conjugate product.
// Folding that multiplication into the sum with FMA and taking the difference
// as 2*first - s saves 2 FP64 instructions per slot pair over multiplying
// first.  Slot indices are compile-time constants after unrolling.
struct InPlain {
  const double2* x;
  __device__ __forceinline__ void pair(int i, int j, double2& s, double2& d) const {
    s = cadd(x[i], x[j]);
    d = csub(x[i], x[j]);
  }
};

// X_r = x_r * w_r with w_0 = 1 (Stockham passes after the first)
struct InTwiddled {
  const double2* x;
  const double2* w;
  __device__ __forceinline__ void pair(int i, int j, double2& s, double2& d) const {
    const double2 t = (i == 0) ? x[0] : cmul(x[i], w[i]);
    s = cmadd(x[j], w[j], t);
    d = cmirror(t, s);
  }
};

// X_e = f[pos(e)] * x_e for a real per-point factor f (a kernel in G space)
template <int N, int L = 0>
struct InScaled;

// X_e = a[pos(e)] * conj(b[pos(e)]) for two columns read from memory (pair densities)
template <int N, int L = 0>
struct InConjProduct;

template <int R, int DIR> struct Dft;

template <int DIR> struct Dft<2, DIR> {
  template <class In>
  __device__ __forceinline__ static void run_from(const In& in, int b, double2* y) {
    double2 s, d;
    in.pair(b, b + 1, s, d);
    y[0] = s;
    y[1] = d;
  }
  __device__ __forceinline__ static void run(double2* x) { run_from(InPlain{x}, 0, x); }
};

template <int DIR> struct Dft<4, DIR> {
  template <class In>
  __device__ __forceinline__ static void run_from(const In& in, int b, double2* y) {
    double2 e0, e1, e2, e3;
    in.pair(b + 0, b + 2, e0, e1);
    in.pair(b + 1, b + 3, e2, e3);
    e3 = rot4<DIR>(e3);
    y[0] = cadd(e0, e2);
    y[2] = csub(e0, e2);
    y[1] = cadd(e1, e3);
    y[3] = csub(e1, e3);
  }
  __device__ __forceinline__ static void run(double2* x) { run_from(InPlain{x}, 0, x); }
};

template <int DIR> struct Dft<8, DIR> {
  template <class In>
  __device__ __forceinline__ static void run_from(const In& in, int b, double2* y) {
    constexpr double c = 0.70710678118654752440084436210485;
    // even / odd halves as two 4-point DFTs
    double2 a0, a1, a2, a3, a4, a5, a6, a7;
    in.pair(b + 0, b + 4, a0, a1);
    in.pair(b + 2, b + 6, a2, a3);
    in.pair(b + 1, b + 5, a4, a5);
    in.pair(b + 3, b + 7, a6, a7);
    a3 = rot4<DIR>(a3);
    a7 = rot4<DIR>(a7);
    double2 b0 = cadd(a0, a2), b2 = csub(a0, a2);
    double2 b1 = cadd(a1, a3), b3 = csub(a1, a3);
    double2 b4 = cadd(a4, a6), b6 = rot4<DIR>(csub(a4, a6));
    double2 b5 = cadd(a5, a7), b7 = csub(a5, a7);
    y[0] = cadd(b0, b4);
    y[4] = csub(b0, b4);
    y[2] = cadd(b2, b6);
    y[6] = csub(b2, b6);
    // b5 * W8^1 and b7 * W8^3, folded into the final butterflies with FMA
    double s5, t5, s7, t7;
    if (DIR < 0) {            // W8 = (1-i)/sqrt2, W8^3 = (-1-i)/sqrt2
      s5 = b5.x + b5.y;  t5 = b5.y - b5.x;
      s7 = b7.y - b7.x;  t7 = -(b7.x + b7.y);
    } else {                  // W8 = (1+i)/sqrt2, W8^3 = (-1+i)/sqrt2
      s5 = b5.x - b5.y;  t5 = b5.x + b5.y;
      s7 = -(b7.x + b7.y); t7 = b7.x - b7.y;
    }
    y[1] = make_double2(fma(c, s5, b1.x), fma(c, t5, b1.y));
    y[5] = make_double2(fma(-c, s5, b1.x), fma(-c, t5, b1.y));
    y[3] = make_double2(fma(c, s7, b3.x), fma(c, t7, b3.y));
    y[7] = make_double2(fma(-c, s7, b3.x), fma(-c, t7, b3.y));
  }
  __device__ __forceinline__ static void run(double2* x) { run_from(InPlain{x}, 0, x); }
};

// Pass plans: radices with equal first and last radix (NP passes, NP <= 8).
// L = 0: the throughput plans, used by every kernel unless it asks otherwise.
template <int N, int L = 0> struct FftPlan;
template <> struct FftPlan<16, 0>  { static constexpr int NP = 2; static constexpr int R[8] = {4, 4}; };
template <> struct FftPlan<32, 0>  { static constexpr int NP = 3; static constexpr int R[8] = {4, 2, 4}; };
// N = 64 takes three radix-4 passes on 16 lanes rather than two radix-8 passes
// on 8: 3 % more FP64 instructions in total, but half as many per lane.  A
// warp issues at most one FP64 instruction per ~64 cycles, even with
// independent operands, so the small grids, which run few transforms at a
// time, finish a transform in about half the time.
template <> struct FftPlan<64, 0>  { static constexpr int NP = 3; static constexpr int R[8] = {4, 4, 4}; };
template <> struct FftPlan<128, 0> { static constexpr int NP = 3; static constexpr int R[8] = {4, 8, 4}; };
template <> struct FftPlan<256, 0> { static constexpr int NP = 3; static constexpr int R[8] = {8, 4, 8}; };
template <> struct FftPlan<512, 0> { static constexpr int NP = 3; static constexpr int R[8] = {8, 8, 8}; };
// L = 1: latency plans for kernels that run few transforms at a time (the
// fused small-problem stages): 32-lane teams with two (N <= 64) or four
// (N = 128) values per lane, so a warp's dependent FP64 chain is about half
// that of the L = 0 plan for a few percent more instructions in total.  Sizes
// without one use the L = 0 plan.
template <int N> struct FftPlan<N, 1> : FftPlan<N, 0> {};
template <> struct FftPlan<16, 1> { static constexpr int NP = 4; static constexpr int R[8] = {2, 2, 2, 2}; };
template <> struct FftPlan<32, 1> { static constexpr int NP = 5; static constexpr int R[8] = {2, 2, 2, 2, 2}; };
template <> struct FftPlan<64, 1> { static constexpr int NP = 6; static constexpr int R[8] = {2, 2, 2, 2, 2, 2}; };
template <> struct FftPlan<128, 1> { static constexpr int NP = 4; static constexpr int R[8] = {4, 2, 4, 4}; };

template <int N, int L>
constexpr int fft_max_radix() {
  int m = 0;
  for (int p = 0; p < FftPlan<N, L>::NP; ++p) m = FftPlan<N, L>::R[p] > m ? FftPlan<N, L>::R[p] : m;
  return m;
}

template <int N, int L = 0> struct Team {
  static constexpr int R0 = FftPlan<N, L>::R[0];
  static constexpr int RMAX = fft_max_radix<N, L>();
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

template <int N, int L>
struct InScaled {
  const double2* x;
  const double* f;  // global memory, read-only for the kernel's lifetime
  int tl;
  __device__ __forceinline__ void pair(int i, int j, double2& s, double2& d) const {
    const double fi = __ldg(f + Team<N, L>::pos(tl, i)), fj = __ldg(f + Team<N, L>::pos(tl, j));
    const double2 t = make_double2(fi * x[i].x, fi * x[i].y);
    s = make_double2(fma(fj, x[j].x, t.x), fma(fj, x[j].y, t.y));
    d = make_double2(fma(-fj, x[j].x, t.x), fma(-fj, x[j].y, t.y));
  }
};

// X_e = f_e * x_e with the factors already in registers, f_e for register
// slot e (loaded before a transform that precedes this one, so that their
// latency overlaps it)
struct InScaledRegs {
  const double2* x;
  const double* f;
  __device__ __forceinline__ void pair(int i, int j, double2& s, double2& d) const {
    const double2 t = make_double2(f[i] * x[i].x, f[i] * x[i].y);
    s = make_double2(fma(f[j], x[j].x, t.x), fma(f[j], x[j].y, t.y));
    d = make_double2(fma(-f[j], x[j].x, t.x), fma(-f[j], x[j].y, t.y));
  }
};

template <int N, int L>
struct InConjProduct {
  const double2* a;
  const double2* b;
  int tl;
  __device__ __forceinline__ void pair(int i, int j, double2& s, double2& d) const {
    const int qi = Team<N, L>::pos(tl, i), qj = Team<N, L>::pos(tl, j);
    const double2 t = cmulc(a[qi], b[qi]);
    s = cmaddc(a[qj], b[qj], t);
    d = cmirror(t, s);
  }
};

// Slot of element i in the team buffer: i ^ ((i >> 3) & 7), a permutation
// inside each aligned group of 8 double2 (128 bytes, one row of the 32
// shared-memory banks).  The first pass stores R0 consecutive elements per
// lane; in natural order lane j's element r sits at j R0 + r, so with R0 = 8
// every lane of the warp hits the same banks (32 wavefronts per store
// instead of 4).  Swizzled, the 8 lanes of a wavefront hit 8 different
// 16-byte bank groups, and the unit-stride accesses of the other passes
// stay conflict-free (a permutation within an aligned group of 8).
__device__ __forceinline__ int fft_slot(int i) { return i ^ ((i >> 3) & 7); }

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
    double2 w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[p][r] = buf[fft_slot(j + r * NBF)];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      w[r] = tw[(r * k) * (N / (NS * R))];
      if (DIR > 0) w[r].y = -w[r].y;
    }
    Dft<R, DIR>::run_from(InTwiddled{v[p], w}, 0, v[p]);
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = tl + T * p;
    const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
    for (int r = 0; r < R; ++r) buf[fft_slot(base + r * NS)] = v[p][r];
  }
  __syncwarp();
}

// The middle passes P = 1 .. NP-2 of plan (N, L); NS is the product of the
// radices before pass P.
template <int N, int L, int DIR, int T, int P, int NS>
__device__ __forceinline__ void fft_mid_passes(double2* buf, const double2* __restrict__ tw, int tl) {
  if constexpr (P < FftPlan<N, L>::NP - 1) {
    constexpr int R = FftPlan<N, L>::R[P];
    fft_mid_pass<N, R, NS, DIR, T>(buf, tw, tl);
    fft_mid_passes<N, L, DIR, T, P + 1, NS * R>(buf, tw, tl);
  }
}

// Transform the input policy's values X (register slots at Team<N, L>::pos)
// into x.  buf: N double2 of team-private shared memory; tw: N forward
// twiddles exp(-2 pi i m / N).
template <int N, int DIR, int L = 0, class In>
__device__ __forceinline__ void fft_team_in(const In& in, double2 (&x)[Team<N, L>::E], double2* buf,
                                            const double2* __restrict__ tw, int tl) {
  using TM = Team<N, L>;
  constexpr int R0 = FftPlan<N, L>::R[0];
  constexpr int NP = FftPlan<N, L>::NP;
  constexpr int T = TM::T;
  // first pass (NS = 1, no twiddles), from the inputs to the buffer
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    Dft<R0, DIR>::run_from(in, p * R0, &x[p * R0]);
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
#pragma unroll
    for (int r = 0; r < R0; ++r) buf[fft_slot(j * R0 + r)] = x[p * R0 + r];
  }
  __syncwarp();
  fft_mid_passes<N, L, DIR, T, 1, R0>(buf, tw, tl);
  // last pass: NS = N / RL, outputs land at j + r*N/RL = register slot positions
  constexpr int RL = FftPlan<N, L>::R[NP - 1];
  static_assert(RL == R0, "plan must be symmetric");
  constexpr int NS = N / RL;
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
    const int k = j;  // j < NS
    double2 w[RL];
#pragma unroll
    for (int r = 0; r < RL; ++r) x[p * RL + r] = buf[fft_slot(j + r * NS)];
#pragma unroll
    for (int r = 1; r < RL; ++r) {
      w[r] = tw[r * k];  // N/(NS*RL) == 1
      if (DIR > 0) w[r].y = -w[r].y;
    }
    Dft<RL, DIR>::run_from(InTwiddled{&x[p * RL], w}, 0, &x[p * RL]);
  }
  __syncwarp();
}

// Transform x (register slots at Team<N, L>::pos) in place.
template <int N, int DIR, int L = 0>
__device__ __forceinline__ void fft_team(double2 (&x)[Team<N, L>::E], double2* buf,
                                         const double2* __restrict__ tw, int tl) {
  fft_team_in<N, DIR, L>(InPlain{x}, x, buf, tw, tl);
}

// Radix-2 decimation-in-time transform of N = 32 W points held one per lane
// by W consecutive warps (lane index L = 32 * (warp - first warp) + lane, W
// = 1 or 2): the input is X[bitrev(L)], the output Y[L] in natural order.
// Every lane forms its own output of each butterfly, A + (+-w) B, in 4 FMA
// (2 in the first stage), against 6 per two outputs in the team transforms
// above: a warp issues at most one FP64 instruction per ~64 cycles, so this
// shortens the chain of a transform that runs alone by a third.  Partners
// within a warp come by shuffle; with W = 2 the last stage goes through
// `xbuf` (N double2) and named barrier `bar` over the N threads.
template <int N, int DIR>
__device__ __forceinline__ double2 fft_lane(double2 x, int L, const double2* __restrict__ tw, double2* xbuf,
                                            int bar) {
  static_assert(N == 32 || N == 64, "one lane per point on one or two warps");
#pragma unroll
  for (int half = 1; half < N; half <<= 1) {
    double2 xp;
    if (half < 32) {
      xp.x = __shfl_xor_sync(0xffffffffu, x.x, half);
      xp.y = __shfl_xor_sync(0xffffffffu, x.y, half);
    } else {
      xbuf[L] = x;
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(N) : "memory");
      xp = xbuf[L ^ half];
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(N) : "memory");
    }
    const bool top = (L & half) == 0;
    const double2 A = top ? x : xp, B = top ? xp : x;
    if (half == 1) {
      const double sg = top ? 1.0 : -1.0;
      x = make_double2(fma(sg, B.x, A.x), fma(sg, B.y, A.y));
    } else {
      // w = W_{2 half}^j (conjugated for the inverse), negated for the bottom
      // output; the sign flips are bit operations, not FP64 instructions
      double2 w = tw[(L & (half - 1)) * (N / (2 * half))];
      const unsigned long long sx = top ? 0ull : 0x8000000000000000ull;
      const unsigned long long sy = sx ^ (DIR > 0 ? 0x8000000000000000ull : 0ull);
      w.x = __longlong_as_double(__double_as_longlong(w.x) ^ sx);
      w.y = __longlong_as_double(__double_as_longlong(w.y) ^ sy);
      x = make_double2(fma(w.x, B.x, fma(-w.y, B.y, A.x)), fma(w.x, B.y, fma(w.y, B.x, A.y)));
    }
  }
  return x;
}

// Team-wide sum of one double; team lanes are contiguous within a warp.
template <int T>
__device__ __forceinline__ double team_sum(double v) {
#pragma unroll
  for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace mattohf
