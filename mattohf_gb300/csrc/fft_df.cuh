// Double-float ("df") arithmetic and the team FFT on it.
//
// A df number is an unevaluated sum hi + lo of two FP32 values with
// |lo| <= ulp(hi)/2, i.e. a 48-bit significand, built from the error-free
// transformations TwoSum (Knuth), FastTwoSum (Dekker) and the FMA-based
// TwoProduct.  Additions use the accurate-high/sloppy-low form, whose error is
// bounded by ~2^-47 (|a| + |b|) — normwise stable, which is what an FFT needs.
// Every operation is spelled with __fadd_rn/__fmul_rn/__fmaf_rn so the
// compiler can neither contract nor reassociate the error terms.
//
// On GB300 the FP32 pipe issues ~63x more operations per second than the
// FP64 pipe, so the transforms of the exchange kernel run several times
// faster in df than in FP64 while staying within ~1e-14 (relative, normwise)
// of the FP64 result.
#pragma once
#include "fft.cuh"

namespace mattohf {
namespace df {

__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 add(float2 a, float2 b) {
  float2 s = two_sum(a.x, b.x);
  s.y = __fadd_rn(s.y, __fadd_rn(a.y, b.y));
  return fast_two_sum(s.x, s.y);
}
__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return add(a, neg(b)); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return fast_two_sum(p, e);
}
// a1*b1 + a2*b2 with one rounding of the high parts' sum
__device__ __forceinline__ float2 dot2(float2 a1, float2 b1, float2 a2, float2 b2) {
  const float p1 = __fmul_rn(a1.x, b1.x);
  const float p2 = __fmul_rn(a2.x, b2.x);
  float e = __fmaf_rn(a1.x, b1.x, -p1);
  e = __fadd_rn(e, __fmaf_rn(a2.x, b2.x, -p2));
  float2 s = two_sum(p1, p2);
  e = __fmaf_rn(a1.x, b1.y, e);
  e = __fmaf_rn(a1.y, b1.x, e);
  e = __fmaf_rn(a2.x, b2.y, e);
  e = __fmaf_rn(a2.y, b2.x, e);
  s.y = __fadd_rn(s.y, e);
  return fast_two_sum(s.x, s.y);
}
__device__ __forceinline__ float2 from_double(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double to_double(float2 a) { return (double)a.x + (double)a.y; }

// complex df: (re, im)
struct cdf {
  float2 re, im;
};
__device__ __forceinline__ cdf make(float2 r, float2 i) {
  cdf c;
  c.re = r;
  c.im = i;
  return c;
}
__device__ __forceinline__ cdf load(const float4* p) {
  const float4 v = *p;
  return make(make_float2(v.x, v.y), make_float2(v.z, v.w));
}
__device__ __forceinline__ void store(float4* p, cdf a) { *p = make_float4(a.re.x, a.re.y, a.im.x, a.im.y); }
__device__ __forceinline__ cdf from_double2(double2 z) { return make(from_double(z.x), from_double(z.y)); }
__device__ __forceinline__ double2 to_double2(cdf a) { return make_double2(to_double(a.re), to_double(a.im)); }
__device__ __forceinline__ cdf cadd(cdf a, cdf b) { return make(add(a.re, b.re), add(a.im, b.im)); }
__device__ __forceinline__ cdf csub(cdf a, cdf b) { return make(sub(a.re, b.re), sub(a.im, b.im)); }
__device__ __forceinline__ cdf conj(cdf a) { return make(a.re, neg(a.im)); }
// a * w
__device__ __forceinline__ cdf cmul(cdf a, cdf w) {
  return make(dot2(a.re, w.re, neg(a.im), w.im), dot2(a.re, w.im, a.im, w.re));
}
// a * conj(b)
__device__ __forceinline__ cdf cmulc(cdf a, cdf b) {
  return make(dot2(a.re, b.re, a.im, b.im), dot2(a.im, b.re, neg(a.re), b.im));
}
__device__ __forceinline__ cdf scale(cdf a, float2 s) { return make(mul(a.re, s), mul(a.im, s)); }
template <int DIR>
__device__ __forceinline__ cdf rot4(cdf a) {
  return DIR < 0 ? make(a.im, neg(a.re)) : make(neg(a.im), a.re);
}

template <int R, int DIR> struct Dft;
template <int DIR> struct Dft<2, DIR> {
  __device__ __forceinline__ static void run(cdf* x) {
    const cdf a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};
template <int DIR> struct Dft<4, DIR> {
  __device__ __forceinline__ static void run(cdf* x) {
    const cdf e0 = cadd(x[0], x[2]), e1 = csub(x[0], x[2]);
    const cdf e2 = cadd(x[1], x[3]), e3 = rot4<DIR>(csub(x[1], x[3]));
    x[0] = cadd(e0, e2);
    x[2] = csub(e0, e2);
    x[1] = cadd(e1, e3);
    x[3] = csub(e1, e3);
  }
};
template <int DIR> struct Dft<8, DIR> {
  __device__ __forceinline__ static void run(cdf* x) {
    // sqrt(1/2) as a df constant
    const float2 c = make_float2(0.70710677f, 1.21016175e-08f);
    const cdf a0 = cadd(x[0], x[4]), a1 = csub(x[0], x[4]);
    const cdf a2 = cadd(x[2], x[6]), a3 = rot4<DIR>(csub(x[2], x[6]));
    const cdf a4 = cadd(x[1], x[5]), a5 = csub(x[1], x[5]);
    const cdf a6 = cadd(x[3], x[7]), a7 = rot4<DIR>(csub(x[3], x[7]));
    const cdf b0 = cadd(a0, a2), b2 = csub(a0, a2);
    const cdf b1 = cadd(a1, a3), b3 = csub(a1, a3);
    const cdf b4 = cadd(a4, a6), b6 = rot4<DIR>(csub(a4, a6));
    const cdf b5 = cadd(a5, a7), b7 = csub(a5, a7);
    x[0] = cadd(b0, b4);
    x[4] = csub(b0, b4);
    x[2] = cadd(b2, b6);
    x[6] = csub(b2, b6);
    float2 s5, t5, s7, t7;
    if (DIR < 0) {
      s5 = add(b5.re, b5.im);  t5 = sub(b5.im, b5.re);
      s7 = sub(b7.im, b7.re);  t7 = neg(add(b7.re, b7.im));
    } else {
      s5 = sub(b5.re, b5.im);  t5 = add(b5.re, b5.im);
      s7 = neg(add(b7.re, b7.im)); t7 = sub(b7.re, b7.im);
    }
    const cdf p5 = make(mul(c, s5), mul(c, t5));
    const cdf p7 = make(mul(c, s7), mul(c, t7));
    x[1] = cadd(b1, p5);
    x[5] = csub(b1, p5);
    x[3] = cadd(b3, p7);
    x[7] = csub(b3, p7);
  }
};

template <int N, int R, int NS, int DIR, int T>
__device__ __forceinline__ void fft_mid_pass(cdf* buf, const cdf* __restrict__ tw, int tl) {
  constexpr int NBF = N / R;
  constexpr int PER = NBF / T;
  cdf v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = tl + T * p;
    const int k = j % NS;
#pragma unroll
    for (int r = 0; r < R; ++r) v[p][r] = buf[j + r * NBF];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      cdf w = tw[(r * k) * (N / (NS * R))];
      if (DIR > 0) w = conj(w);
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

// Same pass structure and slot positions as mattohf::fft_team.
template <int N, int DIR>
__device__ __forceinline__ void fft_team(cdf (&x)[Team<N>::E], cdf* buf, const cdf* __restrict__ tw, int tl) {
  using TM = Team<N>;
  constexpr int R0 = FftPlan<N>::R[0];
  constexpr int NP = FftPlan<N>::NP;
  constexpr int T = TM::T;
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) Dft<R0, DIR>::run(&x[p * R0]);
  __syncwarp();
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
#pragma unroll
    for (int r = 0; r < R0; ++r) buf[j * R0 + r] = x[p * R0 + r];
  }
  __syncwarp();
  if constexpr (NP == 3) {
    constexpr int R1 = FftPlan<N>::R[1];
    fft_mid_pass<N, R1, R0, DIR, T>(buf, tw, tl);
  }
  constexpr int RL = FftPlan<N>::R[NP - 1];
  constexpr int NS = N / RL;
#pragma unroll
  for (int p = 0; p < TM::PER; ++p) {
    const int j = tl + T * p;
#pragma unroll
    for (int r = 0; r < RL; ++r) x[p * RL + r] = buf[j + r * NS];
#pragma unroll
    for (int r = 1; r < RL; ++r) {
      cdf w = tw[r * j];
      if (DIR > 0) w = conj(w);
      x[p * RL + r] = cmul(x[p * RL + r], w);
    }
    Dft<RL, DIR>::run(&x[p * RL]);
  }
  __syncwarp();
}

}  // namespace df
}  // namespace mattohf

namespace mattohf {
namespace df {

// Compact-code variant of fft_team: the same slot interface (values in
// registers at Team<N>::pos), but every pass is the SAME radix-4 Stockham
// butterfly block (plus one radix-2 pass when log2 N is odd), executed from a
// runtime loop over passes through the team's shared-memory buffer.  A few
// percent more arithmetic than the radix-8 plan, but the instruction
// footprint of the whole transform is one butterfly block, which keeps the
// double-float kernel out of instruction-cache stalls.
template <int N>
__device__ __forceinline__ void fft_team_compact(cdf (&x)[Team<N>::E], cdf* buf, const cdf* __restrict__ tw, int tl) {
  using TM = Team<N>;
  constexpr int T = TM::T;
  constexpr int L2 = N == 16 ? 4 : N == 32 ? 5 : N == 64 ? 6 : N == 128 ? 7 : N == 256 ? 8 : 9;
  constexpr int P4 = N / (4 * T);   // radix-4 butterflies per lane
  constexpr int P2 = N / (2 * T);   // radix-2 butterflies per lane
  static_assert(P4 >= 1, "team too large for a radix-4 pass");
#pragma unroll
  for (int e = 0; e < TM::E; ++e) buf[TM::pos(tl, e)] = x[e];
  __syncwarp();
  int ls = 0;  // log2 of the current stride NS
#pragma unroll 1
  for (int s = 0; s < L2 / 2; ++s, ls += 2) {
    const int NS = 1 << ls;
    cdf v[P4 * 4];
#pragma unroll
    for (int p = 0; p < P4; ++p) {
      const int j = tl + T * p;
      const int k = j & (NS - 1);
#pragma unroll
      for (int r = 0; r < 4; ++r) v[p * 4 + r] = buf[j + r * (N / 4)];
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < 4; ++r) v[p * 4 + r] = cmul(v[p * 4 + r], tw[(r * k) << (L2 - ls - 2)]);
      }
      Dft<4, -1>::run(&v[p * 4]);
    }
    __syncwarp();
#pragma unroll
    for (int p = 0; p < P4; ++p) {
      const int j = tl + T * p;
      const int base = ((j >> ls) << (ls + 2)) + (j & (NS - 1));
#pragma unroll
      for (int r = 0; r < 4; ++r) buf[base + r * NS] = v[p * 4 + r];
    }
    __syncwarp();
  }
  if constexpr (L2 & 1) {
    constexpr int NS = N / 2;
    cdf v[P2 * 2];
#pragma unroll
    for (int p = 0; p < P2; ++p) {
      const int j = tl + T * p;
      v[p * 2] = buf[j];
      v[p * 2 + 1] = cmul(buf[j + N / 2], tw[j]);
      Dft<2, -1>::run(&v[p * 2]);
    }
    __syncwarp();
#pragma unroll
    for (int p = 0; p < P2; ++p) {
      const int j = tl + T * p;
      buf[j] = v[p * 2];
      buf[j + NS] = v[p * 2 + 1];
    }
    __syncwarp();
  }
#pragma unroll
  for (int e = 0; e < TM::E; ++e) x[e] = buf[TM::pos(tl, e)];
  __syncwarp();
}

}  // namespace df
}  // namespace mattohf
