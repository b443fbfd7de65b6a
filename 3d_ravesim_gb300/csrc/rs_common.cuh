// rs_common.cuh — complex64 helpers and in-register radix-2/4/8/16 DFT butterflies.
//
// Sign convention: forward transforms use exp(-2*pi*i*j*k/N) (scipy.fft.fft2, as called
// by big-wave/vector.py:341-343); inverse ones use exp(+2*pi*i*j*k/N) and are
// unnormalised here (the 1/N of scipy.fft.ifft2 is applied by the callers).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

namespace rs {

// Blackwell (sm_100+) executes two FP32 adds / multiplies of a register pair in one
// instruction; complex add, subtract and real scaling map onto them one to one, which halves
// the instruction count of the DFT butterflies. RS_PACKED_F32X2=0 selects scalar arithmetic
// (same rounding: each lane is an IEEE round-to-nearest add or multiply either way).
#ifndef RS_PACKED_F32X2
#define RS_PACKED_F32X2 1
#endif
#if RS_PACKED_F32X2 && defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
#define RS_PACKED 1
#else
#define RS_PACKED 0
#endif
#ifndef RS_PACKED_CMUL
#define RS_PACKED_CMUL 1
#endif
#if RS_PACKED
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
#endif
#if RS_PACKED && RS_PACKED_CMUL
// Complex products as two packed operations: a*b = a.x*(b.x, b.y) + a.y*(-b.y, b.x); each lane is
// an IEEE multiply then an IEEE fused multiply-add.
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return __ffma2_rn(make_float2(a.y, a.y), make_float2(-b.y, b.x), __fmul2_rn(make_float2(a.x, a.x), b));
}
// a * conj(b) = a.x*(b.x, -b.y) + a.y*(b.y, b.x)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return __ffma2_rn(make_float2(a.y, a.y), make_float2(b.y, b.x), __fmul2_rn(make_float2(a.x, a.x), make_float2(b.x, -b.y)));
}
#else
#if !RS_PACKED
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
#endif

// Compensated twiddles. A twiddle rounded to float carries the same relative error (~3e-8)
// into every transform of every slice, so over hundreds of slice-steps those errors add up
// coherently (to ~1e-4 after 512 slices). A twiddle is therefore stored as w = hi + lo
// (float4 {hi.x, hi.y, lo.x, lo.y}, lo the float nearest to the FP64 rounding residual,
// hi + lo exact to ~2^-48) and a * w is formed as a*lo + a*hi, the small product first, so
// that only the final roundings, which depend on a, remain.
#if RS_PACKED && RS_PACKED_CMUL
__device__ __forceinline__ float2 cmul_tw(float2 a, float4 w) {
  const float2 ax = make_float2(a.x, a.x), ay = make_float2(a.y, a.y);
  const float2 c = __ffma2_rn(ay, make_float2(-w.w, w.z), __fmul2_rn(ax, make_float2(w.z, w.w)));
  return __ffma2_rn(ax, make_float2(w.x, w.y), __ffma2_rn(ay, make_float2(-w.y, w.x), c));
}
// a * conj(w)
__device__ __forceinline__ float2 cmulc_tw(float2 a, float4 w) {
  const float2 ax = make_float2(a.x, a.x), ay = make_float2(a.y, a.y);
  const float2 c = __ffma2_rn(ay, make_float2(w.w, w.z), __fmul2_rn(ax, make_float2(w.z, -w.w)));
  return __ffma2_rn(ax, make_float2(w.x, -w.y), __ffma2_rn(ay, make_float2(w.y, w.x), c));
}
#else
__device__ __forceinline__ float2 cmul_tw(float2 a, float4 w) {
  const float cr = fmaf(a.x, w.z, -a.y * w.w);
  const float ci = fmaf(a.x, w.w, a.y * w.z);
  return make_float2(fmaf(a.x, w.x, fmaf(-a.y, w.y, cr)), fmaf(a.x, w.y, fmaf(a.y, w.x, ci)));
}
// a * conj(w)
__device__ __forceinline__ float2 cmulc_tw(float2 a, float4 w) {
  const float cr = fmaf(a.x, w.z, a.y * w.w);
  const float ci = fmaf(a.y, w.z, -a.x * w.w);
  return make_float2(fmaf(a.x, w.x, fmaf(a.y, w.y, cr)), fmaf(a.y, w.x, fmaf(-a.x, w.y, ci)));
}
#endif
// x * (hi + lo) for a real constant split the same way, per lane of a pair
// (RS_COMP_CONST=0 drops the residual of the small DFTs' constants: an A/B switch)
#ifndef RS_COMP_CONST
#define RS_COMP_CONST 1
#endif
__device__ __forceinline__ float mulk(float x, float hi, float lo) {
#if RS_COMP_CONST
  return fmaf(hi, x, lo * x);
#else
  return hi * x;
#endif
}
__device__ __forceinline__ float2 mulk2(float2 x, float hi, float lo) {
#if RS_PACKED && RS_COMP_CONST
  return __ffma2_rn(make_float2(hi, hi), x, __fmul2_rn(make_float2(lo, lo), x));
#elif RS_PACKED
  return __fmul2_rn(make_float2(hi, hi), x);
#else
  return make_float2(mulk(x.x, hi, lo), mulk(x.y, hi, lo));
#endif
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// cos(pi/8), sin(pi/8), sqrt(2)/2 (mathematical constants, correctly rounded to float), and
// the floats nearest to their rounding residuals (constant - float(constant)).
constexpr float kC8 = 0.92387953251128675613f;
constexpr float kS8 = 0.38268343236508977173f;
constexpr float kR2 = 0.70710678118654752440f;
constexpr float kC8lo = 2.830748968563057e-08f;
constexpr float kS8lo = 6.2233507236442165e-09f;
constexpr float kR2lo = 1.2101617485882343e-08f;

// Multiply by W16^m = exp(-+2*pi*i*m/16) for the m used inside the 4x4 radix-16 butterfly.
template <int M, bool INV>
__device__ __forceinline__ float2 tw16(float2 a) {
  if constexpr (M == 0) {
    return a;
  } else if constexpr (M == 4) {
    return mul_mi<INV>(a);
  } else if constexpr (M == 2) {
    // fwd: c(1 - i) a = c(x + y, y - x); inv: c(1 + i) a = c(x - y, x + y)
    return INV ? mulk2(cadd(make_float2(a.x, a.x), make_float2(-a.y, a.y)), kR2, kR2lo)
               : mulk2(cadd(a, make_float2(a.y, -a.x)), kR2, kR2lo);
  } else if constexpr (M == 6) {
    // fwd: c(-1 - i) a = c(y - x, -x - y); inv: c(-1 + i) a = c(-x - y, x - y)
    return INV ? mulk2(cadd(make_float2(-a.x, a.x), make_float2(-a.y, -a.y)), kR2, kR2lo)
               : mulk2(cadd(make_float2(-a.x, -a.x), make_float2(a.y, -a.y)), kR2, kR2lo);
  } else {
    // generic: M in {1, 3, 9}
    constexpr float wr = (M == 1) ? kC8 : (M == 3) ? kS8 : -kC8;
    constexpr float wi0 = (M == 1) ? -kS8 : (M == 3) ? -kC8 : kS8;  // forward imaginary part
    constexpr float wrl = (M == 1) ? kC8lo : (M == 3) ? kS8lo : -kC8lo;
    constexpr float wil0 = (M == 1) ? -kS8lo : (M == 3) ? -kC8lo : kS8lo;
    constexpr float wi = INV ? -wi0 : wi0;
    constexpr float wil = INV ? -wil0 : wil0;
#if RS_COMP_CONST
    return cmul_tw(a, make_float4(wr, wi, wrl, wil));
#else
    (void)wrl;
    (void)wil;
    return cmul(a, make_float2(wr, wi));
#endif
  }
}

template <bool INV>
__device__ __forceinline__ void dft2(float2& a0, float2& a1) {
  const float2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  const float2 t2 = cadd(a1, a3), t3 = mul_mi<INV>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

// Natural-order in, natural-order out.
template <bool INV>
__device__ __forceinline__ void dft8(float2 (&a)[8]) {
  dft4<INV>(a[0], a[2], a[4], a[6]);  // E0..E3
  dft4<INV>(a[1], a[3], a[5], a[7]);  // O0..O3
  a[3] = tw16<2, INV>(a[3]);          // W8^1 = W16^2
  a[5] = tw16<4, INV>(a[5]);          // W8^2 = W16^4
  a[7] = tw16<6, INV>(a[7]);          // W8^3 = W16^6
  float2 y[8];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    y[k] = cadd(a[2 * k], a[2 * k + 1]);
    y[k + 4] = csub(a[2 * k], a[2 * k + 1]);
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = y[k];
}

// 16-point DFT as 4x4: column DFT4s, inner twiddles W16^(r2*k1), row DFT4s, transpose.
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&a)[16]) {
#pragma unroll
  for (int r2 = 0; r2 < 4; ++r2) dft4<INV>(a[r2], a[4 + r2], a[8 + r2], a[12 + r2]);
  a[5] = tw16<1, INV>(a[5]);
  a[9] = tw16<2, INV>(a[9]);
  a[13] = tw16<3, INV>(a[13]);
  a[6] = tw16<2, INV>(a[6]);
  a[10] = tw16<4, INV>(a[10]);
  a[14] = tw16<6, INV>(a[14]);
  a[7] = tw16<3, INV>(a[7]);
  a[11] = tw16<6, INV>(a[11]);
  a[15] = tw16<9, INV>(a[15]);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(a[4 * k1], a[4 * k1 + 1], a[4 * k1 + 2], a[4 * k1 + 3]);
  float2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = a[4 * k1 + k2];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = y[k];
}

// 3-point DFT: y0 = a0 + t, y1,2 = a0 - t/2 -+ i*(sqrt(3)/2)*(a1 - a2) (forward), t = a1 + a2.
constexpr float kHalfSqrt3 = 0.86602540378443864676f;
constexpr float kHalfSqrt3lo = 1.5543625053737742e-08f;

template <bool INV>
__device__ __forceinline__ void dft3(float2& a0, float2& a1, float2& a2) {
  const float2 t = cadd(a1, a2);
  const float2 d = csub(a1, a2);
  const float2 m = make_float2(fmaf(-0.5f, t.x, a0.x), fmaf(-0.5f, t.y, a0.y));
  const float2 q = mulk2(mul_mi<INV>(d), kHalfSqrt3, kHalfSqrt3lo);
  a0 = cadd(a0, t);
  a1 = cadd(m, q);
  a2 = csub(m, q);
}

// cos(pi/12), sin(pi/12) (15 degrees) as float + residual, for the radix-24 inner twiddles.
constexpr float kC12 = 0.96592582628906828675f;
constexpr float kS12 = 0.25881904510252076235f;
constexpr float kC12lo = 1.3567816203874372e-08f;
constexpr float kS12lo = 1.4661987179920288e-09f;

// Multiply by W24^M = exp(-+2*pi*i*M/24) for the M used inside the 3 x 8 radix-24 butterfly.
template <int M, bool INV>
__device__ __forceinline__ float2 tw24(float2 a) {
  if constexpr (M == 0) {
    return a;
  } else if constexpr (M == 3) {
    return tw16<2, INV>(a);  // 45 degrees
  } else if constexpr (M == 6) {
    return mul_mi<INV>(a);
  } else if constexpr (M == 12) {
    return make_float2(-a.x, -a.y);
  } else {
    // forward exp(-i*15deg*M) = (wr, wi0), residuals (wrl, wil0); the halves are exact
    constexpr float wr = M == 1 ? kC12 : M == 2 ? kHalfSqrt3 : M == 4 ? 0.5f : M == 5 ? kS12 : M == 7 ? -kS12
                       : M == 8 ? -0.5f : -kHalfSqrt3;                                  // M = 10, 14
    constexpr float wi0 = M == 1 ? -kS12 : M == 2 ? -0.5f : M == 4 ? -kHalfSqrt3 : M == 5 ? -kC12
                        : M == 7 ? -kC12 : M == 8 ? -kHalfSqrt3 : M == 10 ? -0.5f : 0.5f;  // M = 14
    constexpr float wrl = M == 1 ? kC12lo : M == 2 ? kHalfSqrt3lo : M == 5 ? kS12lo : M == 7 ? -kS12lo
                        : (M == 10 || M == 14) ? -kHalfSqrt3lo : 0.0f;
    constexpr float wil0 = M == 1 ? -kS12lo : (M == 4 || M == 8) ? -kHalfSqrt3lo : (M == 5 || M == 7) ? -kC12lo
                         : 0.0f;
    static_assert(M == 1 || M == 2 || M == 4 || M == 5 || M == 7 || M == 8 || M == 10 || M == 14, "W24 power");
    return cmul_tw(a, make_float4(wr, INV ? -wi0 : wi0, wrl, INV ? -wil0 : wil0));
  }
}

// 24-point DFT as 3 x 8: index n = 8 n1 + n2, k = k1 + 3 k2; 3-point DFTs over n1, inner
// twiddles W24^(n2 k1), 8-point DFTs over n2, transpose. Natural order in and out.
template <int K1, bool INV, int... N2>
__device__ __forceinline__ void tw24_row(float2 (&a)[24], std::integer_sequence<int, N2...>) {
  ((a[8 * K1 + N2] = tw24<N2 * K1, INV>(a[8 * K1 + N2])), ...);
}

template <bool INV>
__device__ __forceinline__ void dft24(float2 (&a)[24]) {
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) dft3<INV>(a[n2], a[8 + n2], a[16 + n2]);
  tw24_row<1, INV>(a, std::make_integer_sequence<int, 8>{});
  tw24_row<2, INV>(a, std::make_integer_sequence<int, 8>{});
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    float2 b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = a[8 * k1 + i];
    dft8<INV>(b);
#pragma unroll
    for (int i = 0; i < 8; ++i) a[8 * k1 + i] = b[i];
  }
  float2 y[24];
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) y[k1 + 3 * k2] = a[8 * k1 + k2];
#pragma unroll
  for (int k = 0; k < 24; ++k) a[k] = y[k];
}

// Radix-R DFT on the R registers v[OFF .. OFF+R-1] of an E-register array.
template <int R, bool INV, int OFF, int E>
__device__ __forceinline__ void dft_slice(float2 (&v)[E]) {
  if constexpr (R == 16) {
    static_assert(E == 16 && OFF == 0, "radix-16 stages use the whole 16-register array");
    dft16<INV>(v);
  } else if constexpr (R == 24) {
    static_assert(E == 24 && OFF == 0, "radix-24 stages use the whole 24-register array");
    dft24<INV>(v);
  } else if constexpr (R == 8) {
    float2 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = v[OFF + i];
    dft8<INV>(a);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[OFF + i] = a[i];
  } else if constexpr (R == 4) {
    dft4<INV>(v[OFF], v[OFF + 1], v[OFF + 2], v[OFF + 3]);
  } else if constexpr (R == 3) {
    dft3<INV>(v[OFF], v[OFF + 1], v[OFF + 2]);
  } else if constexpr (R == 2) {
    dft2<INV>(v[OFF], v[OFF + 1]);
  }
}

}  // namespace rs
