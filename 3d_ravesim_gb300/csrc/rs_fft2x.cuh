// rs_fft2x.cuh — the register-resident Stockham FFT of rs_fft.cuh for two sequences at once,
// in split (structure-of-arrays) form, with dithered twiddle tables. Used by the multislice
// passes (rs_x2.cuh); the other entry points keep rs_fft.cuh.
//
// Split form. A thread holds the same positions of two sequences A and B (two rows, or the two
// columns of a strip): value e is cp2{re = (Re A_e, Re B_e), im = (Im A_e, Im B_e)}. Every
// complex add, subtract or product is then two packed f32x2 instructions that touch no operand
// twice, where the interleaved (re, im) form needs register moves and negations to build the
// packed operands, and each twiddle is loaded once for both sequences. Multiplications by -i
// inside the butterflies are folded into the adds and subtracts that consume them.
//
// Dithered twiddles. A twiddle (or DFT constant) rounded to float applies the same relative
// error (~3e-8) to every transform of every slice, so over hundreds of slices the errors add up
// coherently. The compensated tables of rs_fft.cuh remove that error with two extra products per
// value. Here instead each table entry is one of the two floats that bracket the exact value, and
// the plan keeps kDitherTables tables in which the upper neighbour is used in a fraction of the
// tables equal to the exact value's position between the two (to 1/2K of an ulp). Slice k of a run
// uses table k mod K, so the error a slice makes differs from slice to slice and its mean over
// K slices is zero to 1/(2K) ulp; a float32 emulation of 514 slices at K = 64 gives the same
// intensity error as exact twiddles (1.05e-5 vs 1.06e-5; 7.4e-5 with fixed rounded twiddles).
// A table entry holds its twiddle as (wr, wr, wi, wi): both sequences' multiplier pairs.
//
// Single-sequence form. The same butterflies, stage structure and tables also run on one sequence
// per thread group (value type float2 = (re, im), tables of (wr, wi) entries, DftK1 constants):
// every add, subtract and product there is the operation its split-pair counterpart applies to
// each lane, in the same order, so a single-sequence transform gives the bits of the split-pair
// one (up to the sign of zero) with half the registers per thread.
#pragma once
#include <type_traits>

#include "rs_fft.cuh"

namespace rs {

constexpr int kDitherTables = 64;

struct __align__(16) cp2 {
  float2 re, im;
};

__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as one fused multiply-add b * (-1) + a (exact negation, one rounding: the subtraction)
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

__device__ __forceinline__ cp2 x_add(cp2 a, cp2 b) { return {p_add(a.re, b.re), p_add(a.im, b.im)}; }
__device__ __forceinline__ cp2 x_sub(cp2 a, cp2 b) { return {p_sub(a.re, b.re), p_sub(a.im, b.im)}; }
// a + r*b and a - r*b with r = -i (forward) or +i (inverse): -i*b = (b.im, -b.re), +i*b = (-b.im, b.re)
template <bool INV>
__device__ __forceinline__ cp2 x_add_rot(cp2 a, cp2 b) {
  return INV ? cp2{p_sub(a.re, b.im), p_add(a.im, b.re)} : cp2{p_add(a.re, b.im), p_sub(a.im, b.re)};
}
template <bool INV>
__device__ __forceinline__ cp2 x_sub_rot(cp2 a, cp2 b) {
  return INV ? cp2{p_add(a.re, b.im), p_sub(a.im, b.re)} : cp2{p_sub(a.re, b.im), p_add(a.im, b.re)};
}
// a * (wr + i wi) given the pairs WR = (wr, wr), WI = (wi, wi) and NWI = -WI:
// re = fma(re, wr, im * -wi), im = fma(im, wr, re * wi)
__device__ __forceinline__ cp2 x_mul3(cp2 a, float2 wr, float2 wi, float2 nwi) {
  return {p_fma(a.re, wr, p_mul(a.im, nwi)), p_fma(a.im, wr, p_mul(a.re, wi))};
}
// Per-lane product a * h, h = (HR, HI) holding a different multiplier for each sequence.
__device__ __forceinline__ cp2 x_mul_pair(cp2 a, cp2 h) {
  const float2 nhi = make_float2(-h.im.x, -h.im.y);
  return {p_fma(a.re, h.re, p_mul(a.im, nhi)), p_fma(a.im, h.re, p_mul(a.re, h.im))};
}
// Table twiddle w = (wr, wr, wi, wi): forward a * w, inverse a * conj(w).
template <bool INV>
__device__ __forceinline__ cp2 x_mul_tw(cp2 a, float4 w) {
  const float2 wr = make_float2(w.x, w.y), wi = make_float2(w.z, w.w);
  const float2 nwi = make_float2(-w.z, -w.w);
  return INV ? x_mul3(a, wr, nwi, wi) : x_mul3(a, wr, wi, nwi);
}

// The same product from a (wr, wi) table entry (the single-sequence layout), for split pairs
// whose table is kept at half the size.
template <bool INV>
__device__ __forceinline__ cp2 x_mul_tw(cp2 a, float2 w) {
  return x_mul_tw<INV>(a, make_float4(w.x, w.x, w.y, w.y));
}

// The real constants of the small DFTs for one table of a run: cos(pi/8), sin(pi/8) and
// sqrt(2)/2, each dithered like the twiddle tables (host-built, one set per table).
struct DftConsts {
  float c8, s8, r2;
  float c12, s12, h3;  // cos(pi/12), sin(pi/12), sqrt(3)/2: the radix-24 / radix-3 constants
};
struct DftK {
  float2 c8, nc8, s8, ns8, r2, nr2;
};
__device__ __forceinline__ DftK dft_k(const DftConsts& k) {
  return {make_float2(k.c8, k.c8), make_float2(-k.c8, -k.c8), make_float2(k.s8, k.s8),
          make_float2(-k.s8, -k.s8), make_float2(k.r2, k.r2), make_float2(-k.r2, -k.r2)};
}

// ---- single-sequence form: the lane operations above on one (re, im) value
struct DftK1 {
  float c8, s8, r2, c12, s12, h3;
};
__device__ __forceinline__ DftK1 dft_k1(const DftConsts& k) { return {k.c8, k.s8, k.r2, k.c12, k.s12, k.h3}; }

__device__ __forceinline__ float2 x_add(float2 a, float2 b) { return p_add(a, b); }
__device__ __forceinline__ float2 x_sub(float2 a, float2 b) { return p_sub(a, b); }
template <bool INV>
__device__ __forceinline__ float2 x_add_rot(float2 a, float2 b) {
  return INV ? make_float2(a.x - b.y, a.y + b.x) : make_float2(a.x + b.y, a.y - b.x);
}
template <bool INV>
__device__ __forceinline__ float2 x_sub_rot(float2 a, float2 b) {
  return INV ? make_float2(a.x + b.y, a.y - b.x) : make_float2(a.x - b.y, a.y + b.x);
}
// a * (wr + i wi) with nwi = -wi: re = fma(re, wr, im * nwi), im = fma(im, wr, re * wi)
__device__ __forceinline__ float2 x_mul3(float2 a, float wr, float wi, float nwi) {
  return make_float2(fmaf(a.x, wr, a.y * nwi), fmaf(a.y, wr, a.x * wi));
}
// Table twiddle w = (wr, wi): forward a * w, inverse a * conj(w).
template <bool INV>
__device__ __forceinline__ float2 x_mul_tw(float2 a, float2 w) {
  return INV ? x_mul3(a, w.x, -w.y, w.y) : x_mul3(a, w.x, w.y, -w.y);
}
// a * h for a transmission factor h = (Re, Im), as x_mul_pair forms each lane.
__device__ __forceinline__ float2 x_mul_one(float2 a, float2 h) { return x_mul3(a, h.x, h.y, -h.y); }

template <int M, bool INV>
__device__ __forceinline__ float2 tw16x(float2 a, const DftK1& k) {
  if constexpr (M == 0) {
    return a;
  } else if constexpr (M == 2) {
    return INV ? make_float2((a.x - a.y) * k.r2, (a.x + a.y) * k.r2)
               : make_float2((a.x + a.y) * k.r2, (a.y - a.x) * k.r2);
  } else if constexpr (M == 6) {
    return INV ? make_float2((a.x + a.y) * -k.r2, (a.x - a.y) * k.r2)
               : make_float2((a.y - a.x) * k.r2, (a.x + a.y) * -k.r2);
  } else if constexpr (M == 1) {
    return INV ? x_mul3(a, k.c8, k.s8, -k.s8) : x_mul3(a, k.c8, -k.s8, k.s8);
  } else if constexpr (M == 3) {
    return INV ? x_mul3(a, k.s8, k.c8, -k.c8) : x_mul3(a, k.s8, -k.c8, k.c8);
  } else {
    static_assert(M == 9, "W16 power");
    return INV ? x_mul3(a, -k.c8, -k.s8, k.s8) : x_mul3(a, -k.c8, k.s8, -k.s8);
  }
}

// 3-point DFT (as dft3 of rs_common.cuh) with the slice's dithered sqrt(3)/2:
// y0 = a0 + t, y1,2 = a0 - t/2 -+ i h3 (a1 - a2) (forward), t = a1 + a2.
template <bool INV>
__device__ __forceinline__ void dft3x(float2& a0, float2& a1, float2& a2, const DftK1& k) {
  const float2 t = x_add(a1, a2);
  const float2 d = x_sub(a1, a2);
  const float2 m = make_float2(fmaf(-0.5f, t.x, a0.x), fmaf(-0.5f, t.y, a0.y));
  const float2 q = INV ? make_float2(-d.y * k.h3, d.x * k.h3) : make_float2(d.y * k.h3, -d.x * k.h3);
  a0 = x_add(a0, t);
  a1 = x_add(m, q);
  a2 = x_sub(m, q);
}

// Multiply by W24^M = exp(-+2 pi i M/24) for the M used inside the 3 x 8 radix-24 butterfly,
// with the slice's dithered constants (the halves are exact).
template <int M, bool INV>
__device__ __forceinline__ float2 tw24x(float2 a, const DftK1& k) {
  if constexpr (M == 0) {
    return a;
  } else if constexpr (M == 3) {
    return tw16x<2, INV>(a, k);  // 45 degrees
  } else if constexpr (M == 6) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
  } else if constexpr (M == 12) {
    return make_float2(-a.x, -a.y);
  } else {
    static_assert(M == 1 || M == 2 || M == 4 || M == 5 || M == 7 || M == 8 || M == 10 || M == 14, "W24 power");
    // forward exp(-i 15 deg M) = (wr, wi)
    const float wr = M == 1 ? k.c12 : M == 2 ? k.h3 : M == 4 ? 0.5f : M == 5 ? k.s12 : M == 7 ? -k.s12
                   : M == 8 ? -0.5f : -k.h3;                                           // M = 10, 14
    const float wi0 = M == 1 ? -k.s12 : M == 2 ? -0.5f : M == 4 ? -k.h3 : M == 5 ? -k.c12
                    : M == 7 ? -k.c12 : M == 8 ? -k.h3 : M == 10 ? -0.5f : 0.5f;       // M = 14
    const float wi = INV ? -wi0 : wi0;
    return x_mul3(a, wr, wi, -wi);
  }
}

template <int K1, bool INV, int... N2>
__device__ __forceinline__ void tw24x_row(float2 (&a)[24], const DftK1& k, std::integer_sequence<int, N2...>) {
  ((a[8 * K1 + N2] = tw24x<N2 * K1, INV>(a[8 * K1 + N2], k)), ...);
}

template <bool INV, class V, class K>
__device__ __forceinline__ void dft8x(V (&a)[8], const K& k);  // below

// 24-point DFT as 3 x 8 (as dft24 of rs_common.cuh), natural order in and out.
template <bool INV>
__device__ __forceinline__ void dft24x(float2 (&a)[24], const DftK1& k) {
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) dft3x<INV>(a[n2], a[8 + n2], a[16 + n2], k);
  tw24x_row<1, INV>(a, k, std::make_integer_sequence<int, 8>{});
  tw24x_row<2, INV>(a, k, std::make_integer_sequence<int, 8>{});
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    float2 b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = a[8 * k1 + i];
    dft8x<INV>(b, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) a[8 * k1 + i] = b[i];
  }
  float2 y[24];
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) y[k1 + 3 * k2] = a[8 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 24; ++i) a[i] = y[i];
}

// Value type -> its twiddle-table entry and DFT-constant types.
template <class V>
struct XForm;
template <>
struct XForm<cp2> {
  using Tw = float4;
  using K = DftK;
};
template <>
struct XForm<float2> {
  using Tw = float2;
  using K = DftK1;
};

// Multiply by W16^M = exp(-+2 pi i M/16) (M as used inside the radix-16 butterfly; M = 4 is
// folded into the butterfly's adds).
template <int M, bool INV>
__device__ __forceinline__ cp2 tw16x(cp2 a, const DftK& k) {
  if constexpr (M == 0) {
    return a;
  } else if constexpr (M == 2) {
    // forward r2 (1 - i): r2 (re + im, im - re); inverse r2 (1 + i): r2 (re - im, re + im)
    return INV ? cp2{p_mul(p_sub(a.re, a.im), k.r2), p_mul(p_add(a.re, a.im), k.r2)}
               : cp2{p_mul(p_add(a.re, a.im), k.r2), p_mul(p_sub(a.im, a.re), k.r2)};
  } else if constexpr (M == 6) {
    // forward r2 (-1 - i): (r2 (im - re), -r2 (re + im)); inverse r2 (-1 + i): (-r2 (re + im), r2 (re - im))
    return INV ? cp2{p_mul(p_add(a.re, a.im), k.nr2), p_mul(p_sub(a.re, a.im), k.r2)}
               : cp2{p_mul(p_sub(a.im, a.re), k.r2), p_mul(p_add(a.re, a.im), k.nr2)};
  } else if constexpr (M == 1) {  // forward (c8, -s8)
    return INV ? x_mul3(a, k.c8, k.s8, k.ns8) : x_mul3(a, k.c8, k.ns8, k.s8);
  } else if constexpr (M == 3) {  // forward (s8, -c8)
    return INV ? x_mul3(a, k.s8, k.c8, k.nc8) : x_mul3(a, k.s8, k.nc8, k.c8);
  } else {
    static_assert(M == 9, "W16 power");  // forward (-c8, s8)
    return INV ? x_mul3(a, k.nc8, k.ns8, k.s8) : x_mul3(a, k.nc8, k.s8, k.ns8);
  }
}

// 4-point DFT in place; ROT2: a2 arrives still to be multiplied by -i (forward) / +i (inverse).
template <bool INV, bool ROT2 = false, class V>
__device__ __forceinline__ void dft4x(V& a0, V& a1, V& a2, V& a3) {
  const V t0 = ROT2 ? x_add_rot<INV>(a0, a2) : x_add(a0, a2);
  const V t1 = ROT2 ? x_sub_rot<INV>(a0, a2) : x_sub(a0, a2);
  const V t2 = x_add(a1, a3);
  const V d = x_sub(a1, a3);
  a0 = x_add(t0, t2);
  a2 = x_sub(t0, t2);
  a1 = x_add_rot<INV>(t1, d);
  a3 = x_sub_rot<INV>(t1, d);
}

template <bool INV, class V>
__device__ __forceinline__ void dft2x(V& a0, V& a1) {
  const V t = a0;
  a0 = x_add(t, a1);
  a1 = x_sub(t, a1);
}

// Natural order in and out.
template <bool INV, class V, class K>
__device__ __forceinline__ void dft8x(V (&a)[8], const K& k) {
  dft4x<INV>(a[0], a[2], a[4], a[6]);
  dft4x<INV>(a[1], a[3], a[5], a[7]);
  a[3] = tw16x<2, INV>(a[3], k);  // W8^1
  a[7] = tw16x<6, INV>(a[7], k);  // W8^3; W8^2 of a[5] folded below
  V y[8];
  y[0] = x_add(a[0], a[1]);
  y[4] = x_sub(a[0], a[1]);
  y[1] = x_add(a[2], a[3]);
  y[5] = x_sub(a[2], a[3]);
  y[2] = x_add_rot<INV>(a[4], a[5]);
  y[6] = x_sub_rot<INV>(a[4], a[5]);
  y[3] = x_add(a[6], a[7]);
  y[7] = x_sub(a[6], a[7]);
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = y[i];
}

// 16-point DFT as 4 x 4 (as dft16 of rs_common.cuh), natural order in and out.
template <bool INV, class V, class K>
__device__ __forceinline__ void dft16x(V (&a)[16], const K& k) {
#pragma unroll
  for (int r2 = 0; r2 < 4; ++r2) dft4x<INV>(a[r2], a[4 + r2], a[8 + r2], a[12 + r2]);
  a[5] = tw16x<1, INV>(a[5], k);
  a[9] = tw16x<2, INV>(a[9], k);
  a[13] = tw16x<3, INV>(a[13], k);
  a[6] = tw16x<2, INV>(a[6], k);
  a[14] = tw16x<6, INV>(a[14], k);  // a[10] (W16^4) folded into its row butterfly
  a[7] = tw16x<3, INV>(a[7], k);
  a[11] = tw16x<6, INV>(a[11], k);
  a[15] = tw16x<9, INV>(a[15], k);
  dft4x<INV>(a[0], a[1], a[2], a[3]);
  dft4x<INV>(a[4], a[5], a[6], a[7]);
  dft4x<INV, true>(a[8], a[9], a[10], a[11]);
  dft4x<INV>(a[12], a[13], a[14], a[15]);
  V y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = a[4 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 16; ++i) a[i] = y[i];
}

template <int R, bool INV, int OFF, class V, class K, int E>
__device__ __forceinline__ void dft_slice2x(V (&v)[E], const K& k) {
  if constexpr (R == 24) {
    static_assert(OFF == 0 && E == 24, "radix-24 stages use the whole array");
    dft24x<INV>(v, k);
  } else if constexpr (R == 16) {
    static_assert(OFF == 0 && E == 16, "radix-16 stages use the whole array");
    dft16x<INV>(v, k);
  } else if constexpr (R == 8) {
    V a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = v[OFF + i];
    dft8x<INV>(a, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[OFF + i] = a[i];
  } else if constexpr (R == 4) {
    dft4x<INV>(v[OFF], v[OFF + 1], v[OFF + 2], v[OFF + 3]);
  } else if constexpr (R == 2) {
    dft2x<INV>(v[OFF], v[OFF + 1]);
  }
}

template <int R, bool INV, class V, class K, int E, int... Bs>
__device__ __forceinline__ void dft_all2x(V (&v)[E], const K& k, std::integer_sequence<int, Bs...>) {
  (dft_slice2x<R, INV, Bs * R>(v, k), ...);
}

// Stockham stages of FftPlan<N> (powers of two: 16 values per thread) on split pairs (V = cp2)
// or single sequences (V = float2); the same stage structure, register mappings and exchange
// addressing as FftStages, with the exchange buffer holding one V per position. tw: this table's
// stage-major dithered entries.
template <int N, bool INV, int SI, int NS, class AD = PadAddr, bool WARP = false, class TWL = TwGlobal, int STR = 1,
          class V = cp2, class TwT = typename XForm<V>::Tw>
struct FftStages2x {
  using P = FftPlan<N>;
  using Tw = TwT;
  using K = typename XForm<V>::K;
  static constexpr int E = P::E;
  static_assert(P::POW2 || std::is_same<V, float2>::value, "split pairs are built for power-of-two lengths");
  static __device__ __forceinline__ void run(V (&v)[E], V* buf, int t, const Tw* __restrict__ tw, const K& k) {
    constexpr int R = P::radix(INV, SI);
    constexpr int B = E / R;
    constexpr int T = P::T;
    if constexpr (NS > 1) {
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int kk = (t + b * T) % NS;
        constexpr int TW_OFF = (INV ? P::INV_BASE : 0) + P::stage_offset(INV, SI);
        const Tw* tws = tw + TW_OFF + kk;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = x_mul_tw<INV>(v[b * R + r], TWL::load(&tws[(r - 1) * NS]));
      }
    }
    dft_all2x<R, INV>(v, k, std::make_integer_sequence<int, B>{});
    if constexpr (SI + 1 < P::NST) {
      constexpr int R2 = P::radix(INV, SI + 1);
      if constexpr (WARP) __syncwarp();
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int base = (j / NS) * NS * R + (j % NS);
        const int pb = AD::at(base);
#pragma unroll
        for (int q = 0; q < R; ++q) buf[AD::at_plus(base, pb, q * NS, NS == 1 && R % 16 == 0) * STR] = v[b * R + q];
      }
      if constexpr (WARP) __syncwarp(); else __syncthreads();
      const int pt = AD::at(t);
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = buf[AD::at_plus(t, pt, slot_pos<N, R2>(0, e), false) * STR];
      if constexpr (!WARP) __syncthreads();
      FftStages2x<N, INV, SI + 1, NS * R, AD, WARP, TWL, STR, V, TwT>::run(v, buf, t, tw, k);
    }
  }
};

template <int N, bool INV, class AD = PadAddr, class TWL = TwGlobal, class V>
__device__ __forceinline__ void fft_seq2x(V (&v)[FftPlan<N>::E], V* buf, int t,
                                          const typename XForm<V>::Tw* __restrict__ tw,
                                          const typename XForm<V>::K& k) {
  FftStages2x<N, INV, 0, 1, AD, false, TWL, 1, V>::run(v, buf, t, tw, k);
}

// Barrier of the threads that share one transform's block exchange: the whole block, or one
// named group of `count` threads (barrier `id` > 0) when a block runs independent groups.
struct BarBlock {
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};
struct BarGroup {
  int id, count;
  __device__ __forceinline__ void sync() const { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
};

// Two-level transform of Fft2L<N> on split pairs or single sequences (the same steps and
// mappings as fft2l_fwd / fft2l_inv); table: W_N^{c m} at (c-1)*T + m, then the T-point
// stage-major table.
template <int N, class BX, class AD, class TWL, int STR = 1, class BAR = BarBlock, class V, class TwT>
__device__ __forceinline__ void fft2l_fwd2x(V (&v)[16], V* buf, int t, const TwT* __restrict__ tw,
                                            const typename XForm<V>::K& k, const BAR& bar = BAR{}) {
  using F = Fft2L<N>;
  constexpr int T = F::T;
  constexpr int G = F::G;
  dft16x<false>(v, k);
#pragma unroll
  for (int c = 1; c < 16; ++c) v[c] = x_mul_tw<false>(v[c], TWL::load(&tw[(c - 1) * T + t]));
  const int pt = BX::at(t);
#pragma unroll
  for (int c = 0; c < 16; ++c) buf[BX::at_plus(t, pt, c * T, false) * STR] = v[c];
  bar.sync();
  const int c = t / G;
  const int j = t % G;
  const int pg = BX::at(c * T + j);
#pragma unroll
  for (int e = 0; e < 16; ++e) v[e] = buf[BX::at_plus(c * T + j, pg, e * G, false) * STR];
  FftStages2x<T, false, 0, 1, AD, true, TWL, STR, V, TwT>::run(v, buf + BX::at(c * T) * STR, j, tw + 15 * T, k);
}

template <int N, class BX, class AD, class TWL, int STR = 1, class BAR = BarBlock, class V, class TwT>
__device__ __forceinline__ void fft2l_inv2x(V (&v)[16], V* buf, int t, const TwT* __restrict__ tw,
                                            const typename XForm<V>::K& k, const BAR& bar = BAR{}) {
  using F = Fft2L<N>;
  constexpr int T = F::T;
  constexpr int G = F::G;
  const int c = t / G;
  const int j = t % G;
  FftStages2x<T, true, 0, 1, AD, true, TWL, STR, V, TwT>::run(v, buf + BX::at(c * T) * STR, j, tw + 15 * T, k);
  __syncwarp();
  const int pg = BX::at(c * T + j);
#pragma unroll
  for (int e = 0; e < 16; ++e) buf[BX::at_plus(c * T + j, pg, e * G, false) * STR] = v[e];
  bar.sync();
  const int pt = BX::at(t);
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = buf[BX::at_plus(t, pt, q * T, false) * STR];
#pragma unroll
  for (int q = 1; q < 16; ++q) v[q] = x_mul_tw<true>(v[q], TWL::load(&tw[(q - 1) * T + t]));
  dft16x<true>(v, k);
}

}  // namespace rs
