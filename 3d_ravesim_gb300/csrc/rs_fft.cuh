// rs_fft.cuh — register-resident Stockham FFT for power-of-two lengths 16..16384.
//
// Each sequence of length N is processed by T = N/16 threads that each hold 16 complex
// values in registers. A stage of radix R performs 16/R butterflies per thread; between
// stages the values go through a padded shared-memory buffer (one float2 pad per 16
// elements, which makes the stride-16 writes of the first stage bank-conflict free).
//
// Register <-> position mapping. For a stage of radix R, register e = b*R + r of thread t
// holds position  t + b*T + r*(N/R)  (Stockham input order). The last stage of a forward
// transform leaves its outputs in the same kind of mapping, for its own radix, and the
// inverse transform runs the forward's radix list in reverse, so
//   forward exit mapping == inverse entry mapping, inverse exit mapping == forward entry.
// Any position-wise operation (transfer function, transmission) can therefore be applied
// in registers between a forward and an inverse transform with no data exchange.
//
// Stockham stage (Govindaraju et al., SC'08 formulation): butterfly j (0 <= j < N/R),
// k = j mod Ns, inputs x[j + r*N/R] * W_{Ns*R}^{r*k}, radix-R DFT, outputs to
// y[(j/Ns)*Ns*R + k + q*Ns]; Ns *= R.
#pragma once
#include <utility>
#include "rs_common.cuh"

namespace rs {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N>
struct FftPlan {
  static_assert(N >= 16 && (N & (N - 1)) == 0, "power-of-two length >= 16");
  static constexpr int LG = ilog2c(N);
  static constexpr int NFULL = LG / 4;                 // radix-16 stages
  static constexpr int REM = 1 << (LG % 4);            // trailing radix (1 = none)
  static constexpr int NST = NFULL + (REM > 1 ? 1 : 0);
  static constexpr int T = N / 16;                     // threads per sequence
  static constexpr int S = N + N / 16;                 // padded shared buffer length
  __host__ __device__ static constexpr int radix(bool inv, int s) {
    return ((inv ? (NST - 1 - s) : s) < NFULL) ? 16 : REM;
  }
  __host__ __device__ static constexpr int entry_radix(bool inv) { return radix(inv, 0); }
  __host__ __device__ static constexpr int exit_radix(bool inv) { return radix(inv, NST - 1); }
};

__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

// Position held by register e of thread t in a radix-R mapping.
template <int N, int R>
__device__ __forceinline__ int slot_pos(int t, int e) {
  return t + (e / R) * (N / 16) + (e % R) * (N / R);
}

template <int R, bool INV, int... Bs>
__device__ __forceinline__ void dft_all(float2 (&v)[16], std::integer_sequence<int, Bs...>) {
  (dft_slice<R, INV, Bs * R>(v), ...);
}

template <int N, bool INV, int SI, int NS>
struct FftStages {
  static __device__ __forceinline__ void run(float2 (&v)[16], float2* buf, int t,
                                             const float2* __restrict__ tw) {
    using P = FftPlan<N>;
    constexpr int R = P::radix(INV, SI);
    constexpr int B = 16 / R;
    constexpr int T = P::T;
    if constexpr (NS > 1) {
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int k = (t + b * T) & (NS - 1);
        const int step = k * (N / (NS * R));
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = __ldg(&tw[r * step]);
          v[b * R + r] = INV ? cmulc(v[b * R + r], w) : cmul(v[b * R + r], w);
        }
      }
    }
    dft_all<R, INV>(v, std::make_integer_sequence<int, B>{});
    if constexpr (SI + 1 < P::NST) {
      constexpr int R2 = P::radix(INV, SI + 1);
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int base = (j / NS) * NS * R + (j & (NS - 1));
#pragma unroll
        for (int q = 0; q < R; ++q) buf[padi(base + q * NS)] = v[b * R + q];
      }
      __syncthreads();
#pragma unroll
      for (int e = 0; e < 16; ++e) v[e] = buf[padi(slot_pos<N, R2>(t, e))];
      __syncthreads();
      FftStages<N, INV, SI + 1, NS * R>::run(v, buf, t, tw);
    }
  }
};

// Full transform of one sequence. On entry v is in the entry mapping of this direction,
// on exit in its exit mapping. Every thread of the block must call it (it synchronises).
// tw[m] = exp(-2*pi*i*m/N), m in [0, N).
template <int N, bool INV>
__device__ __forceinline__ void fft_seq(float2 (&v)[16], float2* buf, int t,
                                        const float2* __restrict__ tw) {
  FftStages<N, INV, 0, 1>::run(v, buf, t, tw);
}

}  // namespace rs
