// rs_fft.cuh — register-resident Stockham FFT for lengths 2^k and 3*2^k (16..16384).
// The transforms behind NumpyVector.fft2 / ifft2 (big-wave/vector.py:341-347: scipy.fft, forward
// unnormalised, inverse scaled by 1/N), fused with the per-slice operators by the passes.
//
// Each sequence of length N is processed by T = N/E threads that each hold E complex values
// in registers (E = 16, or 24 for 3*2^k). A stage of radix R performs E/R butterflies per
// thread; between
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
  // Power-of-two lengths: 16 values per thread, radix-16 stages plus one radix-2/4/8 stage.
  // Lengths 3*2^k: 24 values per thread, a radix-24 stage (3 x 8 in registers), radix-8
  // stages and one radix-2/4 stage (one exchange fewer than a separate radix-3 stage).
  static constexpr bool POW2 = (N & (N - 1)) == 0;
  static constexpr int M = POW2 ? N : N / 3;
  static_assert((M & (M - 1)) == 0 && (POW2 || M * 3 == N), "N must be 2^k or 3*2^k");
  static_assert(N >= 16, "N >= 16");
  static constexpr int LG = ilog2c(M);
  static constexpr int BIG = POW2 ? 16 : 8;
  static constexpr int LB = POW2 ? 4 : 3;
  static constexpr int NBIG = LG / LB;
  static constexpr int REM = 1 << (LG % LB);
  static constexpr int NST = NBIG + (REM > 1 ? 1 : 0);
  static constexpr int E = POW2 ? 16 : 24;       // values per thread
  static constexpr int T = N / E;                // threads per sequence
  static constexpr int S = N + N / 16;           // padded shared buffer length
  __host__ __device__ static constexpr int fwd_radix(int s) {
    return s < NBIG ? ((!POW2 && s == 0) ? 24 : BIG) : REM;
  }
  __host__ __device__ static constexpr int radix(bool inv, int s) { return fwd_radix(inv ? (NST - 1 - s) : s); }
  __host__ __device__ static constexpr int entry_radix(bool inv) { return radix(inv, 0); }
  __host__ __device__ static constexpr int exit_radix(bool inv) { return radix(inv, NST - 1); }
  // Ns (product of the radices before stage s) in the given direction.
  __host__ __device__ static constexpr int ns(bool inv, int s) { return s == 0 ? 1 : ns(inv, s - 1) * radix(inv, s - 1); }
  // Stage-major twiddle table: stage s (Ns > 1) holds W_N^{r*k*N/(Ns*R)} at
  // stage_offset(s) + (r-1)*Ns + k, so consecutive k (consecutive lanes) read consecutive
  // entries. The forward table comes first, the inverse one (conjugated on use) at N_TW.
  __host__ __device__ static constexpr int stage_offset(bool inv, int s) {
    return s <= 1 ? 0 : stage_offset(inv, s - 1) + (radix(inv, s - 1) - 1) * ns(inv, s - 1);
  }
  __host__ __device__ static constexpr int table_len(bool inv) { return stage_offset(inv, NST); }
  static constexpr int N_TW = table_len(false);
  // palindromic radix list: the inverse stages see the same (Ns, R) as the forward ones, so they
  // read the forward table (conjugated on use) and the inverse copy is never touched
  __host__ __device__ static constexpr bool symmetric(int s = 0) {
    return s >= NST ? true : (radix(false, s) == radix(true, s) && symmetric(s + 1));
  }
  static constexpr int INV_BASE = symmetric() ? 0 : N_TW;
  static constexpr int TW_USED = symmetric() ? N_TW : N_TW + table_len(true);
};

__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

// Exchange-buffer addressing policies: element p of a sequence lives at AD::at(p) * STR.
// PadAddr: one pad per 16 elements (buffers of FftPlan::S elements).
// SwzAddr: XOR swizzle of p within its 16-element group (dense buffers of N elements, as
// filled by bulk copies); conflict-free for all power-of-two exchange patterns.
// at_plus(base, pb, off, base16) is at(base + off) given pb = at(base); off and base16 are
// compile-time constants after unrolling, and where the policy is affine in off the address
// is pb plus an immediate (base16: base is a multiple of 16).
struct PadAddr {
  static __device__ __forceinline__ int at(int p) { return padi(p); }
  static __device__ __forceinline__ int at_plus(int base, int pb, int off, bool base16) {
    if (off % 16 == 0) return pb + off + off / 16;
    if (base16 && off >= 0 && off < 16) return pb + off;
    return padi(base + off);
  }
};
struct SwzAddr {
  static __device__ __forceinline__ int at(int p) { return p ^ ((p >> 4) & 15); }
  static __device__ __forceinline__ int at_plus(int base, int pb, int off, bool) {
    if (off % 256 == 0) return pb + off;  // bits 4..7, which pick the swizzle, are unchanged
    return at(base + off);
  }
};
// NatAddr: natural order (the layout bulk copies fill and drain).
struct NatAddr {
  static __device__ __forceinline__ int at(int p) { return p; }
  static __device__ __forceinline__ int at_plus(int, int pb, int off, bool) { return pb + off; }
};

// Position held by register e of thread t in a radix-R mapping.
template <int N, int R>
__device__ __forceinline__ int slot_pos(int t, int e) {
  return t + (e / R) * FftPlan<N>::T + (e % R) * (N / R);
}

template <int R, bool INV, int E, int... Bs>
__device__ __forceinline__ void dft_all(float2 (&v)[E], std::integer_sequence<int, Bs...>) {
  (dft_slice<R, INV, Bs * R, E>(v), ...);
}

// Twiddle-load policies: from global memory through the read-only path, or from a copy of the
// table in shared memory (a generic pointer into the block's shared window).
struct TwGlobal {
  static __device__ __forceinline__ float4 load(const float4* p) { return __ldg(p); }
  static __device__ __forceinline__ float2 load(const float2* p) { return __ldg(p); }
};
struct TwShared {
  static __device__ __forceinline__ float4 load(const float4* p) { return *p; }
  static __device__ __forceinline__ float2 load(const float2* p) { return *p; }
};

// WARP = false: the sequence spans the block; each exchange is write, barrier, read, barrier.
// WARP = true : the sequence's threads share one warp (the sub-transforms of Fft2L); each
//               exchange is warp-synchronised: sync, write, sync, read.
template <int N, bool INV, int SI, int NS, class AD = PadAddr, int STR = 1, class TWL = TwGlobal, bool WARP = false>
struct FftStages {
  using P = FftPlan<N>;
  static __device__ __forceinline__ void run(float2 (&v)[P::E], float2* buf, int t,
                                             const float4* __restrict__ tw) {
    constexpr int E = P::E;
    constexpr int R = P::radix(INV, SI);
    constexpr int B = E / R;
    constexpr int T = P::T;
    if constexpr (NS > 1) {
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int k = (t + b * T) % NS;
        constexpr int TW_OFF = (INV ? P::INV_BASE : 0) + P::stage_offset(INV, SI);
        const float4* tws = tw + TW_OFF + k;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float4 w = TWL::load(&tws[(r - 1) * NS]);
          v[b * R + r] = INV ? cmulc_tw(v[b * R + r], w) : cmul_tw(v[b * R + r], w);
        }
      }
    }
    dft_all<R, INV, E>(v, std::make_integer_sequence<int, B>{});
    if constexpr (SI + 1 < P::NST) {
      constexpr int R2 = P::radix(INV, SI + 1);
      if constexpr (WARP) __syncwarp();
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        const int base = (j / NS) * NS * R + (j % NS);  // a multiple of 16 when NS == 1, R == 16
        const int pb = AD::at(base);
#pragma unroll
        for (int q = 0; q < R; ++q) buf[AD::at_plus(base, pb, q * NS, NS == 1 && R % 16 == 0) * STR] = v[b * R + q];
      }
      if constexpr (WARP) __syncwarp(); else __syncthreads();
      const int pt = AD::at(t);
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = buf[AD::at_plus(t, pt, slot_pos<N, R2>(0, e), false) * STR];
      if constexpr (!WARP) __syncthreads();
      FftStages<N, INV, SI + 1, NS * R, AD, STR, TWL, WARP>::run(v, buf, t, tw);
    }
  }
};

// Full transform of one sequence. On entry v is in the entry mapping of this direction,
// on exit in its exit mapping. Every thread of the block must call it (it synchronises).
// tw: the stage-major tables of compensated twiddles (FftPlan::stage_offset).
template <int N, bool INV, class AD = PadAddr, int STR = 1, class TWL = TwGlobal>
__device__ __forceinline__ void fft_seq(float2 (&v)[FftPlan<N>::E], float2* buf, int t,
                                        const float4* __restrict__ tw) {
  FftStages<N, INV, 0, 1, AD, STR, TWL>::run(v, buf, t, tw);
}

// ------------------------------------------------------------------ two-level transform
// For N = 16*T (power of two, T = N/16 threads per sequence, G = T/16 threads per group):
//   X[c + 16 d] = sum_m W_T^{m d} [ W_N^{m c} sum_a x[m + T a] W_16^{a c} ]
// Thread m computes the 16-point DFT over a of its entry values x[m + T a] and twiddles them by
// W_N^{m c}; one block-wide exchange hands the T values of frequency c to the G threads
// t = c*G + j; those G threads (one warp or part of one) run the T-point transform with
// FftStages<T> and warp-level exchanges only. A transform therefore has a single block
// barrier, against NST-1 pairs for the Stockham sequence.
// Entry mapping (forward) : register e of thread t holds x[t + T e]      (as FftPlan<N>, radix 16)
// Exit mapping  (forward) : register e of thread t holds X[exit_pos(t, e)]
// The inverse runs the same steps backwards (exit mapping in, entry mapping out).
// Block exchange: slot BX::at(c*T + m) holds frequency c of thread m; region c (slots of
// c*T .. c*T+T-1) is read by group c only, and the group's own exchanges stay inside it (AD
// addressing relative to the region base). With BX = NatAddr a thread's exchange slots are the
// slots of its entry values, so a block that loaded its values from the buffer may overwrite
// them without a barrier.
// Twiddle table (compensated, float4): [0, 15T): W_N^{c m} at (c-1)*T + m; then FftPlan<T>'s
// stage-major table.
template <int N>
struct Fft2L {
  static constexpr int T = N / 16;
  static constexpr int G = T / 16;
  using SP = FftPlan<(T >= 16 ? T : 16)>;
  static constexpr bool POW2 = (N & (N - 1)) == 0;
  static constexpr int TW_LEN = 15 * T + SP::TW_USED;
  // usable by a kernel that interleaves W sequences lane by lane (thread = t*W + column):
  // the G*W threads of a group must form one aligned part of a warp
  __host__ __device__ static constexpr bool ok(int W) { return POW2 && T >= 16 && G * W <= 32 && 32 % (G * W) == 0; }
  static __device__ __forceinline__ int exit_pos(int t, int e) {
    return t / G + 16 * slot_pos<T, SP::exit_radix(false)>(t % G, e);
  }
};

template <int N, class BX, class AD, int STR, class TWL>
__device__ __forceinline__ void fft2l_fwd(float2 (&v)[16], float2* buf, int t, const float4* __restrict__ tw) {
  using F = Fft2L<N>;
  constexpr int T = F::T;
  constexpr int G = F::G;
  dft16<false>(v);
#pragma unroll
  for (int c = 1; c < 16; ++c) v[c] = cmul_tw(v[c], TWL::load(&tw[(c - 1) * T + t]));
  const int pt = BX::at(t);
#pragma unroll
  for (int c = 0; c < 16; ++c) buf[BX::at_plus(t, pt, c * T, false) * STR] = v[c];
  __syncthreads();
  const int c = t / G;
  const int j = t % G;
  const int pg = BX::at(c * T + j);
#pragma unroll
  for (int e = 0; e < 16; ++e) v[e] = buf[BX::at_plus(c * T + j, pg, e * G, false) * STR];
  FftStages<T, false, 0, 1, AD, STR, TWL, true>::run(v, buf + BX::at(c * T) * STR, j, tw + 15 * T);
}

template <int N, class BX, class AD, int STR, class TWL>
__device__ __forceinline__ void fft2l_inv(float2 (&v)[16], float2* buf, int t, const float4* __restrict__ tw) {
  using F = Fft2L<N>;
  constexpr int T = F::T;
  constexpr int G = F::G;
  const int c = t / G;
  const int j = t % G;
  FftStages<T, true, 0, 1, AD, STR, TWL, true>::run(v, buf + BX::at(c * T) * STR, j, tw + 15 * T);
  __syncwarp();
  const int pg = BX::at(c * T + j);
#pragma unroll
  for (int e = 0; e < 16; ++e) buf[BX::at_plus(c * T + j, pg, e * G, false) * STR] = v[e];
  __syncthreads();
  const int pt = BX::at(t);
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = buf[BX::at_plus(t, pt, k * T, false) * STR];
#pragma unroll
  for (int k = 1; k < 16; ++k) v[k] = cmulc_tw(v[k], TWL::load(&tw[(k - 1) * T + t]));
  dft16<true>(v);
}

}  // namespace rs
