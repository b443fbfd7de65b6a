// rs_pipe.cuh — persistent, bulk-copy pipelined versions of the fused row and column passes.
//
// Each block owns a sequence of tiles (W whole rows, or a strip of W whole columns) and keeps
// NB tile buffers in shared memory. While it transforms tile i in buffer i % NB, the bulk-copy
// engine already fetches tile i+1 into the next buffer (rows: one 1D cp.async.bulk of W*N*8
// bytes; columns: N/256 2D tensor copies of a W x 256 box). The tile buffer doubles as the FFT
// exchange buffer (XOR-swizzled addressing) and as the staging area of the result, which one
// thread writes back with bulk stores. No thread issues a global load or store for the field.
//
// Waits on the copy barriers are bounded: after kSpinLimit polls a block records an error in
// *status and stops; the host reads it with rs_plan_status.
#pragma once
#include <cuda.h>

#include <type_traits>

#include "rs_kernels.cuh"

namespace rs {

constexpr uint32_t kSpinLimit = 1u << 22;
constexpr uint32_t kTestSpinLimit = 1u << 14;  // the test hook's wait (ColArgs::test_stall)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait; returns false (and records the failure) when the copy never landed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status,
                                                  uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (status) atomicExch(status, 1);
  return false;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_addr(src))
               : "memory");
}
// 3D forms: field z of a stack of equal fields (the tensor map's third dimension)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int K>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(K) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// --------------------------------------------------------------------------- geometry
template <int N>
struct RowPipeGeom {
  static constexpr int T = FftPlan<N>::T;
  static constexpr int RW = T >= 256 ? 1 : 256 / T;           // rows per tile
  static constexpr int SLACK = 64;                            // room for a voxel row of nx + 2
  static constexpr int TILE = RW * (N + SLACK);               // float2 per tile buffer
#ifdef RS_ROWPIPE_NB
  static constexpr int NB = RS_ROWPIPE_NB;
#else
  static constexpr int NB = (3 * TILE * 8 <= 200 * 1024) ? 3 : 2;
#endif
  static constexpr int THREADS = RW * T;
  static constexpr size_t SMEM = static_cast<size_t>(NB) * TILE * sizeof(float2) + NB * sizeof(uint64_t);
  // blocks per SM the register budget is sized for (as many as shared memory admits, up to 3)
  static constexpr int MINB = (3 * SMEM <= 227 * 1024) ? 3 : (2 * SMEM <= 227 * 1024) ? 2 : 1;
};

// Largest box height <= 256 (the tensor-copy limit) that divides n.
constexpr int box_rows(int n, int b = 256) { return (b <= 1 || n % b == 0) ? b : box_rows(n, b - 1); }

template <int N, bool DITH = false>
struct ColPipeGeom {
  static constexpr int T = FftPlan<N>::T;
#ifndef RS_COLPIPE_THREADS
#define RS_COLPIPE_THREADS 512
#endif
  // Threads per strip: 256 at 1536 and 2048 (compensated column passes 12 % and 10 % faster,
  // measured), RS_COLPIPE_THREADS (512) elsewhere (256 was 7 % slower at 1024 and 3072 there).
  // Every form runs one block per SM with two or three strip buffers, except the dithered 3*2^k
  // columns (the one-level transform with a radix-24 first stage) at 1536 and 3072: two
  // 256-thread blocks per SM with one strip buffer each (the other block computes while one
  // waits for its next strip), column passes 26.6 / 92.0 us against 28.8 / 95.0 with one block
  // and two or three buffers; three blocks per SM (80 registers) spill and took 29.2 / 95.2 us.
  // RS_COLPIPE_D3_MINB / RS_COLPIPE_D3_THREADS force one choice for every 3*2^k size.
  static constexpr bool D3 = DITH && !FftPlan<N>::POW2;
  static constexpr bool D3_PAIR = D3 && (N == 1536 || N == 3072);
#ifdef RS_COLPIPE_D3_MINB
  static constexpr int MINB = D3 ? RS_COLPIPE_D3_MINB : 1;
#else
  static constexpr int MINB = D3_PAIR ? 2 : 1;
#endif
#ifndef RS_COLPIPE_D3_THREADS
#define RS_COLPIPE_D3_THREADS 0
#endif
  static constexpr int THR = (D3 && RS_COLPIPE_D3_THREADS > 0) ? RS_COLPIPE_D3_THREADS
                             : (D3_PAIR || N == 1536 || N == 2048) ? 256
                                                                   : RS_COLPIPE_THREADS;
  // shared memory of one block when MINB blocks share an SM (228 KB, 1 KB reserved per block)
  static constexpr size_t BUDGET = MINB == 1 ? 227 * 1024 : 228 * 1024 / MINB - 1024;
  // columns per strip (>= 2: 16-byte boxes) for about THR threads
  static constexpr int W = T >= THR / 2 ? 2 : THR / T;
  static constexpr int BH = box_rows(N);                      // rows per tensor-copy box
  static_assert(N % BH == 0, "the boxes must tile a column exactly");
  static constexpr int TILE = W * N;
  static constexpr int THREADS = W * T;
  static constexpr bool L2 = Fft2L<N>::ok(W);                 // two-level column transforms
  // twiddles (compensated tables, or with DITH the dithered (wr, wi) tables) copied to shared
  // memory when they fit
  static constexpr int TW_LEN = L2 ? Fft2L<N>::TW_LEN : FftPlan<N>::TW_USED;
  static constexpr size_t TW_BYTES = static_cast<size_t>(TW_LEN) * (DITH ? sizeof(float2) : sizeof(float4));
  static_assert(!DITH || L2 || !FftPlan<N>::POW2, "dithered 2^k columns use the two-level transform");
  // Three tile buffers when they fit beside the twiddle tables, else two: the twiddles in shared
  // memory matter more than the third buffer (the L1 left beside three 64 KB tiles cannot hold
  // the compensated tables of 4096-point columns). With DITH the third buffer is also given up
  // for ey in shared memory.
#ifndef RS_COLPIPE_D3_NB
#define RS_COLPIPE_D3_NB 0
#endif
#ifdef RS_COLPIPE_NB
  static constexpr int NB = RS_COLPIPE_NB;
#else
  static constexpr int NB = (D3 && RS_COLPIPE_D3_NB > 0) ? RS_COLPIPE_D3_NB
                            : MINB >= 2                  ? 1
                            : (3 * TILE * 8 + TW_BYTES + (DITH ? N * sizeof(float2) : 0) + 64 <= BUDGET) ? 3
                                                                                                        : 2;
#endif
  static constexpr size_t TILES_BYTES = static_cast<size_t>(NB) * TILE * sizeof(float2);
#ifndef RS_COLPIPE_TW_SMEM
#define RS_COLPIPE_TW_SMEM 1
#endif
  // At 1536 and 3072 (two blocks per SM) ey takes the shared memory beside the strip and the
  // table is read through L1: column passes 24.7 / 83.3 us against 26.9 / 91.5 with the table in
  // shared memory and ey through L1. RS_COLPIPE_D3_TW_SMEM forces one choice for every 3*2^k size.
#ifdef RS_COLPIPE_D3_TW_SMEM
  static constexpr bool D3_TW_SMEM = RS_COLPIPE_D3_TW_SMEM;
#else
  static constexpr bool D3_TW_SMEM = !D3_PAIR;
#endif
  static constexpr bool TW_SMEM = RS_COLPIPE_TW_SMEM && (!D3 || D3_TW_SMEM) && TW_LEN > 0 &&
                                  TILES_BYTES + TW_BYTES + 64 <= BUDGET;
  // ey in shared memory too when it fits, stored in the register order of the forward exit
  // mapping (entry e * T + t), so that a warp's reads are consecutive
#ifndef RS_COLPIPE_EY_SMEM
#define RS_COLPIPE_EY_SMEM 1
#endif
  static constexpr size_t EY_BYTES = static_cast<size_t>(N) * sizeof(float2);
  static constexpr bool EY_SMEM =
      RS_COLPIPE_EY_SMEM && TILES_BYTES + (TW_SMEM ? TW_BYTES : 0) + EY_BYTES + 64 <= BUDGET;
  static constexpr size_t SMEM =
      TILES_BYTES + (TW_SMEM ? TW_BYTES : 0) + (EY_SMEM ? EY_BYTES : 0) + NB * sizeof(uint64_t);
};

// ---------------------------------------------------------------------- row pipeline
template <int N>
__global__ void __launch_bounds__(RowPipeGeom<N>::THREADS, RowPipeGeom<N>::MINB)
    row_pipe_kernel(const RowArgs a, int* status) {
  using P = FftPlan<N>;
  using G = RowPipeGeom<N>;
  constexpr int T = P::T;
  constexpr int E = P::E;
  constexpr int RF = P::entry_radix(false);
  constexpr int RX = P::exit_radix(false);
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* tiles = reinterpret_cast<float2*>(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(tiles + G::NB * G::TILE);
  const int t = threadIdx.x % T;
  const int lr = threadIdx.x / T;
  const int ntiles = (a.ny + G::RW - 1) / G::RW;
  const int flags = a.flags;
  const bool loads = !(flags & ROW_SRC);
  if (threadIdx.x == 0) {
    for (int b = 0; b < G::NB; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
  }
  __syncthreads();

  int tile = blockIdx.x;
  if (threadIdx.x == 0 && loads && tile < ntiles) {
    const int r0 = tile * G::RW;
    const uint32_t bytes = static_cast<uint32_t>(min(G::RW, a.ny - r0)) * N * 8u;
    mbar_arrive_expect(&bars[0], bytes);
    bulk_load(tiles, a.in + static_cast<size_t>(r0) * N, bytes, &bars[0]);
  }
  bool ok = true;
  for (int i = 0; tile < ntiles && ok; ++i, tile += gridDim.x) {
    const int b = i % G::NB;
    float2* tb = tiles + b * G::TILE;
    const int next = tile + gridDim.x;
    // Started after this tile's first transform (below): by then the store that last used the
    // target buffer has been read out, so thread 0 does not hold the block up waiting for it.
    auto prefetch_next = [&]() {
      if (threadIdx.x == 0 && loads && next < ntiles) {
        bulk_wait_read<G::NB - 2>();  // the buffer's previous store has been read out
        const int bn = (i + 1) % G::NB;
        const int r0n = next * G::RW;
        const uint32_t bytes = static_cast<uint32_t>(min(G::RW, a.ny - r0n)) * N * 8u;
        mbar_arrive_expect(&bars[bn], bytes);
        bulk_load(tiles + bn * G::TILE, a.in + static_cast<size_t>(r0n) * N, bytes, &bars[bn]);
      }
    };
    if (loads) {
      ok = mbar_wait_bounded(&bars[b], (i / G::NB) & 1, status);
    } else if (threadIdx.x == 0) {
      bulk_wait_read<G::NB - 1>();  // no loads: the store that last used buffer b has been read out
    }
    ok = __syncthreads_and(ok);  // block-uniform: a failed wait stops every thread together
    if (!ok) break;
    const int r0 = tile * G::RW;
    const int rows = min(G::RW, a.ny - r0);
    const int row = r0 + lr;
    const bool valid = lr < rows;
    float2* seq = tb + lr * N;
    float2 v[E];
    if (flags & ROW_INV) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = seq[slot_pos<N, RX>(t, e)];
      __syncthreads();
      fft_seq<N, true, SwzAddr, 1>(v, seq, t, a.tw);
    } else if (flags & ROW_SRC) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = point_source_value(a.ps, slot_pos<N, RF>(t, e), row);
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = seq[slot_pos<N, RF>(t, e)];
      __syncthreads();
    }
    prefetch_next();

    if (flags & (ROW_TVOX | ROW_TPLASMA)) {
      const bool vox = flags & ROW_TVOX;
      const int nxv = vox ? a.vox.nxv : a.pl.nxv;
      const bool staged = nxv <= N + G::SLACK;
      float2* vrow = tb + lr * (N + G::SLACK);
      int yi = -1;
      float fy = 0.0f;
      if (valid) {
        const int ar = a.axis_rows ? row % a.axis_rows : row;  // row of its own field
        yi = __ldg(&a.ax.yi[ar]);
        if (yi >= 0) fy = __ldg(&a.ax.yf[ar]);
      }
      if (staged) {
        if (yi >= 0) {
          for (int j = t; j < nxv; j += T) vrow[j] = vox ? voxel_col_blend(a.vox, j, yi, fy) : plasma_col_blend(a.pl, j, yi, fy);
        }
        __syncthreads();
      }
      // Branch-free over the E pixels (their gathers and transcendentals interleave); vacuum
      // gives a factor of exactly 1; an all-vacuum warp skips the transcendentals.
      constexpr int CH = E % 8 == 0 ? 8 : E;  // pixels per interleaved chunk
#pragma unroll
      for (int c0 = 0; c0 < E; c0 += CH) {
        float2 d[CH];
        bool any = false;
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          d[i] = make_float2(0.f, 0.f);
          const int x = slot_pos<N, RF>(t, c0 + i);
          const int2 xe = yi >= 0 ? __ldg(&a.ax.xp[x]) : make_int2(-1, 0);
          const int xi = xe.x;
          if (xi >= 0) {
            const float fx = __int_as_float(xe.y);
            if (staged) {
              d[i] = lerp2(vrow[xi], vrow[xi + 1], fx);  // exact for fx = 0; xi + 1 < nxv
            } else {
              d[i] = vox ? voxel_db(a.vox, xi, fx, yi, fy) : plasma_db(a.pl, xi, fx, yi, fy);
            }
            any |= ((__float_as_uint(d[i].x) | __float_as_uint(d[i].y)) << 1) != 0u;  // +-0 is vacuum
          }
        }
        if (__any_sync(0xffffffffu, any)) {
          const float at = vox ? a.vox.a : a.pl.a;
#pragma unroll
          for (int i = 0; i < CH; ++i) v[c0 + i] = cmul(v[c0 + i], material_factor(d[i].x, d[i].y, at));
        }
      }
      if (staged) __syncthreads();
    }

    if (flags & ROW_FWD) {
      fft_seq<N, false, SwzAddr, 1>(v, seq, t, a.tw);
#pragma unroll
      for (int e = 0; e < E; ++e) seq[slot_pos<N, RX>(t, e)] = (flags & ROW_SCALE) ? cscale(v[e], a.scale) : v[e];
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) seq[slot_pos<N, RF>(t, e)] = (flags & ROW_SCALE) ? cscale(v[e], a.scale) : v[e];
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_store(a.out + static_cast<size_t>(r0) * N, tb, static_cast<uint32_t>(rows) * N * 8u);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

// ------------------------------------------------------------------- column pipeline
// DITH: the slice's dithered two-level table (twd1, kc) in the single-sequence form of the
// split-pair arithmetic, H and the mask applied as col_x2_pipe_kernel applies them: the result is
// that kernel's, with one column per thread group.
template <int N, bool DITH = false>
__global__ void __launch_bounds__(ColPipeGeom<N, DITH>::THREADS, ColPipeGeom<N, DITH>::MINB)
    col_pipe_kernel(const ColArgs a, const __grid_constant__ CUtensorMap map_in,
                    const __grid_constant__ CUtensorMap map_out, int* status) {
  using P = FftPlan<N>;
  using G = ColPipeGeom<N, DITH>;
  using TwT = typename std::conditional<DITH, float2, float4>::type;
  constexpr int W = G::W;
  constexpr int E = P::E;
  constexpr int RF = P::entry_radix(false);
  constexpr uint32_t TILE_BYTES = G::TILE * 8u;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* tiles = reinterpret_cast<float2*>(smem_raw);
  TwT* tw_s = reinterpret_cast<TwT*>(tiles + G::NB * G::TILE);
  float2* ey_s = reinterpret_cast<float2*>(smem_raw + G::TILES_BYTES + (G::TW_SMEM ? G::TW_BYTES : 0));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + G::TILES_BYTES + (G::TW_SMEM ? G::TW_BYTES : 0) +
                                               (G::EY_SMEM ? G::EY_BYTES : 0));
  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int nx = a.nx;
  // tiles run over the strips of every field of a stack (the maps are 3D: x, y, field)
  const int strips = (nx + W - 1) / W;
  const int nfields = a.batches > 1 ? a.batches : 1;
  const int ntiles = strips * nfields;
  const int flags = a.flags;
  if (threadIdx.x == 0) {
    for (int b = 0; b < G::NB; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (a.test_stall) {
    // Phase 0 of a fresh barrier completes only on an arrival, and none is made: every thread's
    // bounded wait runs out, the status word records it, and the block returns with no copy issued.
    mbar_wait_bounded(&bars[0], 0, status, kTestSpinLimit);
    return;
  }

  const TwT* tw_g;
  if constexpr (DITH) {
    tw_g = a.twd1;
  } else {
    tw_g = G::L2 ? a.tw2 : a.tw;
  }
  if constexpr (G::TW_SMEM) {  // the block's copy of the twiddle tables (read from L2 once)
    for (int i = threadIdx.x; i < G::TW_LEN; i += blockDim.x) tw_s[i] = __ldg(&tw_g[i]);
    __syncthreads();
  }
  const TwT* tw = G::TW_SMEM ? tw_s : tw_g;
  const DftK1 k1 = dft_k1(a.kc);  // DITH only
  using TWL = typename std::conditional<G::TW_SMEM, TwShared, TwGlobal>::type;
  // with H applied, the 1/N of the inverse is folded into ey (one product per element fewer)
  const bool fold = (flags & COL_H) && (flags & COL_SCALE) && !(flags & COL_SPEC);  // U stays unscaled
  if constexpr (G::EY_SMEM) {
    if (flags & COL_H) {  // uniform: a.ey is set whenever H is applied
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float2 eyv = __ldg(&a.ey[col_exit_pos<N, G::L2>(i % P::T, i / P::T)]);
        ey_s[i] = fold ? cscale(eyv, a.scale) : eyv;
      }
    }
    __syncthreads();
  }
  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles) {
    mbar_arrive_expect(&bars[0], TILE_BYTES);
    for (int k = 0; k < N / G::BH; ++k)
      tma_load_3d(tiles + k * G::BH * W, &map_in, (tile % strips) * W, k * G::BH, tile / strips, &bars[0]);
  }
  bool ok = true;
  for (int i = 0; tile < ntiles && ok; ++i, tile += gridDim.x) {
    const int b = i % G::NB;
    float2* tb = tiles + b * G::TILE;
    const int next = tile + gridDim.x;
    // The next strip goes into the buffer whose store was issued at the end of the previous
    // iteration; the copy is started halfway through this strip's work (below), by when that
    // store has long been read out, so no thread waits for it.
    auto prefetch_next = [&]() {
      if constexpr (G::NB >= 2) {
        if (threadIdx.x == 0 && next < ntiles) {
          bulk_wait_read<G::NB - 2>();
          const int bn = (i + 1) % G::NB;
          mbar_arrive_expect(&bars[bn], TILE_BYTES);
          for (int k = 0; k < N / G::BH; ++k)
            tma_load_3d(tiles + bn * G::TILE + k * G::BH * W, &map_in, (next % strips) * W, k * G::BH,
                        next / strips, &bars[bn]);
        }
      }
    };
    ok = __syncthreads_and(mbar_wait_bounded(&bars[b], (i / G::NB) & 1, status));
    if (!ok) break;
    const int fb = tile / strips;  // field of the stack
    const int x = (tile % strips) * W + c;
    const bool live = x < nx;
    float2* col = tb + c;
    float2 v[E];
    if (flags & COL_FWD) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = col[slot_pos<N, RF>(t, e) * W];
      if constexpr (DITH && G::L2) {
        fft2l_fwd2x<N, NatAddr, SwzAddr, TWL, W>(v, col, t, tw, k1);
      } else if constexpr (DITH) {  // 3*2^k: the stage-major dithered table, radix-24 first stage
        __syncthreads();
        FftStages2x<N, false, 0, 1, SwzAddr, false, TWL, W, float2>::run(v, col, t, tw, k1);
      } else if constexpr (G::L2) {
        // the block exchange writes exactly the slots this thread just read: no barrier
        fft2l_fwd<N, NatAddr, SwzAddr, W, TWL>(v, col, t, tw);
      } else {
        __syncthreads();
        fft_seq<N, false, SwzAddr, W, TWL>(v, col, t, tw);
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = col[col_exit_pos<N, G::L2>(t, e) * W];
      __syncthreads();
    }
    if (flags & (COL_H | COL_MASK)) {
      const int lim = live ? __ldg(&a.ylim[x]) : -1;
      const float2 exv = ((flags & COL_H) && live) ? __ldg(&a.ex[x]) : make_float2(1.f, 0.f);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int fy = col_exit_pos<N, G::L2>(t, e);
        const int m = fy < (N + 1) / 2 ? fy : fy - N;
        if ((m < 0 ? -m : m) > lim) {
          v[e] = make_float2(0.f, 0.f);
        } else if (flags & COL_H) {
          const float2 eyv =
              G::EY_SMEM ? ey_s[e * P::T + t] : (fold ? cscale(__ldg(&a.ey[fy]), a.scale) : __ldg(&a.ey[fy]));
          if constexpr (DITH) {
            v[e] = x_mul_one(v[e], x_mul3(exv, eyv.x, eyv.y, -eyv.y));
          } else {
            v[e] = cmul(v[e], cmul(exv, eyv));
          }
        }
      }
    }
    prefetch_next();
    if ((flags & COL_SPEC) && live) {
#pragma unroll
      for (int e = 0; e < E; ++e)
        a.spec[static_cast<size_t>(fb) * a.bstride + static_cast<size_t>(col_exit_pos<N, G::L2>(t, e)) * nx + x] = v[e];
    }
    if ((flags & COL_SCALE) && !fold) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = cscale(v[e], a.scale);
    }
    if (flags & COL_INV) {
      // two-level: the last exchange read exactly the slots this thread writes back
      if constexpr (DITH && G::L2) fft2l_inv2x<N, NatAddr, SwzAddr, TWL, W>(v, col, t, tw, k1);
      else if constexpr (DITH) FftStages2x<N, true, 0, 1, SwzAddr, false, TWL, W, float2>::run(v, col, t, tw, k1);
      else if constexpr (G::L2) fft2l_inv<N, NatAddr, SwzAddr, W, TWL>(v, col, t, tw);
      else fft_seq<N, true, SwzAddr, W, TWL>(v, col, t, tw);
#pragma unroll
      for (int e = 0; e < E; ++e) col[slot_pos<N, RF>(t, e) * W] = v[e];
    } else {
      if constexpr (G::L2) __syncthreads();  // other groups may still read their exchange regions
#pragma unroll
      for (int e = 0; e < E; ++e) col[col_exit_pos<N, G::L2>(t, e) * W] = v[e];
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < N / G::BH; ++k)
        tma_store_3d(&map_out, (tile % strips) * W, k * G::BH, fb, tb + k * G::BH * W);
      bulk_commit();
      if constexpr (G::NB == 1) {
        // one buffer: the next strip lands in it once this store has read it out (the other
        // blocks of the SM compute meanwhile)
        if (next < ntiles) {
          bulk_wait_read<0>();
          mbar_arrive_expect(&bars[0], TILE_BYTES);
          for (int k = 0; k < N / G::BH; ++k)
            tma_load_3d(tiles + k * G::BH * W, &map_in, (next % strips) * W, k * G::BH, next / strips, &bars[0]);
        }
      }
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

}  // namespace rs
