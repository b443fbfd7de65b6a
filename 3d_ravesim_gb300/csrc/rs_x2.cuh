// rs_x2.cuh — the fused multislice passes on split pairs (rs_fft2x.cuh): each thread group
// transforms two rows, or the two columns of a strip pair, at once, with the slice's dithered
// twiddle table. Same data flow as row_pass_kernel<N, ROWS, true> and col_pipe_kernel<N>:
//   row pass    : [row IFFT] -> voxel transmission -> row FFT
//   column pass : column FFT -> H(fx, fy) * mask / N -> column IFFT  (+ spectrum on the last slice)
// which compute u_{k+1} = IFFT2[H * FFT2[T_k u_k]] (big-wave/propagation.py:396-442 after the
// transmission multiply of big-wave/optical_element.py:565-584).
#pragma once
#include "rs_pipe.cuh"

namespace rs {

// ------------------------------------------------------------------------------- row pass
template <int N>
struct RowX2Geom {
  using P = FftPlan<N>;
  static constexpr int T = P::T;
  static constexpr int PAIRS = T >= 256 ? 1 : 256 / T;  // row pairs per block
  static constexpr int THREADS = PAIRS * T;
  static constexpr int S = P::S;                        // exchange slots (cp2) per pair
  static constexpr int PF_WORDS = 2 * S < 2048 ? 2 * S : 2048;  // prefetch words per pair: 4 voxel rows
  static constexpr size_t SMEM = static_cast<size_t>(PAIRS) * (static_cast<size_t>(S) * sizeof(cp2) + PF_WORDS * 4);
  static constexpr int MINB = SMEM * 3 <= 227 * 1024 ? 3 : SMEM * 2 <= 227 * 1024 ? 2 : 1;
};

// Voxel rows (yi, yi + 1) of one sim row blended in y at voxel column j, from the prefetched copy
// (ids or per-voxel (delta, beta)) or from global memory.
__device__ __forceinline__ float2 x2_col_blend(const VoxelArgs& v, const uint32_t* pf, int j, int yi, float fy) {
  if (pf) {
    const int nxv = v.nxv;
    float2 d0, d1;
    if (v.dbv) {
      const float2* r = reinterpret_cast<const float2*>(pf);
      d0 = r[j];
      if (fy == 0.0f) return d0;
      d1 = r[nxv + j];
    } else {
      d0 = db_of_id(v, pf[j]);
      if (fy == 0.0f) return d0;
      d1 = db_of_id(v, pf[nxv + j]);
    }
    return lerp2(d0, d1, fy);
  }
  return voxel_col_blend(v, j, yi, fy);
}

// Flags: ROW_INV (inverse transform first, with twd_inv), ROW_STORE_U (the spatial rows entering
// the transmission to aux), ROW_TVOX (voxel transmission), ROW_FWD (forward transform last, with
// twd_fwd), ROW_SCALE. Rows 2p and 2p + 1 form pair p.
template <int N>
__global__ void __launch_bounds__(RowX2Geom<N>::THREADS, RowX2Geom<N>::MINB) row_x2_kernel(const RowArgs a) {
  using P = FftPlan<N>;
  using G = RowX2Geom<N>;
  constexpr int T = P::T;
  constexpr int RF = P::entry_radix(false);
  constexpr int RX = P::exit_radix(false);
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int t = threadIdx.x % T;
  const int lp = threadIdx.x / T;
  const int rowA = 2 * (blockIdx.x * G::PAIRS + lp);
  const int rowB = rowA + 1;
  const bool validA = rowA < a.ny, validB = rowB < a.ny;
  cp2* buf = reinterpret_cast<cp2*>(smem_raw) + lp * G::S;
  uint32_t* pfa = reinterpret_cast<uint32_t*>(smem_raw + G::PAIRS * G::S * sizeof(cp2)) + lp * G::PF_WORDS;
  const int flags = a.flags;
  const bool tvox = flags & ROW_TVOX;

  int yiA = -1, yiB = -1;
  float fyA = 0.0f, fyB = 0.0f;
  const uint32_t* pfA = nullptr;
  const uint32_t* pfB = nullptr;
  if (tvox) {
    if (validA) {
      const int ar = a.axis_rows ? rowA % a.axis_rows : rowA;
      yiA = __ldg(&a.ax.yi[ar]);
      if (yiA >= 0) fyA = __ldg(&a.ax.yf[ar]);
    }
    if (validB) {
      const int br = a.axis_rows ? rowB % a.axis_rows : rowB;
      yiB = __ldg(&a.ax.yi[br]);
      if (yiB >= 0) fyB = __ldg(&a.ax.yf[br]);
    }
    // the two voxel rows of each sim row, copied asynchronously while the inverse transform runs
    const int w = a.vox.dbv ? 2 : 1;
    const int words = 2 * a.vox.nxv * w;  // two voxel rows
    if (2 * words <= G::PF_WORDS) {        // block-uniform
      const uint32_t* src = a.vox.dbv ? reinterpret_cast<const uint32_t*>(a.vox.dbv)
                                      : static_cast<const uint32_t*>(a.vox.slice);
      if (yiA >= 0) {
        const uint32_t* s0 = src + static_cast<size_t>(yiA) * a.vox.nxv * w;
        for (int i = t; i < words; i += T) cp_async4(pfa + i, s0 + i);
        pfA = pfa;
      }
      if (yiB >= 0) {
        const uint32_t* s1 = src + static_cast<size_t>(yiB) * a.vox.nxv * w;
        for (int i = t; i < words; i += T) cp_async4(pfa + words + i, s1 + i);
        pfB = pfa + words;
      }
    }
  }

  const float2* inA = a.in + static_cast<size_t>(validA ? rowA : 0) * N;
  const float2* inB = a.in + static_cast<size_t>(validB ? rowB : 0) * N;
  cp2 v[16];
  const bool inv = flags & ROW_INV;
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const int pos = inv ? slot_pos<N, RX>(t, e) : slot_pos<N, RF>(t, e);
    const float2 fa = validA ? inA[pos] : make_float2(0.f, 0.f);
    const float2 fb = validB ? inB[pos] : make_float2(0.f, 0.f);
    v[e] = cp2{make_float2(fa.x, fb.x), make_float2(fa.y, fb.y)};
  }
  if (inv) fft_seq2x<N, true>(v, buf, t, a.twd_inv, dft_k(a.k_inv));
  if (flags & ROW_STORE_U) {  // the spatial rows entering the transmission (for the adjoint sweep)
    float2* auxA = a.aux + static_cast<size_t>(validA ? rowA : 0) * N;
    float2* auxB = a.aux + static_cast<size_t>(validB ? rowB : 0) * N;
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const int pos = slot_pos<N, RF>(t, e);
      if (validA) auxA[pos] = make_float2(v[e].re.x, v[e].im.x);
      if (validB) auxB[pos] = make_float2(v[e].re.y, v[e].im.y);
    }
  }

  if (tvox) {
    // The exchange buffer is idle between the transforms: stage the y-blended voxel rows of both
    // sim rows there as {deltaA, betaA, deltaB, betaB} per voxel column, then interpolate in x.
    const int nxv = a.vox.nxv;
    cp_async_wait_all();
    __syncthreads();
    float4* vrow = reinterpret_cast<float4*>(buf);
    for (int j = t; j < nxv; j += T) {
      const float2 dA = yiA >= 0 ? x2_col_blend(a.vox, pfA, j, yiA, fyA) : make_float2(0.f, 0.f);
      const float2 dB = yiB >= 0 ? x2_col_blend(a.vox, pfB, j, yiB, fyB) : make_float2(0.f, 0.f);
      vrow[j] = make_float4(dA.x, dA.y, dB.x, dB.y);
    }
    __syncthreads();
    const float at = a.vox.a;
#pragma unroll
    for (int c0 = 0; c0 < 16; c0 += 8) {
      float4 d[8];
      bool any = false;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        d[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int x = slot_pos<N, RF>(t, c0 + i);
        const int2 xe = (yiA >= 0 || yiB >= 0) ? __ldg(&a.ax.xp[x]) : make_int2(-1, 0);
        if (xe.x >= 0) {
          const float fx = __int_as_float(xe.y);
          const float4 q0 = vrow[xe.x], q1 = vrow[xe.x + 1];
          const float2 dA = lerp2(make_float2(q0.x, q0.y), make_float2(q1.x, q1.y), fx);
          const float2 dB = lerp2(make_float2(q0.z, q0.w), make_float2(q1.z, q1.w), fx);
          d[i] = make_float4(dA.x, dA.y, dB.x, dB.y);
          any |= ((__float_as_uint(dA.x) | __float_as_uint(dA.y) | __float_as_uint(dB.x) | __float_as_uint(dB.y))
                  << 1) != 0u;  // +-0 is vacuum
        }
      }
      if (__any_sync(0xffffffffu, any)) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const cp2 tr = material_factor2(make_float2(d[i].x, d[i].y), make_float2(d[i].z, d[i].w), at);
          v[c0 + i] = x_mul_pair(v[c0 + i], tr);
        }
      }
    }
    __syncthreads();  // the forward transform reuses the buffer
  }

  float2* outA = a.out + static_cast<size_t>(validA ? rowA : 0) * N;
  float2* outB = a.out + static_cast<size_t>(validB ? rowB : 0) * N;
  const bool fwd = flags & ROW_FWD;
  if (fwd) fft_seq2x<N, false>(v, buf, t, a.twd_fwd, dft_k(a.k_fwd));
  const float2 sc = make_float2(a.scale, a.scale);
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const int pos = fwd ? slot_pos<N, RX>(t, e) : slot_pos<N, RF>(t, e);
    cp2 o = v[e];
    if (flags & ROW_SCALE) o = cp2{p_mul(o.re, sc), p_mul(o.im, sc)};
    if (validA) outA[pos] = make_float2(o.re.x, o.im.x);
    if (validB) outB[pos] = make_float2(o.re.y, o.im.y);
  }
}

// --------------------------------------------------------------------------- column pass
// MINB = 1: one block per SM with two or three strip buffers and the (wr, wr, wi, wi) table.
// MINB = 2: two blocks per SM, each with one strip buffer (the other block computes while one
// waits for its next strip), the half-size (wr, wi) table and half the register file.
template <int N, int MINB = 1>
struct ColX2Geom {
  using P = FftPlan<N>;
  static constexpr int T = P::T;
  static constexpr int PAIRS = T >= 256 ? 1 : 256 / T;  // column pairs per strip
  static constexpr int W = 2 * PAIRS;                   // columns per strip
  static constexpr int THREADS = PAIRS * T;
  static constexpr int GROUPS = 1;
  static constexpr int BH = box_rows(N);
  static_assert(N % BH == 0, "the boxes must tile a column exactly");
  static constexpr int TILE = W * N;  // float2 per tile buffer
  static constexpr bool L2 = Fft2L<N>::ok(PAIRS);
  static_assert(L2, "the split-pair column pass uses the two-level transform");
  static constexpr bool HALF_TW = MINB >= 2;
  using TwT = typename std::conditional<HALF_TW, float2, float4>::type;
  static constexpr int TW_LEN = Fft2L<N>::TW_LEN;
  static constexpr size_t TW_BYTES = static_cast<size_t>(TW_LEN) * sizeof(TwT);
  static constexpr size_t BUDGET = 227 * 1024 / MINB;
  static constexpr int NB = MINB >= 2 ? 1 : (3 * TILE * 8 + TW_BYTES + 64 <= BUDGET) ? 3 : 2;
  static constexpr size_t TILES_BYTES = static_cast<size_t>(NB) * TILE * sizeof(float2);
  static constexpr bool TW_SMEM = TILES_BYTES + TW_BYTES + 64 <= BUDGET;
  static constexpr size_t EY_BYTES = static_cast<size_t>(N) * sizeof(float2);
  static constexpr bool EY_SMEM = TILES_BYTES + (TW_SMEM ? TW_BYTES : 0) + EY_BYTES + 64 <= BUDGET;
  static constexpr size_t SMEM =
      TILES_BYTES + (TW_SMEM ? TW_BYTES : 0) + (EY_SMEM ? EY_BYTES : 0) + NB * sizeof(uint64_t);
};

// Flags: COL_FWD | COL_H | COL_SCALE | COL_INV, optionally COL_SPEC (the multislice column pass).
template <int N, int MINB = 1>
__global__ void __launch_bounds__(ColX2Geom<N, MINB>::THREADS, MINB)
    col_x2_pipe_kernel(const ColArgs a, const __grid_constant__ CUtensorMap map_in,
                       const __grid_constant__ CUtensorMap map_out, int* status) {
  using P = FftPlan<N>;
  using G = ColX2Geom<N, MINB>;
  using TwT = typename G::TwT;
  constexpr int W = G::W;
  constexpr int PAIRS = G::PAIRS;
  constexpr int RF = P::entry_radix(false);
  constexpr uint32_t TILE_BYTES = G::TILE * 8u;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* tiles = reinterpret_cast<float2*>(smem_raw);
  TwT* tw_s = reinterpret_cast<TwT*>(smem_raw + G::TILES_BYTES);
  float2* ey_s = reinterpret_cast<float2*>(smem_raw + G::TILES_BYTES + (G::TW_SMEM ? G::TW_BYTES : 0));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + G::TILES_BYTES + (G::TW_SMEM ? G::TW_BYTES : 0) +
                                               (G::EY_SMEM ? G::EY_BYTES : 0));
  const int p = threadIdx.x % PAIRS;  // pair within the strip
  const int t = threadIdx.x / PAIRS;
  const int nx = a.nx;
  // tiles run over the strips of every field of a stack (the maps are 3D: x, y, field)
  const int strips = (nx + W - 1) / W;
  const int ntiles = strips * (a.batches > 1 ? a.batches : 1);
  const int flags = a.flags;
  if (threadIdx.x == 0) {
    for (int b = 0; b < G::NB; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (a.test_stall) {
    mbar_wait_bounded(&bars[0], 0, status, kTestSpinLimit);
    return;
  }
  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles) {  // the first strip, before the tables are staged
    mbar_arrive_expect(&bars[0], TILE_BYTES);
    for (int kb = 0; kb < N / G::BH; ++kb)
      tma_load_3d(tiles + kb * G::BH * W, &map_in, (tile % strips) * W, kb * G::BH, tile / strips, &bars[0]);
  }
  const TwT* tw_g;
  if constexpr (G::HALF_TW) {
    tw_g = a.twd1;
  } else {
    tw_g = a.twd;
  }
  if constexpr (G::TW_SMEM) {
    for (int i = threadIdx.x; i < G::TW_LEN; i += blockDim.x) tw_s[i] = __ldg(&tw_g[i]);
  }
  const TwT* tw = G::TW_SMEM ? tw_s : tw_g;
  using TWL = typename std::conditional<G::TW_SMEM, TwShared, TwGlobal>::type;
  const bool fold = (flags & COL_H) && (flags & COL_SCALE) && !(flags & COL_SPEC);
  if constexpr (G::EY_SMEM) {
    if (flags & COL_H) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float2 eyv = __ldg(&a.ey[col_exit_pos<N, true>(i % P::T, i / P::T)]);
        ey_s[i] = fold ? cscale(eyv, a.scale) : eyv;
      }
    }
  }
  __syncthreads();
  const DftK k = dft_k(a.kc);
  bool ok = true;
  for (int i = 0; tile < ntiles && ok; ++i, tile += gridDim.x) {
    const int b = i % G::NB;
    float2* tb = tiles + b * G::TILE;
    const int next = tile + gridDim.x;
    auto prefetch_next = [&]() {
      if constexpr (G::NB >= 2) {
        if (threadIdx.x == 0 && next < ntiles) {
          bulk_wait_read<G::NB - 2>();
          const int bn = (i + 1) % G::NB;
          mbar_arrive_expect(&bars[bn], TILE_BYTES);
          for (int kb = 0; kb < N / G::BH; ++kb)
            tma_load_3d(tiles + bn * G::TILE + kb * G::BH * W, &map_in, (next % strips) * W, kb * G::BH,
                        next / strips, &bars[bn]);
        }
      }
    };
    const int fb = tile / strips;  // field of the stack
    const int xA = (tile % strips) * W + 2 * p;
    const int xB = xA + 1;
    const bool liveA = xA < nx, liveB = xB < nx;
    // the strip's per-column tables, fetched while its copy lands
    const int limA = liveA ? __ldg(&a.ylim[xA]) : -1;
    const int limB = liveB ? __ldg(&a.ylim[xB]) : -1;
    const float2 exA = ((flags & COL_H) && liveA) ? __ldg(&a.ex[xA]) : make_float2(1.f, 0.f);
    const float2 exB = ((flags & COL_H) && liveB) ? __ldg(&a.ex[xB]) : make_float2(1.f, 0.f);
    ok = __syncthreads_and(mbar_wait_bounded(&bars[b], (i / G::NB) & 1, status));
    if (!ok) break;
    // strip slots: position y of pair p holds {A.re, A.im, B.re, B.im} at cp2 index y*PAIRS + p
    cp2* col = reinterpret_cast<cp2*>(tb) + p;
    cp2 v[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const cp2 q = col[slot_pos<N, RF>(t, e) * PAIRS];
      v[e] = cp2{make_float2(q.re.x, q.im.x), make_float2(q.re.y, q.im.y)};
    }
    // the block exchange writes exactly the slots this thread just read: no barrier
    fft2l_fwd2x<N, NatAddr, SwzAddr, TWL, PAIRS>(v, col, t, tw, k);
    if (flags & (COL_H | COL_MASK)) {
      const cp2 ex = cp2{make_float2(exA.x, exB.x), make_float2(exA.y, exB.y)};
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int fy = col_exit_pos<N, true>(t, e);
        const int m = fy < (N + 1) / 2 ? fy : fy - N;
        const int am = m < 0 ? -m : m;
        if (flags & COL_H) {
          const float2 eyv =
              G::EY_SMEM ? ey_s[e * P::T + t] : (fold ? cscale(__ldg(&a.ey[fy]), a.scale) : __ldg(&a.ey[fy]));
          const cp2 h = x_mul3(ex, make_float2(eyv.x, eyv.x), make_float2(eyv.y, eyv.y),
                               make_float2(-eyv.y, -eyv.y));
          v[e] = x_mul_pair(v[e], h);
        }
        if (am > limA) v[e].re.x = v[e].im.x = 0.f;
        if (am > limB) v[e].re.y = v[e].im.y = 0.f;
      }
    }
    prefetch_next();
    if (flags & COL_SPEC) {
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const size_t r = static_cast<size_t>(fb) * a.bstride + static_cast<size_t>(col_exit_pos<N, true>(t, e)) * nx;
        if (liveA) a.spec[r + xA] = make_float2(v[e].re.x, v[e].im.x);
        if (liveB) a.spec[r + xB] = make_float2(v[e].re.y, v[e].im.y);
      }
    }
    if ((flags & COL_SCALE) && !fold) {
      const float2 sc = make_float2(a.scale, a.scale);
#pragma unroll
      for (int e = 0; e < 16; ++e) v[e] = cp2{p_mul(v[e].re, sc), p_mul(v[e].im, sc)};
    }
    // two-level inverse: the last exchange read exactly the slots this thread writes back
    fft2l_inv2x<N, NatAddr, SwzAddr, TWL, PAIRS>(v, col, t, tw, k);
#pragma unroll
    for (int e = 0; e < 16; ++e)
      col[slot_pos<N, RF>(t, e) * PAIRS] = cp2{make_float2(v[e].re.x, v[e].im.x), make_float2(v[e].re.y, v[e].im.y)};
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int kb = 0; kb < N / G::BH; ++kb)
        tma_store_3d(&map_out, (tile % strips) * W, kb * G::BH, fb, tb + kb * G::BH * W);
      bulk_commit();
      if constexpr (G::NB == 1) {
        // one buffer: the next strip lands in it once this store has read it out
        if (next < ntiles) {
          bulk_wait_read<0>();
          mbar_arrive_expect(&bars[0], TILE_BYTES);
          for (int kb = 0; kb < N / G::BH; ++kb)
            tma_load_3d(tiles + kb * G::BH * W, &map_in, (next % strips) * W, kb * G::BH, next / strips, &bars[0]);
        }
      }
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

}  // namespace rs
