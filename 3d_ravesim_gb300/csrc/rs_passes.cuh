// rs_passes.cuh — launch templates of the fused row / column passes and of the stage-major
// twiddle tables. rs_pass_pow{2,3}_{rows,cols}.cu instantiate them for the two size
// families (2^k and 3*2^k) in separate translation units that compile in parallel.
#pragma once
#include "rs_pipe.cuh"

namespace rs {

// Rows per block: one row when a row has >= RS_ROW_THREADS threads, otherwise enough rows for
// about that many threads (128: twice as many blocks of short rows as with 256, which fills the
// SMs better at 1024..3072: row passes 4-7.5 % faster; 4096 and up are one row per block anyway).
#ifndef RS_ROW_THREADS
#define RS_ROW_THREADS 128
#endif
template <int N>
constexpr int rows_per_block() {
  return FftPlan<N>::T >= RS_ROW_THREADS ? 1 : RS_ROW_THREADS / FftPlan<N>::T;
}

#ifndef RS_ROW_VOXMODE
#define RS_ROW_VOXMODE 1
#endif
template <int N, bool VOX, bool DITH>
cudaError_t launch_rows_nvd(const RowArgs& a, cudaStream_t s) {
  constexpr int ROWS = rows_per_block<N>();
  constexpr int THREADS = ROWS * FftPlan<N>::T;
  constexpr size_t SMEM = RowGeom<N, ROWS>::SMEM;
  static unsigned configured = 0;  // one bit per device ordinal
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<N, ROWS, VOX, DITH>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(SMEM));
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const int blocks = (a.ny + ROWS - 1) / ROWS;
  row_pass_kernel<N, ROWS, VOX, DITH><<<blocks, THREADS, SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

template <int N, bool VOX>
cudaError_t launch_rows_nv(const RowArgs& a, cudaStream_t s) {
  return launch_rows_nvd<N, VOX, false>(a, s);
}

// The voxel-transmission specialisation takes the multislice hot path and the plain row
// transforms (flags within INV | FWD | TVOX | STORE_U | SCALE) unless the caller's schedule turns
// it off for the multislice rows (vox = false, TVOX set); the point source (SRC) and the in-row
// plasma transmission (TPLASMA) run the general kernel.
template <int N>
cudaError_t launch_rows_n(const RowArgs& a, bool vox, cudaStream_t s) {
  constexpr int HOT = ROW_INV | ROW_FWD | ROW_TVOX | ROW_STORE_U | ROW_SCALE;
  const bool hot = !(a.flags & ~HOT) && (vox || !(a.flags & ROW_TVOX));
  if (RS_ROW_VOXMODE && hot) return launch_rows_nv<N, true>(a, s);
  return launch_rows_nv<N, false>(a, s);
}

template <int N, bool DITH = false>
cudaError_t launch_row_adjoint_n(const RowArgs& a, cudaStream_t s) {
  constexpr int ROWS = rows_per_block<N>();
  constexpr int THREADS = ROWS * FftPlan<N>::T;
  constexpr size_t SMEM = static_cast<size_t>(ROWS) * FftPlan<N>::S * sizeof(float2);
  static unsigned configured = 0;  // one bit per device ordinal
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(row_adjoint_kernel<N, ROWS, DITH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(SMEM));
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  row_adjoint_kernel<N, ROWS, DITH><<<(a.ny + ROWS - 1) / ROWS, THREADS, SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

// exp(-2*pi*i*m/N) evaluated in FP64, split into a float and the float of its residual.
__device__ __forceinline__ float4 twiddle_fp64(long long m, int n) {
  double sn, cs;
  sincospi(-2.0 * static_cast<double>(m) / static_cast<double>(n), &sn, &cs);
  const float ch = static_cast<float>(cs), sh = static_cast<float>(sn);
  return make_float4(ch, sh, static_cast<float>(cs - static_cast<double>(ch)),
                     static_cast<float>(sn - static_cast<double>(sh)));
}

// Entry i of FftPlan<N>'s stage-major tables (forward plan, then inverse plan).
template <int N>
__device__ __forceinline__ float4 stage_twiddle(int i) {
  using P = FftPlan<N>;
  constexpr int NF = P::table_len(false);
  const bool inv = i >= NF;
  const int j = inv ? i - NF : i;
  int s = 1;
  while (s + 1 < P::NST && P::stage_offset(inv, s + 1) <= j) ++s;
  const int ns = P::ns(inv, s);
  const int r = (j - P::stage_offset(inv, s)) / ns + 1;
  const int k = (j - P::stage_offset(inv, s)) % ns;
  return twiddle_fp64(static_cast<long long>(r) * k * (N / (ns * P::radix(inv, s))), N);
}

template <int N>
__global__ void stage_twiddles_kernel(float4* tw) {
  using P = FftPlan<N>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P::table_len(false) + P::table_len(true)) return;
  tw[i] = stage_twiddle<N>(i);
}

// Two-level table (Fft2L<N>): W_N^{c m} at (c-1)*T + m, then FftPlan<T>'s stage-major table.
template <int N>
__global__ void twiddles_2l_kernel(float4* tw) {
  using F = Fft2L<N>;
  constexpr int T = F::T;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F::TW_LEN) return;
  if (i < 15 * T) tw[i] = twiddle_fp64(static_cast<long long>(i / T + 1) * (i % T), N);
  else tw[i] = stage_twiddle<T>(i - 15 * T);
}

template <int N>
cudaError_t launch_twiddles_2l_n(float4* tw, cudaStream_t s) {
  if constexpr (!Fft2L<N>::POW2 || Fft2L<N>::T < 16) {
    return cudaErrorInvalidValue;
  } else {
    twiddles_2l_kernel<N><<<(Fft2L<N>::TW_LEN + 255) / 256, 256, 0, s>>>(tw);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
    return e;
  }
}

template <int N>
cudaError_t launch_stage_twiddles_n(float4* tw, cudaStream_t s) {
  constexpr int total = FftPlan<N>::table_len(false) + FftPlan<N>::table_len(true);
  if (total == 0) return cudaSuccess;
  stage_twiddles_kernel<N><<<(total + 255) / 256, 256, 0, s>>>(tw);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

template <int N>
constexpr int stage_twiddle_len_n() { return FftPlan<N>::table_len(false) + FftPlan<N>::table_len(true); }


// Columns per block: W*T threads (T = threads per column), capped at 512 threads so that the
// 16 or 24 complex values each thread keeps in registers fit without spilling, and W <= 16.
template <int N>
constexpr int strip_width() {
  constexpr int t = FftPlan<N>::T;
  constexpr int w = t >= 512 ? 1 : 512 / t;
  return w > 16 ? 16 : w;
}

template <int N, int W>
cudaError_t launch_cols_nw(const ColArgs& a, cudaStream_t s) {
  using G = ColGeom<N, W>;
  static unsigned configured = 0;  // one bit per device ordinal
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(col_pass_kernel<N, W>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(G::SMEM));
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const dim3 grid((a.nx + W - 1) / W, a.batches > 0 ? a.batches : 1);
  col_pass_kernel<N, W><<<grid, G::THREADS, G::SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}


// Persistent pipelined passes: one launch covers all tiles with (SMs x resident blocks) blocks.
template <class K>
int resident_grid(K kernel, int threads, size_t smem, int tiles) {
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  return tiles < sms * per_sm ? tiles : sms * per_sm;
}

template <int N>
cudaError_t launch_row_pipe_n(const RowArgs& a, int* status, cudaStream_t s) {
  using G = RowPipeGeom<N>;
  static unsigned configured = 0;
  static int grid_cache[32];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(row_pipe_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(G::SMEM));
    if (e != cudaSuccess) return e;
    grid_cache[dev & 31] = resident_grid(row_pipe_kernel<N>, G::THREADS, G::SMEM, 1 << 30);
    configured |= bit;
  }
  const int tiles = (a.ny + G::RW - 1) / G::RW;
  const int grid = tiles < grid_cache[dev & 31] ? tiles : grid_cache[dev & 31];
  row_pipe_kernel<N><<<grid, G::THREADS, G::SMEM, s>>>(a, status);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

template <int N, bool DITH = false>
cudaError_t launch_col_pipe_n(const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                              int* status, cudaStream_t s) {
  using G = ColPipeGeom<N, DITH>;
  if (box.w != G::W || box.bh != G::BH) return cudaErrorInvalidValue;
  static unsigned configured = 0;
  static int grid_cache[32];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(col_pipe_kernel<N, DITH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(G::SMEM));
    if (e != cudaSuccess) {
      cudaGetLastError();  // leave no error behind for the caller's next check
      return e;
    }
    grid_cache[dev & 31] = resident_grid(col_pipe_kernel<N, DITH>, G::THREADS, G::SMEM, 1 << 30);
    configured |= bit;
  }
  const int tiles = (a.nx + G::W - 1) / G::W * (a.batches > 1 ? a.batches : 1);
  const int grid = tiles < grid_cache[dev & 31] ? tiles : grid_cache[dev & 31];
  col_pipe_kernel<N, DITH><<<grid, G::THREADS, G::SMEM, s>>>(a, in, out, status);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

// Sizes with a pipelined variant: rows need 3 tile buffers of >= 1 row; columns need strips of
// >= 2 columns (16-byte tensor-copy boxes) with <= 512 threads.
#define RS_POW2_PIPE_ROW(X) X(256) X(512) X(1024) X(2048) X(4096) X(8192)
#define RS_POW2_PIPE_COL(X) X(256) X(512) X(1024) X(2048) X(4096)
#define RS_POW3_PIPE_ROW(X) X(384) X(768) X(1536) X(3072) X(6144)
#define RS_POW3_PIPE_COL(X) X(384) X(768) X(1536) X(3072) X(6144)

cudaError_t launch_row_pipe_pow2(int n, const RowArgs& a, int* status, cudaStream_t s);
cudaError_t launch_row_pipe_pow3(int n, const RowArgs& a, int* status, cudaStream_t s);
cudaError_t launch_col_pipe_pow2(int n, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out,
                                 StripBox box, int* status, cudaStream_t s);
cudaError_t launch_col_pipe_pow3(int n, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out,
                                 StripBox box, int* status, cudaStream_t s);
// box of the compensated column pipeline for length n: columns per strip and rows per copy;
// false if none.
bool col_pipe_box_pow2(int n, int* w, int* bh);
bool col_pipe_box_pow3(int n, int* w, int* bh);
bool row_pipe_ok_pow2(int n);
bool row_pipe_ok_pow3(int n);

#define RS_POW2_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192) X(16384)
#define RS_POW3_SIZES(X) X(24) X(48) X(96) X(192) X(384) X(768) X(1536) X(3072) X(6144) X(12288)

// Per-family dispatchers (rs_pass_pow{2,3}_{rows,cols}.cu); return cudaErrorInvalidValue
// for a size outside the family.
cudaError_t launch_row_pass_pow2(int n, const RowArgs& a, bool vox, cudaStream_t s);
cudaError_t launch_row_adjoint_pow2(int n, const RowArgs& a, cudaStream_t s);
cudaError_t launch_row_pass_pow3(int n, const RowArgs& a, bool vox, cudaStream_t s);
cudaError_t launch_col_pass_pow2(int n, const ColArgs& a, cudaStream_t s);
cudaError_t launch_col_pass_pow3(int n, const ColArgs& a, cudaStream_t s);
cudaError_t launch_stage_twiddles_pow2(int n, float4* tw, cudaStream_t s);
// Two-level column-transform table (power-of-two n >= 256); length 0 when n has none.
int twiddles_2l_len_pow2(int n);
cudaError_t launch_twiddles_2l_pow2(int n, float4* tw, cudaStream_t s);
cudaError_t launch_stage_twiddles_pow3(int n, float4* tw, cudaStream_t s);
int stage_twiddle_len_pow2(int n);
int stage_twiddle_len_pow3(int n);

}  // namespace rs
