// rs_pass_x2.cu — launchers of the split-pair multislice passes (rs_x2.cuh) for the 2^k sizes,
// and the builder of the dithered twiddle tables they read.
#include "rs_passes.cuh"
#include "rs_x2.cuh"
#include "rs_x2_api.cuh"

namespace rs {

template <int N>
cudaError_t launch_row_x2_n(const RowArgs& a, cudaStream_t s) {
  using G = RowX2Geom<N>;
  static_assert(G::SMEM <= 227 * 1024, "a row pair's exchange buffer must fit in shared memory");
  static unsigned configured = 0;  // one bit per device ordinal
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(row_x2_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(G::SMEM));
    if (e != cudaSuccess) {
      cudaGetLastError();  // leave no error behind for the caller's next check
      return e;
    }
    configured |= bit;
  }
  const int pairs = (a.ny + 1) / 2;
  row_x2_kernel<N><<<(pairs + G::PAIRS - 1) / G::PAIRS, G::THREADS, G::SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

// Blocks per SM of the split-pair column pass: two single-buffer blocks up to 2048 rows
// (2048^2 column pass 31.2 against 38.3 us, 1024^2 13.8 against 14.7), one block with two
// strip buffers at 4096 (123.5 against 140.7 us: at 128 registers the 4096-point form spills).
// RS_COLX2_MINB forces one choice for every size.
template <int N>
constexpr int col_x2_minb() {
#ifdef RS_COLX2_MINB
  return RS_COLX2_MINB;
#else
  return N <= 2048 ? 2 : 1;
#endif
}

template <int N, int MINB = col_x2_minb<N>()>
cudaError_t launch_col_x2_n(const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                            int* status, cudaStream_t s) {
  using G = ColX2Geom<N, MINB>;
  if (box.w != G::W || box.bh != G::BH) return cudaErrorInvalidValue;
  static unsigned configured = 0;
  static int grid_cache[32];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(col_x2_pipe_kernel<N, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(G::SMEM));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    grid_cache[dev & 31] = resident_grid(col_x2_pipe_kernel<N, MINB>, G::THREADS, G::SMEM, 1 << 30);
    configured |= bit;
  }
  const int tiles = (a.nx + G::W - 1) / G::W * (a.batches > 1 ? a.batches : 1);
  const int grid = tiles < grid_cache[dev & 31] ? tiles : grid_cache[dev & 31];
  col_x2_pipe_kernel<N, MINB><<<grid, G::THREADS, G::SMEM, s>>>(a, in, out, status);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

#define RS_X2_ROW_SIZES(X) X(256) X(512) X(1024) X(2048) X(4096) X(8192)
#define RS_X2_COL_SIZES(X) X(256) X(512) X(1024) X(2048) X(4096)

#define RS_X2ROW_CASE(N) \
  case N: return launch_row_x2_n<N>(a, s);
#define RS_X2COL_CASE(N) \
  case N: return launch_col_x2_n<N>(a, in, out, box, status, s);
#define RS_X2BOX_CASE(N) \
  case N: *w = ColX2Geom<N>::W; *bh = ColX2Geom<N>::BH; return true;
#define RS_X2OK_CASE(N) \
  case N: return true;

#define RS_D1COL_CASE(N) \
  case N: return launch_col_pipe_n<N, true>(a, in, out, box, status, s);
#define RS_D1BOX_CASE(N) \
  case N: *w = ColPipeGeom<N, true>::W; *bh = ColPipeGeom<N, true>::BH; return true;

// the dithered columns one per thread group also run at the 3*2^k lengths of the column pipeline
// (the one-level transform with a radix-24 first stage), which have no split-pair form
#define RS_D1_ONLY_COL_SIZES(X) X(384) X(768) X(1536) X(3072) X(6144)

cudaError_t launch_col_d1(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                          int* status, cudaStream_t s) {
  switch (ny) {
    RS_X2_COL_SIZES(RS_D1COL_CASE)
    RS_D1_ONLY_COL_SIZES(RS_D1COL_CASE)
    default: return cudaErrorInvalidValue;
  }
}

bool col_d1_box(int ny, int* w, int* bh) {
  switch (ny) {
    RS_X2_COL_SIZES(RS_D1BOX_CASE)
    RS_D1_ONLY_COL_SIZES(RS_D1BOX_CASE)
    default: return false;
  }
}

bool col_d1_only(int ny) {
  switch (ny) {
    RS_D1_ONLY_COL_SIZES(RS_X2OK_CASE)
    default: return false;
  }
}

#define RS_D1ROW_CASE(N) \
  case N: return launch_rows_nvd<N, true, true>(a, s);

// the dithered rows one per thread group also run at 16384, where a row pair does not fit shared
// memory, and at the 3*2^k lengths (radix-24 first stage), which have no split-pair form
#define RS_D1_ONLY_ROW_SIZES(X) X(16384) X(384) X(768) X(1536) X(3072) X(6144)

cudaError_t launch_row_d1(int nx, const RowArgs& a, cudaStream_t s) {
  switch (nx) {
    RS_X2_ROW_SIZES(RS_D1ROW_CASE)
    RS_D1_ONLY_ROW_SIZES(RS_D1ROW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

#define RS_D1ADJ_CASE(N) \
  case N: return launch_row_adjoint_n<N, true>(a, s);

cudaError_t launch_row_adjoint_d1(int nx, const RowArgs& a, cudaStream_t s) {
  switch (nx) {
    RS_X2_ROW_SIZES(RS_D1ADJ_CASE)
    RS_D1ADJ_CASE(16384)
    default: return cudaErrorInvalidValue;
  }
}

bool row_d1_only(int nx) {
  switch (nx) {
    RS_D1_ONLY_ROW_SIZES(RS_X2OK_CASE)
    default: return false;
  }
}

cudaError_t launch_row_x2(int nx, const RowArgs& a, cudaStream_t s) {
  switch (nx) {
    RS_X2_ROW_SIZES(RS_X2ROW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

bool row_x2_ok(int nx) {
  switch (nx) {
    RS_X2_ROW_SIZES(RS_X2OK_CASE)
    default: return false;
  }
}

cudaError_t launch_col_x2(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                          int* status, cudaStream_t s) {
  switch (ny) {
    RS_X2_COL_SIZES(RS_X2COL_CASE)
    default: return cudaErrorInvalidValue;
  }
}

bool col_x2_box(int ny, int* w, int* bh) {
  switch (ny) {
    RS_X2_COL_SIZES(RS_X2BOX_CASE)
    default: return false;
  }
}

// Largest exchange-buffer slot count of a row pair (the staged voxel row must fit in it).
int row_x2_slots(int nx) { return nx + nx / 16; }

// ---- dithered tables ----------------------------------------------------------------------
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// One component hi + lo (|lo| <= half an ulp of hi): in table j the float other than hi that
// brackets hi + lo is used when (j + offset) mod K < round(K * |lo| / ulp), so its mean over the
// K tables is hi + lo to within 1/(2K) of an ulp.
__device__ __forceinline__ float dither_pick(float hi, float lo, int j, uint32_t seed) {
  if (lo == 0.0f) return hi;
  const float other = nextafterf(hi, lo > 0.0f ? INFINITY : -INFINITY);
  const double frac = static_cast<double>(lo) / (static_cast<double>(other) - static_cast<double>(hi));
  const int n_other = static_cast<int>(rint(frac * kDitherTables));
  const int off = static_cast<int>(mix32(seed) % kDitherTables);
  return ((j + off) % kDitherTables) < n_other ? other : hi;
}

// From a compensated table (hi.x, hi.y, lo.x, lo.y) of `len` entries: kDitherTables tables of
// (wr, wr, wi, wi) entries, table j at out + j * len.
__global__ void dither_tables_kernel(const float4* comp, float4* out, int len) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  const float4 w = comp[i];
  for (int j = 0; j < kDitherTables; ++j) {
    const float wr = dither_pick(w.x, w.z, j, 2u * static_cast<uint32_t>(i) + 1u);
    const float wi = dither_pick(w.y, w.w, j, 2u * static_cast<uint32_t>(i) + 0x9e3779b9u);
    out[static_cast<size_t>(j) * len + i] = make_float4(wr, wr, wi, wi);
  }
}

// The (wr, wi) lanes of split-pair table entries (wr, wr, wi, wi): the single-sequence tables.
__global__ void single_tables_kernel(const float4* in, float2* out, size_t n) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 w = in[i];
  out[i] = make_float2(w.x, w.z);
}

cudaError_t launch_single_tables(const float4* in, float2* out, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  single_tables_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(in, out, n);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

cudaError_t launch_dither_tables(const float4* comp, float4* out, int len, cudaStream_t s) {
  if (len <= 0) return cudaSuccess;
  dither_tables_kernel<<<(len + 255) / 256, 256, 0, s>>>(comp, out, len);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

}  // namespace rs
