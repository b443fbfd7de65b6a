// rs_rows.cu — instantiations and launcher of the fused row pass for nx = 16 .. 16384.
#include "rs_kernels.cuh"

namespace rs {

namespace {
// Rows per block: one row for nx >= 256, otherwise enough rows for 256 threads.
template <int N>
constexpr int rows_per_block() { return N >= 256 ? 1 : 256 / (N / 16); }

template <int N>
cudaError_t launch_rows_n(const RowArgs& a, cudaStream_t s) {
  constexpr int ROWS = rows_per_block<N>();
  constexpr int THREADS = ROWS * (N / 16);
  constexpr size_t SMEM = static_cast<size_t>(ROWS) * FftPlan<N>::S * sizeof(float2);
  static unsigned configured = 0;  // one bit per device ordinal
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<N, ROWS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(SMEM));
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const int blocks = (a.ny + ROWS - 1) / ROWS;
  row_pass_kernel<N, ROWS><<<blocks, THREADS, SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}
}  // namespace

bool fast_size(int n) { return n >= 16 && n <= 16384 && (n & (n - 1)) == 0; }

cudaError_t launch_row_pass(int nx, const RowArgs& a, cudaStream_t s) {
  switch (nx) {
    case 16: return launch_rows_n<16>(a, s);
    case 32: return launch_rows_n<32>(a, s);
    case 64: return launch_rows_n<64>(a, s);
    case 128: return launch_rows_n<128>(a, s);
    case 256: return launch_rows_n<256>(a, s);
    case 512: return launch_rows_n<512>(a, s);
    case 1024: return launch_rows_n<1024>(a, s);
    case 2048: return launch_rows_n<2048>(a, s);
    case 4096: return launch_rows_n<4096>(a, s);
    case 8192: return launch_rows_n<8192>(a, s);
    case 16384: return launch_rows_n<16384>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace rs
