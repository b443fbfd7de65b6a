// rs_cols.cu — instantiations and launcher of the fused column pass for ny = 16 .. 16384.
#include "rs_kernels.cuh"

namespace rs {

// Columns per block: W*N/16 threads, capped at 512 threads so that the 16 complex values
// each thread keeps in registers fit without spilling: W = 8192/N for N >= 512, 16 below.
int col_strip_width(int ny) {
  if (ny >= 8192) return 1;
  if (ny >= 512) return 8192 / ny;
  return 16;
}

namespace {
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
  if (a.nx % W != 0) return cudaErrorInvalidValue;
  col_pass_kernel<N, W><<<a.nx / W, G::THREADS, G::SMEM, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}
}  // namespace

cudaError_t launch_col_pass(int ny, const ColArgs& a, cudaStream_t s) {
  switch (ny) {
    case 16: return launch_cols_nw<16, 16>(a, s);
    case 32: return launch_cols_nw<32, 16>(a, s);
    case 64: return launch_cols_nw<64, 16>(a, s);
    case 128: return launch_cols_nw<128, 16>(a, s);
    case 256: return launch_cols_nw<256, 16>(a, s);
    case 512: return launch_cols_nw<512, 16>(a, s);
    case 1024: return launch_cols_nw<1024, 8>(a, s);
    case 2048: return launch_cols_nw<2048, 4>(a, s);
    case 4096: return launch_cols_nw<4096, 2>(a, s);
    case 8192: return launch_cols_nw<8192, 1>(a, s);
    case 16384: return launch_cols_nw<16384, 1>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace rs
