// rs_dispatch.cu — size dispatch of the fused passes over the two size families.
#include "rs_passes.cuh"

namespace rs {

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

bool fast_size(int n) {
  if (n < 16) return false;
  if (is_pow2(n)) return n <= 16384;
  return n % 3 == 0 && is_pow2(n / 3) && n >= 24 && n <= 12288;
}

cudaError_t launch_row_pass(int nx, const RowArgs& a, cudaStream_t s, bool vox) {
  return is_pow2(nx) ? launch_row_pass_pow2(nx, a, vox, s) : launch_row_pass_pow3(nx, a, vox, s);
}

cudaError_t launch_row_adjoint(int nx, const RowArgs& a, cudaStream_t s) {
  return is_pow2(nx) ? launch_row_adjoint_pow2(nx, a, s) : cudaErrorInvalidValue;
}

cudaError_t launch_col_pass(int ny, const ColArgs& a, cudaStream_t s) {
  return is_pow2(ny) ? launch_col_pass_pow2(ny, a, s) : launch_col_pass_pow3(ny, a, s);
}

__global__ void power_twiddles_kernel(float4* tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n) tw[m] = twiddle_fp64(m, n);
}

cudaError_t launch_power_twiddles(int n, float4* tw, cudaStream_t s) {
  if (!is_pow2(n)) return cudaErrorInvalidValue;
  power_twiddles_kernel<<<(n + 255) / 256, 256, 0, s>>>(tw, n);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) note_launch();
  return e;
}

cudaError_t launch_stage_twiddles(int n, float4* tw, cudaStream_t s) {
  return is_pow2(n) ? launch_stage_twiddles_pow2(n, tw, s) : launch_stage_twiddles_pow3(n, tw, s);
}

int stage_twiddle_len(int n) { return is_pow2(n) ? stage_twiddle_len_pow2(n) : stage_twiddle_len_pow3(n); }

int twiddles_2l_len(int n) { return is_pow2(n) ? twiddles_2l_len_pow2(n) : 0; }
cudaError_t launch_twiddles_2l(int n, float4* tw, cudaStream_t s) {
  return is_pow2(n) ? launch_twiddles_2l_pow2(n, tw, s) : cudaErrorInvalidValue;
}

bool row_pipe_ok(int n) { return is_pow2(n) ? row_pipe_ok_pow2(n) : row_pipe_ok_pow3(n); }
bool col_pipe_box(int n, int* w, int* bh) { return is_pow2(n) ? col_pipe_box_pow2(n, w, bh) : col_pipe_box_pow3(n, w, bh); }

cudaError_t launch_row_pipe(int nx, const RowArgs& a, int* status, cudaStream_t s) {
  return is_pow2(nx) ? launch_row_pipe_pow2(nx, a, status, s) : launch_row_pipe_pow3(nx, a, status, s);
}

cudaError_t launch_col_pipe(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                            int* status, cudaStream_t s) {
  return is_pow2(ny) ? launch_col_pipe_pow2(ny, a, in, out, box, status, s)
                     : launch_col_pipe_pow3(ny, a, in, out, box, status, s);
}

}  // namespace rs
