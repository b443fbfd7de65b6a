// rs_pass_pow2_rows.cu — row-pass instantiations (fused, adjoint, pipelined) for the 2^k sizes.
#include "rs_passes.cuh"

namespace rs {

#define RS_ROW_CASE(N) \
  case N: return launch_rows_n<N>(a, vox, s);

cudaError_t launch_row_pass_pow2(int n, const RowArgs& a, bool vox, cudaStream_t s) {
  switch (n) {
    RS_POW2_SIZES(RS_ROW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

#define RS_ROWADJ_CASE(N) \
  case N: return launch_row_adjoint_n<N>(a, s);

cudaError_t launch_row_adjoint_pow2(int n, const RowArgs& a, cudaStream_t s) {
  switch (n) {
    RS_POW2_SIZES(RS_ROWADJ_CASE)
    default: return cudaErrorInvalidValue;
  }
}

#define RS_ROWPIPE_CASE(N) \
  case N: return launch_row_pipe_n<N>(a, status, s);

#define RS_ROWOK_CASE(N) \
  case N: return true;

cudaError_t launch_row_pipe_pow2(int n, const RowArgs& a, int* status, cudaStream_t s) {
  switch (n) {
    RS_POW2_PIPE_ROW(RS_ROWPIPE_CASE)
    default: return cudaErrorInvalidValue;
  }
}

bool row_pipe_ok_pow2(int n) {
  switch (n) {
    RS_POW2_PIPE_ROW(RS_ROWOK_CASE)
    default: return false;
  }
}

}  // namespace rs
