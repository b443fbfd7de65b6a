// rs_pass_pow2.cu — fused pass and twiddle-table instantiations for the 2^k sizes.
#include "rs_passes.cuh"

namespace rs {

#define RS_ROW_CASE(N) \
  case N: return launch_rows_n<N>(a, s);
#define RS_COL_CASE(N) \
  case N: return launch_cols_nw<N, strip_width<N>()>(a, s);
#define RS_TW_CASE(N) \
  case N: return launch_stage_twiddles_n<N>(tw, s);
#define RS_TWLEN_CASE(N) \
  case N: return stage_twiddle_len_n<N>();

cudaError_t launch_row_pass_pow2(int n, const RowArgs& a, cudaStream_t s) {
  switch (n) {
    RS_POW2_SIZES(RS_ROW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_col_pass_pow2(int n, const ColArgs& a, cudaStream_t s) {
  switch (n) {
    RS_POW2_SIZES(RS_COL_CASE)
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_stage_twiddles_pow2(int n, float2* tw, cudaStream_t s) {
  switch (n) {
    RS_POW2_SIZES(RS_TW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

int stage_twiddle_len_pow2(int n) {
  switch (n) {
    RS_POW2_SIZES(RS_TWLEN_CASE)
    default: return -1;
  }
}

}  // namespace rs
