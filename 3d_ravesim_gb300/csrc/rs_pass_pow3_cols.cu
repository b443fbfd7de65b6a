// rs_pass_pow3_cols.cu — column-pass and twiddle-table instantiations for the 3*2^k sizes.
#include "rs_passes.cuh"

namespace rs {

#define RS_COL_CASE(N) \
  case N: return launch_cols_nw<N, strip_width<N>()>(a, s);

#define RS_TW_CASE(N) \
  case N: return launch_stage_twiddles_n<N>(tw, s);

#define RS_TWLEN_CASE(N) \
  case N: return stage_twiddle_len_n<N>();

cudaError_t launch_col_pass_pow3(int n, const ColArgs& a, cudaStream_t s) {
  switch (n) {
    RS_POW3_SIZES(RS_COL_CASE)
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_stage_twiddles_pow3(int n, float4* tw, cudaStream_t s) {
  switch (n) {
    RS_POW3_SIZES(RS_TW_CASE)
    default: return cudaErrorInvalidValue;
  }
}

int stage_twiddle_len_pow3(int n) {
  switch (n) {
    RS_POW3_SIZES(RS_TWLEN_CASE)
    default: return -1;
  }
}

#define RS_COLPIPE_CASE(N) \
  case N: return launch_col_pipe_n<N>(a, in, out, box, status, s);

#define RS_COLBOX_CASE(N) \
  case N: *w = ColPipeGeom<N>::W; *bh = ColPipeGeom<N>::BH; return true;

cudaError_t launch_col_pipe_pow3(int n, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out,
                                 StripBox box, int* status, cudaStream_t s) {
  switch (n) {
    RS_POW3_PIPE_COL(RS_COLPIPE_CASE)
    default: return cudaErrorInvalidValue;
  }
}

bool col_pipe_box_pow3(int n, int* w, int* bh) {
  switch (n) {
    RS_POW3_PIPE_COL(RS_COLBOX_CASE)
    default: return false;
  }
}

}  // namespace rs
