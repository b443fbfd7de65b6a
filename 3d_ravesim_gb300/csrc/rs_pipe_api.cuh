// rs_pipe_api.cuh — host entry points of the pipelined passes (rs_dispatch.cu).
#pragma once
#include <cuda.h>

#include "rs_kernels.cuh"

namespace rs {
bool row_pipe_ok(int n);
bool col_pipe_box(int n, int* w, int* bh);
cudaError_t launch_row_pipe(int nx, const RowArgs& a, int* status, cudaStream_t s);
// box: the one the maps were encoded with (col_pipe_box); any other is refused
cudaError_t launch_col_pipe(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                            int* status, cudaStream_t s);
}  // namespace rs
