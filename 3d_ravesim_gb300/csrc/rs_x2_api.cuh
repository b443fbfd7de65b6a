// rs_x2_api.cuh — host entry points of the split-pair multislice passes (rs_pass_x2.cu).
#pragma once
#include <cuda.h>

#include "rs_kernels.cuh"

namespace rs {
bool row_x2_ok(int nx);
int row_x2_slots(int nx);
bool col_x2_box(int ny, int* w, int* bh);
cudaError_t launch_row_x2(int nx, const RowArgs& a, cudaStream_t s);
// the same row pass with one row per thread group (row_pass_kernel<N, ROWS, true, true>), for the
// row_x2_ok sizes; reads twd1_inv / twd1_fwd
cudaError_t launch_row_d1(int nx, const RowArgs& a, cudaStream_t s);
// the adjoint row pass with the dithered tables (row_adjoint_kernel<N, ROWS, true>)
cudaError_t launch_row_adjoint_d1(int nx, const RowArgs& a, cudaStream_t s);
// sizes with dithered rows one per thread group but no split-pair rows (16384, 3*2^k in [384, 6144])
bool row_d1_only(int nx);
// sizes with dithered columns one per thread group but no split-pair columns (3*2^k in [384, 6144])
bool col_d1_only(int ny);
// box: the one the maps were encoded with (col_x2_box); any other is refused
cudaError_t launch_col_x2(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                          int* status, cudaStream_t s);
// the same column pass with one column per thread group (col_pipe_kernel<N, true>; strips and
// boxes of col_d1_box), for the split-pair column sizes and the col_d1_only sizes; reads twd1
// (the two-level table, or for col_d1_only the stage-major table) and kc
cudaError_t launch_col_d1(int ny, const ColArgs& a, const CUtensorMap& in, const CUtensorMap& out, StripBox box,
                          int* status, cudaStream_t s);
// box of the dithered one-column pass (its own strip geometry, which may differ from the
// compensated pipeline's); false if none
bool col_d1_box(int ny, int* w, int* bh);
// kDitherTables dithered copies of a compensated table of `len` entries (rs_fft2x.cuh)
cudaError_t launch_dither_tables(const float4* comp, float4* out, int len, cudaStream_t s);
// (wr, wi) of each of `n` split-pair entries (wr, wr, wi, wi)
cudaError_t launch_single_tables(const float4* in, float2* out, size_t n, cudaStream_t s);
}  // namespace rs
