// rs_misc.cuh — table builders, generic-size DFT, elementwise and detector kernels.
#pragma once
#include "rs_kernels.cuh"

namespace rs {

// Transfer-function tables for one (dx, dy, wl, dz, cutoff) (big-wave/propagation.py:427-441).
struct PropTabArgs {
  int nx, ny;
  double dx, dy;
  double ps;       // -(pi*wl)*dz  (imaginary part of numpy's phase_scale)
  double gphi;     // ((2*pi)/wl)*dz (global phase)
  double freq_sq;  // 2.0*freq**2
  int with_h;      // 0: only the cutoff limits are built
  float2* ex;
  float2* ey;
  int* ylim;
  // Four-step storage order (0 = natural): entry i of an axis of length n describes frequency
  // i / n2 + (n / n2) * (i % n2), the order the four-step transforms leave the spectrum in.
  int n2x, n2y;
  int* kyi;        // with n2y: signed y-frequency index of each storage row
};

// Sample coordinate table for one axis (big-wave/optical_element.py:538-546, 555-563).
struct AxisTabArgs {
  int n;            // sim points on this axis
  double spacing;   // sim spacing
  double cs;        // coordinate scale
  double pos;       // x_pos / y_pos
  int len;          // voxel count on this axis
  double pitch;     // voxel pitch
  int* idx;
  float* frac;
  int2* packed;     // optional {idx, bits of frac} copy
};

struct DetArgs {
  const float2* u;
  double* out;
  int nx, out_x, out_y;
  const int* xptr; const int* xcell; const float* xw;
  const int* yptr; const int* ycell; const double* yw;
  const double* xdet; const double* ydet;
  double z;
  int accumulate;
};

cudaError_t launch_twiddles(float2* tw, int n, cudaStream_t s);
cudaError_t launch_prop_tables(const PropTabArgs& a, cudaStream_t s);
cudaError_t launch_axis_table(const AxisTabArgs& a, cudaStream_t s);
// Direct O(n^2) DFT along rows (axis 0) or columns (axis 1); inv uses exp(+...). scale multiplies the output.
cudaError_t launch_dft_axis(const float2* in, float2* out, int nx, int ny, int axis, int inv,
                            const float2* tw, float scale, cudaStream_t s);
cudaError_t launch_transfer(float2* U, int nx, int ny, const float2* ex, const float2* ey,
                            const int* ylim, int with_h, float2* spec_copy, cudaStream_t s);
cudaError_t launch_scale(float2* u, size_t n, float scale, cudaStream_t s);
cudaError_t launch_point_source(float2* u, int nx, int ny, const PointSrcArgs& p, cudaStream_t s);
cudaError_t launch_transmission(float2* u, int nx, int ny, const AxisTab& ax, const VoxelArgs* vox,
                                const PlasmaArgs* pl, cudaStream_t s);
// (delta, beta) of the `count` voxels of one plasma slice plane into dbv.
cudaError_t launch_plasma_plane(const PlasmaArgs& pl, float2* dbv, int count, cudaStream_t s);
cudaError_t launch_detector(const DetArgs& a, cudaStream_t s);

// Adjoint of one slice of the multislice forward u' = P (t * u): given v = P^H g' (in `v`),
// accumulates dL/d(delta, beta) of the slice's voxels (float2 per voxel, `grad`) through the
// bilinear weights and replaces v by conj(t) * v = dL/dconj(u).
struct AdjointSliceArgs {
  float2* v;
  const float2* u;          // forward field entering the slice (before its transmission)
  const float2* dbv;        // (delta, beta) per voxel of this slice, (nyv, nxv)
  float2* grad;             // dL/d(delta, beta) per voxel of this slice
  int nx, ny, nxv, nyv;
  AxisTab ax;
  float a;                  // thickness / wavelength
};
cudaError_t launch_adjoint_slice(const AdjointSliceArgs& a, cudaStream_t s);

// Transposed detector: g = s * u with s(cell) = sum over overlapping detector pixels of
// weight * cosine * r(pixel) (inverse overlap tables per axis, built on the host).
struct DetAdjArgs {
  const float2* u;
  float2* g;
  const double* r;          // dL/dI, (out_y, out_x)
  int nx, ny, out_x;
  const int* xptr; const int* xdet; const float* xw;      // per grid column: detector columns
  const int* yptr; const int* ydet; const double* yw;     // per grid row: detector rows
  const double* xpos; const double* ypos;                  // detector pixel centres
  double z;
};
cudaError_t launch_detector_adjoint(const DetAdjArgs& a, cudaStream_t s);

}  // namespace rs
