// rs_misc.cu — FP64 table builders, generic-size DFT, elementwise and detector kernels.
//
// The FP64 table kernels reproduce numpy's operation order with explicitly rounded
// intrinsics (__dmul_rn/__dadd_rn/__ddiv_rn), so that no multiply-add is contracted and the
// cutoff mask and sample indices are bit-identical to big-wave's.
#include "rs_misc.cuh"

namespace rs {

namespace {

constexpr int kTPB = 256;

inline int nblocks(size_t n, int tpb = kTPB) { return static_cast<int>((n + tpb - 1) / tpb); }

inline cudaError_t counted(cudaError_t e) {
  if (e == cudaSuccess) note_launch();
  return e;
}

__global__ void twiddle_kernel(float2* tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  double s, c;
  sincospi(-2.0 * static_cast<double>(m) / static_cast<double>(n), &s, &c);
  tw[m] = make_float2(static_cast<float>(c), static_cast<float>(s));
}

// (numpy.fft.fftfreq(n)[|m|] / spacing)^2, big-wave/propagation.py:293-295.
__device__ __forceinline__ double kfreq2_abs(int am, int n, double spacing) {
  const double val = __ddiv_rn(1.0, static_cast<double>(n));
  const double f = __ddiv_rn(__dmul_rn(static_cast<double>(am), val), spacing);
  return __dmul_rn(f, f);
}

__device__ __forceinline__ int signed_index(int i, int n) {
  return i < (n - 1) / 2 + 1 ? i : i - n;
}

// Frequency index held by storage entry i of an axis of length n (four-step order when n2 > 0).
__device__ __forceinline__ int storage_freq(int i, int n, int n2) {
  return n2 > 0 ? i / n2 + (n / n2) * (i % n2) : i;
}

__global__ void prop_tables_kernel(const PropTabArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.nx && (a.ex || a.ylim)) {
    const int mx = signed_index(storage_freq(i, a.nx, a.n2x), a.nx);
    const double kx2 = kfreq2_abs(mx < 0 ? -mx : mx, a.nx, a.dx);
    if (a.with_h && a.ex) {
      double s, c;
      sincos(__dmul_rn(a.ps, kx2), &s, &c);
      a.ex[i] = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
    // largest |my| with ky2 + kx2 <= freq_sq (mask of propagation.py:322-323 is "> freq_sq")
    const int mmax = a.ny / 2;
    int lim = -1;
    if (__dadd_rn(kfreq2_abs(0, a.ny, a.dy), kx2) <= a.freq_sq) {
      int lo = 0, hi = mmax + 1;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__dadd_rn(kfreq2_abs(mid, a.ny, a.dy), kx2) <= a.freq_sq) lo = mid; else hi = mid;
      }
      lim = lo;
    }
    if (a.ylim) a.ylim[i] = lim;
  }
  if (a.kyi && i < a.ny) a.kyi[i] = signed_index(storage_freq(i, a.ny, a.n2y), a.ny);
  if (a.with_h && a.ey && i < a.ny) {
    const int my = signed_index(storage_freq(i, a.ny, a.n2y), a.ny);
    const double ky2 = kfreq2_abs(my < 0 ? -my : my, a.ny, a.dy);
    double s, c, gs, gc;
    sincos(__dmul_rn(a.ps, ky2), &s, &c);
    sincos(a.gphi, &gs, &gc);
    const double re = gc * c - gs * s;
    const double im = gc * s + gs * c;
    a.ey[i] = make_float2(static_cast<float>(re), static_cast<float>(im));
  }
}

__global__ void axis_table_kernel(const AxisTabArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double sim = __dmul_rn(__dsub_rn(static_cast<double>(i), static_cast<double>(a.n) / 2.0), a.spacing);
  const double half = __dmul_rn(__dmul_rn(static_cast<double>(a.len), a.pitch), 0.5);
  const double idx = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(sim, a.cs), a.pos), half), a.pitch);
  const double fl = floor(idx);
  const bool inside = (idx >= 0.0) && (idx < static_cast<double>(a.len) - 1.0);
  const int id = inside ? static_cast<int>(fl) : -1;
  const float fr = static_cast<float>(__dsub_rn(idx, fl));
  a.idx[i] = id;
  a.frac[i] = fr;
  if (a.packed) a.packed[i] = make_int2(id, __float_as_int(fr));
}

// One block per line; the line is staged in shared memory, so in == out is allowed.
__global__ void dft_axis_kernel(const float2* in, float2* out, int nx, int ny, int axis, int inv,
                                const float2* __restrict__ tw, float scale) {
  extern __shared__ float2 line[];
  const int n = axis == 0 ? nx : ny;
  const int l = blockIdx.x;
  const size_t base = axis == 0 ? static_cast<size_t>(l) * nx : static_cast<size_t>(l);
  const size_t stride = axis == 0 ? 1 : static_cast<size_t>(nx);
  for (int j = threadIdx.x; j < n; j += blockDim.x) line[j] = in[base + j * stride];
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    int m = 0;
    for (int j = 0; j < n; ++j) {
      const float2 w = __ldg(&tw[m]);
      acc = cadd(acc, inv ? cmulc(line[j], w) : cmul(line[j], w));
      m += k;
      if (m >= n) m -= n;
    }
    out[base + k * stride] = cscale(acc, scale);
  }
}

__global__ void transfer_kernel(float2* U, int nx, int ny, const float2* __restrict__ ex,
                                const float2* __restrict__ ey, const int* __restrict__ ylim,
                                int with_h, float2* spec_copy) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<size_t>(nx) * ny) return;
  const int fx = static_cast<int>(i % nx);
  const int fy = static_cast<int>(i / nx);
  const int m = signed_index(fy, ny);
  float2 v = U[i];
  if ((m < 0 ? -m : m) > __ldg(&ylim[fx])) {
    v = make_float2(0.f, 0.f);
  } else if (with_h) {
    v = cmul(v, cmul(__ldg(&ex[fx]), __ldg(&ey[fy])));
  }
  U[i] = v;
  if (spec_copy) spec_copy[i] = v;
}

__global__ void scale_kernel(float2* u, size_t n, float s) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) u[i] = cscale(u[i], s);
}

__global__ void point_source_kernel(float2* u, int nx, int ny, const PointSrcArgs p) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<size_t>(nx) * ny) return;
  u[i] = point_source_value(p, static_cast<int>(i % nx), static_cast<int>(i / nx));
}

__global__ void transmission_kernel(float2* u, int nx, int ny, const AxisTab ax, const VoxelArgs vox,
                                    const PlasmaArgs pl, int plasma) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<size_t>(nx) * ny) return;
  const int x = static_cast<int>(i % nx);
  const int y = static_cast<int>(i / nx);
  const int yi = __ldg(&ax.yi[y]);
  const int xi = __ldg(&ax.xi[x]);
  if (yi < 0 || xi < 0) return;
  const float fx = __ldg(&ax.xf[x]);
  const float fy = __ldg(&ax.yf[y]);
  const float2 d = plasma ? plasma_db(pl, xi, fx, yi, fy) : voxel_db(vox, xi, fx, yi, fy);
  if (d.x == 0.0f && d.y == 0.0f) return;
  u[i] = cmul(u[i], material_factor(d.x, d.y, plasma ? pl.a : vox.a));
}

// One thread per detector pixel: sum over its (row, cell) footprint of weight*|u|^2, times the
// obliquity cosine z/sqrt(x^2 + y^2 + z^2) (big-wave/propagation.py:1044-1060).
__global__ void detector_kernel(const DetArgs a) {
  const int ox = blockIdx.x * blockDim.x + threadIdx.x;
  const int oy = blockIdx.y;
  if (ox >= a.out_x || oy >= a.out_y) return;
  const int x0 = __ldg(&a.xptr[ox]), x1 = __ldg(&a.xptr[ox + 1]);
  const int y0 = __ldg(&a.yptr[oy]), y1 = __ldg(&a.yptr[oy + 1]);
  double acc = 0.0;
  for (int yk = y0; yk < y1; ++yk) {
    const float2* row = a.u + static_cast<size_t>(__ldg(&a.ycell[yk])) * a.nx;
    float inner = 0.0f;
    for (int xk = x0; xk < x1; ++xk) {
      const float2 v = row[__ldg(&a.xcell[xk])];
      inner = fmaf(__ldg(&a.xw[xk]), fmaf(v.x, v.x, v.y * v.y), inner);
    }
    acc += __ldg(&a.yw[yk]) * static_cast<double>(inner);
  }
  const double xd = __ldg(&a.xdet[ox]), yd = __ldg(&a.ydet[oy]);
  const double cosine = a.z / sqrt(xd * xd + yd * yd + a.z * a.z);
  const size_t o = static_cast<size_t>(oy) * a.out_x + ox;
  const double val = acc * cosine;
  a.out[o] = a.accumulate ? a.out[o] + val : val;
}

// One block per field row. The row's voxel rows (yi, yi+1) get their gradient contributions
// summed in shared memory first (shared atomics), then one global atomic per touched entry.
__global__ void adjoint_slice_kernel(const AdjointSliceArgs a) {
  extern __shared__ float acc[];  // 4 * nxv floats: (d, b) of voxel rows yi and yi + 1
  const int y = blockIdx.x;
  const int nxv = a.nxv;
  for (int j = threadIdx.x; j < 4 * nxv; j += blockDim.x) acc[j] = 0.0f;
  __syncthreads();
  const int yi = __ldg(&a.ax.yi[y]);
  const float fy = yi >= 0 ? __ldg(&a.ax.yf[y]) : 0.0f;
  const size_t rb = static_cast<size_t>(y) * a.nx;
  for (int x = threadIdx.x; x < a.nx; x += blockDim.x) {
    const int xi = __ldg(&a.ax.xi[x]);
    const float2 vv = a.v[rb + x];
    if (yi < 0 || xi < 0) continue;  // outside the grid: t = 1, no voxel depends on this pixel
    const float fx = __ldg(&a.ax.xf[x]);
    const float2* r0 = a.dbv + static_cast<size_t>(yi) * nxv;
    const float2* r1 = r0 + nxv;
    const float2 d0 = lerp2(__ldg(&r0[xi]), __ldg(&r0[xi + 1]), fx);
    const float2 d1 = lerp2(__ldg(&r1[xi]), __ldg(&r1[xi + 1]), fx);
    const float2 d = lerp2(d0, d1, fy);
    const float2 t = material_factor(d.x, d.y, a.a);
    const float2 uu = __ldg(&a.u[rb + x]);
    // G = conj(u) v; q = conj(G) t; dL/ddelta = 4 pi a Im(q); dL/dbeta = -4 pi a Re(q)
    const float2 G = make_float2(fmaf(uu.x, vv.x, uu.y * vv.y), fmaf(uu.x, vv.y, -uu.y * vv.x));
    const float2 q = cmulc(t, G);
    const float k = 12.566370614359172f * a.a;
    const float gd = k * q.y, gb = -k * q.x;
    const float w00 = (1.0f - fx) * (1.0f - fy), w01 = fx * (1.0f - fy), w10 = (1.0f - fx) * fy, w11 = fx * fy;
    atomicAdd(&acc[2 * xi], w00 * gd);
    atomicAdd(&acc[2 * xi + 1], w00 * gb);
    atomicAdd(&acc[2 * xi + 2], w01 * gd);
    atomicAdd(&acc[2 * xi + 3], w01 * gb);
    atomicAdd(&acc[2 * nxv + 2 * xi], w10 * gd);
    atomicAdd(&acc[2 * nxv + 2 * xi + 1], w10 * gb);
    atomicAdd(&acc[2 * nxv + 2 * xi + 2], w11 * gd);
    atomicAdd(&acc[2 * nxv + 2 * xi + 3], w11 * gb);
    a.v[rb + x] = cmulc(vv, t);  // conj(t) * v
  }
  __syncthreads();
  if (yi < 0) return;
  float* g0 = reinterpret_cast<float*>(a.grad + static_cast<size_t>(yi) * nxv);
  for (int j = threadIdx.x; j < 4 * nxv; j += blockDim.x) {
    const float val = acc[j];
    if (val != 0.0f) atomicAdd(&g0[j], val);  // rows yi and yi + 1 are contiguous in the grid
  }
}

__global__ void detector_adjoint_kernel(const DetAdjArgs a) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x;
  const int gy = blockIdx.y;
  if (gx >= a.nx || gy >= a.ny) return;
  double sacc = 0.0;
  const int y0 = __ldg(&a.yptr[gy]), y1 = __ldg(&a.yptr[gy + 1]);
  const int x0 = __ldg(&a.xptr[gx]), x1 = __ldg(&a.xptr[gx + 1]);
  for (int yk = y0; yk < y1; ++yk) {
    const int oy = __ldg(&a.ydet[yk]);
    const double yd = __ldg(&a.ypos[oy]);
    double inner = 0.0;
    for (int xk = x0; xk < x1; ++xk) {
      const int ox = __ldg(&a.xdet[xk]);
      const double xd = __ldg(&a.xpos[ox]);
      const double cosine = a.z / sqrt(xd * xd + yd * yd + a.z * a.z);
      inner += static_cast<double>(__ldg(&a.xw[xk])) * cosine * a.r[static_cast<size_t>(oy) * a.out_x + ox];
    }
    sacc += __ldg(&a.yw[yk]) * inner;
  }
  const size_t i = static_cast<size_t>(gy) * a.nx + gx;
  a.g[i] = cscale(a.u[i], static_cast<float>(sacc));
}

}  // namespace

cudaError_t launch_adjoint_slice(const AdjointSliceArgs& a, cudaStream_t s) {
  const size_t smem = static_cast<size_t>(4) * a.nxv * sizeof(float);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(adjoint_slice_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  adjoint_slice_kernel<<<a.ny, 256, smem, s>>>(a);
  return counted(cudaGetLastError());
}

cudaError_t launch_detector_adjoint(const DetAdjArgs& a, cudaStream_t s) {
  dim3 grid((a.nx + 127) / 128, a.ny);
  detector_adjoint_kernel<<<grid, 128, 0, s>>>(a);
  return counted(cudaGetLastError());
}

// delta, beta of every voxel of one plasma slice plane, for the voxel-only row kernel: the same
// plasma_db_voxel values the plasma row pass computes, once per voxel instead of once per row.
__global__ void plasma_plane_kernel(const PlasmaArgs pl, float2* dbv, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dbv[i] = plasma_db_voxel(pl, i);
}

cudaError_t launch_plasma_plane(const PlasmaArgs& pl, float2* dbv, int count, cudaStream_t s) {
  plasma_plane_kernel<<<nblocks(count), kTPB, 0, s>>>(pl, dbv, count);
  return counted(cudaGetLastError());
}

cudaError_t launch_twiddles(float2* tw, int n, cudaStream_t s) {
  twiddle_kernel<<<nblocks(n), kTPB, 0, s>>>(tw, n);
  return counted(cudaGetLastError());
}

cudaError_t launch_prop_tables(const PropTabArgs& a, cudaStream_t s) {
  const int n = a.nx > a.ny ? a.nx : a.ny;
  prop_tables_kernel<<<nblocks(n, 128), 128, 0, s>>>(a);
  return counted(cudaGetLastError());
}

cudaError_t launch_axis_table(const AxisTabArgs& a, cudaStream_t s) {
  axis_table_kernel<<<nblocks(a.n), kTPB, 0, s>>>(a);
  return counted(cudaGetLastError());
}

cudaError_t launch_dft_axis(const float2* in, float2* out, int nx, int ny, int axis, int inv,
                            const float2* tw, float scale, cudaStream_t s) {
  const int n = axis == 0 ? nx : ny;
  const int lines = axis == 0 ? ny : nx;
  const size_t smem = static_cast<size_t>(n) * sizeof(float2);
  if (smem > 48 * 1024) return cudaErrorInvalidValue;
  dft_axis_kernel<<<lines, 128, smem, s>>>(in, out, nx, ny, axis, inv, tw, scale);
  return counted(cudaGetLastError());
}

cudaError_t launch_transfer(float2* U, int nx, int ny, const float2* ex, const float2* ey,
                            const int* ylim, int with_h, float2* spec_copy, cudaStream_t s) {
  const size_t n = static_cast<size_t>(nx) * ny;
  transfer_kernel<<<nblocks(n), kTPB, 0, s>>>(U, nx, ny, ex, ey, ylim, with_h, spec_copy);
  return counted(cudaGetLastError());
}

cudaError_t launch_scale(float2* u, size_t n, float scale, cudaStream_t s) {
  scale_kernel<<<nblocks(n), kTPB, 0, s>>>(u, n, scale);
  return counted(cudaGetLastError());
}

cudaError_t launch_point_source(float2* u, int nx, int ny, const PointSrcArgs& p, cudaStream_t s) {
  const size_t n = static_cast<size_t>(nx) * ny;
  point_source_kernel<<<nblocks(n), kTPB, 0, s>>>(u, nx, ny, p);
  return counted(cudaGetLastError());
}

cudaError_t launch_transmission(float2* u, int nx, int ny, const AxisTab& ax, const VoxelArgs* vox,
                                const PlasmaArgs* pl, cudaStream_t s) {
  const size_t n = static_cast<size_t>(nx) * ny;
  VoxelArgs v{};
  PlasmaArgs p{};
  if (vox) v = *vox;
  if (pl) p = *pl;
  transmission_kernel<<<nblocks(n), kTPB, 0, s>>>(u, nx, ny, ax, v, p, pl ? 1 : 0);
  return counted(cudaGetLastError());
}

cudaError_t launch_detector(const DetArgs& a, cudaStream_t s) {
  dim3 grid((a.out_x + 127) / 128, a.out_y);
  detector_kernel<<<grid, 128, 0, s>>>(a);
  return counted(cudaGetLastError());
}

}  // namespace rs
