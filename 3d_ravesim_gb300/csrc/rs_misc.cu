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

__global__ void prop_tables_kernel(const PropTabArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.nx) {
    const int mx = signed_index(i, a.nx);
    const double kx2 = kfreq2_abs(mx < 0 ? -mx : mx, a.nx, a.dx);
    if (a.with_h) {
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
    a.ylim[i] = lim;
  }
  if (a.with_h && i < a.ny) {
    const int my = signed_index(i, a.ny);
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
  a.idx[i] = inside ? static_cast<int>(fl) : -1;
  a.frac[i] = static_cast<float>(__dsub_rn(idx, fl));
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

}  // namespace

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
