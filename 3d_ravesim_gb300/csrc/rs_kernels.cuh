// rs_kernels.cuh — argument blocks and the fused row / column pass kernels.
//
// One multislice slice-step costs two HBM round trips of the field:
//   row pass    : [row IFFT] -> transmission T_k -> row FFT          (rows of the field)
//   column pass : column FFT -> H(fx,fy)*mask/N -> column IFFT       (strips of columns)
// which together compute u_{k+1} = IFFT2[H * FFT2[T_k u_k]] (big-wave/propagation.py:396-442
// after the transmission multiply of big-wave/optical_element.py:565-584). Both passes read
// their whole row / column strip into registers before writing, so they run in place.
#pragma once
#include "rs_fft.cuh"

namespace rs {

// ----------------------------------------------------------------------------- arguments
enum RowFlags : int {
  ROW_INV = 1,      // inverse x-transform first (input is x-spectral, natural order)
  ROW_FWD = 2,      // forward x-transform last
  ROW_SRC = 4,      // generate the point-source field instead of loading `in`
  ROW_TVOX = 8,     // voxel-Sample transmission between the transforms
  ROW_TPLASMA = 16, // PlasmaSample transmission between the transforms
  ROW_SCALE = 32,   // multiply the stored values by `scale`
};

enum ColFlags : int {
  COL_FWD = 1,      // forward y-transform first
  COL_INV = 2,      // inverse y-transform last
  COL_H = 4,        // multiply by ex[fx]*ey[fy] inside the circular cutoff, zero outside
  COL_MASK = 8,     // zero outside the circular cutoff only
  COL_SPEC = 16,    // store the masked/multiplied spectrum to `spec`
  COL_SCALE = 32,   // multiply the data path by `scale` before the inverse
};

// Per-axis sample-coordinate tables (built in FP64, big-wave/optical_element.py:538-563):
// idx = clipped floor of the voxel coordinate, or -1 when the column/row is outside
// the grid (the reference zeroes delta+i*beta there, 579).
struct AxisTab {
  const int* xi;
  const float* xf;
  const int* yi;
  const float* yf;
};

struct VoxelArgs {
  const void* slice;   // uint32 or int32 ids of this z slice, (nyv, nxv)
  int grid_signed;
  int nxv, nyv;
  const float2* db;    // (delta, beta) per material id; index 0 = vacuum
  int n_db;
  float a;             // thickness / wavelength
};

struct PlasmaArgs {
  const void* ne; const void* ni; const void* te; const void* zs;  // this z slice, (nyv, nxv)
  int f64;
  int nxv, nyv;
  // delta = pref * (ne + ni*(1-q)*f1bar); beta = pref*ni*(1-q)*f2eff + cff*ne*ni*q^2/sqrt(te)
  double pref, f1bar, f2eff, inv_zbar, zbar_pos, z2bar_pos, cff;
  float a;
};

struct PointSrcArgs {
  double dx, dy, xs, ys, z2, k;  // k = (2*pi)/wl exactly as numpy forms it
  double half_nx, half_ny;
  int fresnel_plane;             // 1: Fresnel-scaled plane exp(-i k (x xs + y ys)/dz)/dz
  double dz;                     // source-to-plane distance of the Fresnel-scaled plane
};

struct RowArgs {
  const float2* in;
  float2* out;
  int ny;
  int flags;
  float scale;
  const float2* tw;      // twiddles of length nx
  AxisTab ax;
  VoxelArgs vox;
  PlasmaArgs pl;
  PointSrcArgs ps;
};

struct ColArgs {
  const float2* in;
  float2* out;
  float2* spec;
  int nx;
  int flags;
  float scale;
  const float2* tw;      // twiddles of length ny
  const float2* ex;      // nx entries: exp(-i pi wl dz kx^2)
  const float2* ey;      // ny entries: exp(2 pi i dz/wl) * exp(-i pi wl dz ky^2)
  const int* ylim;       // nx entries: largest |signed y index| kept by the cutoff, -1 = none
};

// ----------------------------------------------------------------------------- physics
__device__ __forceinline__ float2 material_factor(float delta, float beta, float a) {
  // exp(-2*pi*i*a*conj(delta + i*beta)) = exp(-2*pi*a*beta) * exp(-2*pi*i*a*delta)
  // (big-wave/optical_element.py:39-42)
  float s, c;
  sincospif(2.0f * a * delta, &s, &c);
  const float amp = expf(-6.283185307179586f * a * beta);
  return make_float2(amp * c, -amp * s);
}

__device__ __forceinline__ float2 db_lookup(const VoxelArgs& p, const void* slice, int lin) {
  int id;
  if (p.grid_signed) {
    id = static_cast<const int*>(slice)[lin];
    if (id < 0) id += p.n_db;  // numpy negative indexing of db_list
  } else {
    const uint32_t u = static_cast<const uint32_t*>(slice)[lin];
    id = u > 0x7fffffffu ? p.n_db : static_cast<int>(u);
  }
  id = min(max(id, 0), p.n_db - 1);  // ids are validated on the host; clamp keeps reads in bounds
  return __ldg(&p.db[id]);
}

// Bilinear (delta, beta) at sim pixel with voxel corner (xi, yi) and fractions (fx, fy),
// in the reference's order: rows blended in x first, then in y (optical_element.py:576-580).
// Corners whose weight is exactly zero are not read (their contribution is exactly zero).
__device__ __forceinline__ float2 voxel_db(const VoxelArgs& p, int xi, float fx, int yi, float fy) {
  const int l0 = yi * p.nxv + xi;
  const float2 d00 = db_lookup(p, p.slice, l0);
  float2 y0 = d00;
  if (fx != 0.0f) {
    const float2 d01 = db_lookup(p, p.slice, l0 + 1);
    y0 = make_float2(d00.x * (1.0f - fx) + d01.x * fx, d00.y * (1.0f - fx) + d01.y * fx);
  }
  if (fy == 0.0f) return y0;
  const int l1 = l0 + p.nxv;
  const float2 d10 = db_lookup(p, p.slice, l1);
  float2 y1 = d10;
  if (fx != 0.0f) {
    const float2 d11 = db_lookup(p, p.slice, l1 + 1);
    y1 = make_float2(d10.x * (1.0f - fx) + d11.x * fx, d10.y * (1.0f - fx) + d11.y * fx);
  }
  return make_float2(y0.x * (1.0f - fy) + y1.x * fy, y0.y * (1.0f - fy) + y1.y * fy);
}

__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float f) {
  return make_float2(a.x * (1.0f - f) + b.x * f, a.y * (1.0f - f) + b.y * f);
}

// Voxel column j of grid row yi blended in y with weight fy (zero-weight rows are not read).
__device__ __forceinline__ float2 voxel_col_blend(const VoxelArgs& p, int j, int yi, float fy) {
  const float2 d0 = db_lookup(p, p.slice, yi * p.nxv + j);
  if (fy == 0.0f) return d0;
  return lerp2(d0, db_lookup(p, p.slice, (yi + 1) * p.nxv + j), fy);
}

__device__ __forceinline__ double plasma_load(const void* g, int f64, int lin) {
  return f64 ? __ldg(static_cast<const double*>(g) + lin)
             : static_cast<double>(__ldg(static_cast<const float*>(g) + lin));
}

// delta, beta of one plasma voxel (big-wave/plasma.py:380-434), FP32 arithmetic on
// pre-scaled densities so that n_e*n_i (~1e42 cm^-6) never overflows.
__device__ __forceinline__ float2 plasma_db_voxel(const PlasmaArgs& p, int lin) {
  const float ne = static_cast<float>(plasma_load(p.ne, p.f64, lin) * 1e-20);
  const float ni = static_cast<float>(plasma_load(p.ni, p.f64, lin) * 1e-20);
  const float te = static_cast<float>(plasma_load(p.te, p.f64, lin));
  const float zs = static_cast<float>(plasma_load(p.zs, p.f64, lin));
  float q = p.zbar_pos ? zs * static_cast<float>(p.inv_zbar) : 0.0f;
  q = fminf(fmaxf(q, 0.0f), 1.0f);
  const float fb = 1.0f - q;
  const float pref = static_cast<float>(p.pref * 1e20);
  float delta = ne * pref;
  float beta = 0.0f;
  if (fb > 0.0f && ni > 0.0f) {
    const float bs = ni * pref * fb;
    delta += bs * static_cast<float>(p.f1bar);
    beta += bs * static_cast<float>(p.f2eff);
  }
  if (ne > 0.0f && ni > 0.0f && q > 0.0f && p.z2bar_pos && te > 0.0f) {
    beta += static_cast<float>(p.cff) * ne * ni * q * q * rsqrtf(te);
  }
  return make_float2(delta, beta);
}

__device__ __forceinline__ float2 plasma_db(const PlasmaArgs& p, int xi, float fx, int yi, float fy) {
  const int l0 = yi * p.nxv + xi;
  const float2 d00 = plasma_db_voxel(p, l0);
  const float2 d01 = plasma_db_voxel(p, l0 + 1);
  const float2 d10 = plasma_db_voxel(p, l0 + p.nxv);
  const float2 d11 = plasma_db_voxel(p, l0 + p.nxv + 1);
  const float2 y0 = make_float2(d00.x * (1.0f - fx) + d01.x * fx, d00.y * (1.0f - fx) + d01.y * fx);
  const float2 y1 = make_float2(d10.x * (1.0f - fx) + d11.x * fx, d10.y * (1.0f - fx) + d11.y * fx);
  return make_float2(y0.x * (1.0f - fy) + y1.x * fy, y0.y * (1.0f - fy) + y1.y * fy);
}

__device__ __forceinline__ float2 plasma_col_blend(const PlasmaArgs& p, int j, int yi, float fy) {
  const float2 d0 = plasma_db_voxel(p, yi * p.nxv + j);
  if (fy == 0.0f) return d0;
  return lerp2(d0, plasma_db_voxel(p, (yi + 1) * p.nxv + j), fy);
}

// 1/(2*pi) as a double-double (hi + lo), for reducing the FP64 phase r*(2*pi/wl) to cycles.
constexpr double kInv2PiHi = 0.15915494309189535;
constexpr double kInv2PiLo = -9.839338337591243e-18;

// exp(i*r*k)/r with r = sqrt(y^2 + x^2 + z^2), k = 2*pi/wl, evaluated as in
// big-wave/propagation.py:474-483: the FP64 phase phi = r*k is formed with the same IEEE
// operations as numpy, then reduced to a fraction of a cycle with a double-double 1/(2*pi)
// (error ~|phi|*2^-106) before a single-precision sincospi.
// Fresnel-scaled source plane (big-wave/source.py:81-90): x = (ix - nx/2) dx,
// phase = -k (x xs + y ys) / dz formed in FP64 like numpy, value exp(i phase) / dz.
__device__ __forceinline__ float2 fresnel_plane_value(const PointSrcArgs& p, int ix, int iy) {
  const double x = __dmul_rn(__dsub_rn(static_cast<double>(ix), p.half_nx), p.dx);
  const double y = __dmul_rn(__dsub_rn(static_cast<double>(iy), p.half_ny), p.dy);
  const double phi = -__ddiv_rn(__dmul_rn(p.k, __dadd_rn(__dmul_rn(x, p.xs), __dmul_rn(y, p.ys))), p.dz);
  const double c_hi = __dmul_rn(phi, kInv2PiHi);
  const double c_err = __fma_rn(phi, kInv2PiHi, -c_hi);
  const double n = rint(c_hi);
  const double f = __dadd_rn(__dsub_rn(c_hi, n), __fma_rn(phi, kInv2PiLo, c_err));
  float s, c;
  sincospif(static_cast<float>(2.0 * f), &s, &c);
  const float inv = static_cast<float>(1.0 / p.dz);
  return make_float2(c * inv, s * inv);
}

__device__ __forceinline__ float2 point_source_value(const PointSrcArgs& p, int ix, int iy) {
  if (p.fresnel_plane) return fresnel_plane_value(p, ix, iy);
  const double x = __dsub_rn(__dmul_rn(__dsub_rn(static_cast<double>(ix), p.half_nx), p.dx), p.xs);
  const double y = __dsub_rn(__dmul_rn(__dsub_rn(static_cast<double>(iy), p.half_ny), p.dy), p.ys);
  const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(y, y), __dmul_rn(x, x)), p.z2));
  const double phi = __dmul_rn(r, p.k);
  const double c_hi = __dmul_rn(phi, kInv2PiHi);
  const double c_err = __fma_rn(phi, kInv2PiHi, -c_hi);
  const double n = rint(c_hi);
  const double f = __dadd_rn(__dsub_rn(c_hi, n), __fma_rn(phi, kInv2PiLo, c_err));
  float s, c;
  sincospif(static_cast<float>(2.0 * f), &s, &c);
  const float inv_r = static_cast<float>(1.0 / r);
  return make_float2(c * inv_r, s * inv_r);
}

// ----------------------------------------------------------------------------- row pass
#ifndef RS_ROW_MINB
#define RS_ROW_MINB 3
#endif
// blocks per SM the row pass's registers are sized for (one 256-thread row block: 3 -> <= 85 regs)
template <int N, int ROWS>
constexpr int row_minb() {
  return ROWS * FftPlan<N>::T <= 256 ? (FftPlan<N>::E == 16 ? RS_ROW_MINB : 2) : 1;
}

template <int N, int ROWS>
__global__ void __launch_bounds__(ROWS * FftPlan<N>::T, row_minb<N, ROWS>()) row_pass_kernel(const RowArgs a) {
  using P = FftPlan<N>;
  constexpr int T = P::T;
  constexpr int RF = P::entry_radix(false);   // forward entry == inverse exit mapping
  constexpr int RX = P::exit_radix(false);    // forward exit  == inverse entry mapping
  extern __shared__ float2 smem[];
  const int t = threadIdx.x % T;
  const int lr = threadIdx.x / T;
  const int row = blockIdx.x * ROWS + lr;
  const bool valid = row < a.ny;
  float2* buf = smem + lr * P::S;
  const size_t rbase = static_cast<size_t>(valid ? row : 0) * N;
  const int flags = a.flags;
  constexpr int E = P::E;
  float2 v[E];

  if (flags & ROW_INV) {
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = valid ? a.in[rbase + slot_pos<N, RX>(t, e)] : make_float2(0.f, 0.f);
    fft_seq<N, true>(v, buf, t, a.tw);
  } else if (flags & ROW_SRC) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = point_source_value(a.ps, slot_pos<N, RF>(t, e), row);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = valid ? a.in[rbase + slot_pos<N, RF>(t, e)] : make_float2(0.f, 0.f);
  }

  if (flags & (ROW_TVOX | ROW_TPLASMA)) {
    // The exchange buffer is idle between the two transforms: stage the voxel row blended in y
    // there (one gather per voxel column instead of four per pixel), then interpolate in x.
    const bool vox = flags & ROW_TVOX;
    const int nxv = vox ? a.vox.nxv : a.pl.nxv;
    const bool staged = nxv <= P::S;  // uniform across the block
    int yi = -1;
    float fy = 0.0f;
    if (valid) {
      yi = __ldg(&a.ax.yi[row]);
      if (yi >= 0) fy = __ldg(&a.ax.yf[row]);
    }
    if (staged) {
      if (yi >= 0) {
        for (int j = t; j < nxv; j += T) buf[j] = vox ? voxel_col_blend(a.vox, j, yi, fy) : plasma_col_blend(a.pl, j, yi, fy);
      }
      __syncthreads();
    }
    // Branch-free over the E pixels of this thread so their gathers and transcendentals
    // interleave; vacuum (delta = beta = 0) gives a factor of exactly 1. A warp whose pixels are
    // all vacuum skips the transcendentals.
    constexpr int CH = E % 8 == 0 ? 8 : E;  // pixels per interleaved chunk
#pragma unroll
    for (int c0 = 0; c0 < E; c0 += CH) {
      float2 d[CH];
      bool any = false;
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        d[i] = make_float2(0.f, 0.f);
        const int x = slot_pos<N, RF>(t, c0 + i);
        const int xi = yi >= 0 ? __ldg(&a.ax.xi[x]) : -1;
        if (xi >= 0) {
          const float fx = __ldg(&a.ax.xf[x]);
          if (staged) {
            d[i] = buf[xi];
            if (fx != 0.0f) d[i] = lerp2(d[i], buf[xi + 1], fx);
          } else {
            d[i] = vox ? voxel_db(a.vox, xi, fx, yi, fy) : plasma_db(a.pl, xi, fx, yi, fy);
          }
          any |= (d[i].x != 0.0f) | (d[i].y != 0.0f);
        }
      }
      if (__any_sync(0xffffffffu, any)) {
        const float at = vox ? a.vox.a : a.pl.a;
#pragma unroll
        for (int i = 0; i < CH; ++i) v[c0 + i] = cmul(v[c0 + i], material_factor(d[i].x, d[i].y, at));
      }
    }
    if (staged) __syncthreads();  // the forward transform reuses the buffer
  }

  if (flags & ROW_FWD) {
    fft_seq<N, false>(v, buf, t, a.tw);
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const float2 o = (flags & ROW_SCALE) ? cscale(v[e], a.scale) : v[e];
        a.out[rbase + slot_pos<N, RX>(t, e)] = o;
      }
    }
  } else if (valid) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float2 o = (flags & ROW_SCALE) ? cscale(v[e], a.scale) : v[e];
      a.out[rbase + slot_pos<N, RF>(t, e)] = o;
    }
  }
}

// -------------------------------------------------------------------------- column pass
// W adjacent columns per block; column c of the strip uses its own padded buffer whose
// stride is offset by 16/W elements so the W columns fall in different banks.
template <int N, int W>
struct ColGeom {
  static constexpr int SC = FftPlan<N>::S + 16 / W;
  static constexpr int THREADS = W * FftPlan<N>::T;
  static constexpr size_t SMEM = static_cast<size_t>(W) * SC * sizeof(float2);
};

template <int N, int W>
__global__ void __launch_bounds__(W * FftPlan<N>::T) col_pass_kernel(const ColArgs a) {
  using P = FftPlan<N>;
  constexpr int RF = P::entry_radix(false);
  constexpr int RX = P::exit_radix(false);
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int nx = a.nx;
  // the last strip may be partial; its idle columns still take part in the block barriers
  const bool live = blockIdx.x * W + c < nx;
  const int x = live ? blockIdx.x * W + c : nx - 1;
  float2* buf = smem + c * ColGeom<N, W>::SC;
  const int flags = a.flags;
  constexpr int E = P::E;
  float2 v[E];

  if (flags & COL_FWD) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = a.in[static_cast<size_t>(slot_pos<N, RF>(t, e)) * nx + x];
    fft_seq<N, false>(v, buf, t, a.tw);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = a.in[static_cast<size_t>(slot_pos<N, RX>(t, e)) * nx + x];
  }

  // registers are in the forward-exit (== inverse-entry) mapping: position = fy
  if (flags & (COL_H | COL_MASK)) {
    const int lim = __ldg(&a.ylim[x]);
    const float2 exv = (flags & COL_H) ? __ldg(&a.ex[x]) : make_float2(1.f, 0.f);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int fy = slot_pos<N, RX>(t, e);
      const int m = fy < (N + 1) / 2 ? fy : fy - N;
      const bool keep = (m < 0 ? -m : m) <= lim;
      if (!keep) {
        v[e] = make_float2(0.f, 0.f);
      } else if (flags & COL_H) {
        v[e] = cmul(v[e], cmul(exv, __ldg(&a.ey[fy])));
      }
    }
  }
  if ((flags & COL_SPEC) && live) {
#pragma unroll
    for (int e = 0; e < E; ++e) a.spec[static_cast<size_t>(slot_pos<N, RX>(t, e)) * nx + x] = v[e];
  }
  if (flags & COL_SCALE) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cscale(v[e], a.scale);
  }
  if (flags & COL_INV) {
    fft_seq<N, true>(v, buf, t, a.tw);
    if (live) {
#pragma unroll
      for (int e = 0; e < E; ++e) a.out[static_cast<size_t>(slot_pos<N, RF>(t, e)) * nx + x] = v[e];
    }
  } else if (live) {
#pragma unroll
    for (int e = 0; e < E; ++e) a.out[static_cast<size_t>(slot_pos<N, RX>(t, e)) * nx + x] = v[e];
  }
}

// --------------------------------------------------------------------------- launchers
// Implemented in rs_rows.cu / rs_cols.cu; return cudaErrorInvalidValue for unsupported N.
// Counts kernel launches made by this library (read through rs_launch_count).
void note_launch(unsigned n = 1);

cudaError_t launch_row_pass(int nx, const RowArgs& a, cudaStream_t s);
// Twiddles used by the fused passes of length n (fast sizes only): stage-major tables, or the
// plain table tw[m] = exp(-2*pi*i*m/n) when RS_TW_STAGE_MAJOR is 0.
cudaError_t launch_stage_twiddles(int n, float2* tw, cudaStream_t s);
int stage_twiddle_len(int n);
cudaError_t launch_col_pass(int ny, const ColArgs& a, cudaStream_t s);
bool fast_size(int n);

}  // namespace rs
