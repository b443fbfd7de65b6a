// rs_kernels.cuh — argument blocks and the fused row / column pass kernels.
//
// One multislice slice-step costs two HBM round trips of the field:
//   row pass    : [row IFFT] -> transmission T_k -> row FFT          (rows of the field)
//   column pass : column FFT -> H(fx,fy)*mask/N -> column IFFT       (strips of columns)
// which together compute u_{k+1} = IFFT2[H * FFT2[T_k u_k]] (big-wave/propagation.py:396-442
// after the transmission multiply of big-wave/optical_element.py:565-584). Both passes read
// their whole row / column strip into registers before writing, so they run in place.
#pragma once
#include "rs_fft2x.cuh"

namespace rs {

// ----------------------------------------------------------------------------- arguments
enum RowFlags : int {
  ROW_INV = 1,      // inverse x-transform first (input is x-spectral, natural order)
  ROW_FWD = 2,      // forward x-transform last
  ROW_SRC = 4,      // generate the point-source field instead of loading `in`
  ROW_TVOX = 8,     // voxel-Sample transmission between the transforms
  ROW_TPLASMA = 16, // PlasmaSample transmission between the transforms
  ROW_SCALE = 32,   // multiply the stored values by `scale`
  ROW_STORE_U = 64, // store the spatial row entering the transmission to `aux`
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
  const int2* xp;      // x entries packed as {xi, bits of xf}: one 8-byte load per pixel
};

struct VoxelArgs {
  const void* slice;   // uint32 or int32 ids of this z slice, (nyv, nxv)
  int grid_signed;
  int nxv, nyv;
  const float2* db;    // (delta, beta) per material id; index 0 = vacuum
  int n_db;
  float a;             // thickness / wavelength
  const float2* dbv;   // when set: (delta, beta) per voxel of this slice instead of ids + table
};

struct PlasmaArgs {
  const void* ne; const void* ni; const void* te; const void* zs;  // this z slice, (nyv, nxv)
  int f64;
  int nxv, nyv;
  // With densities scaled by 1e-20: delta = pref20 * (ne + ni*(1-q)*f1bar);
  // beta = pref20*ni*(1-q)*f2eff + cff*ne*ni*q^2/sqrt(te). All constants are rounded to float on
  // the host, so the kernels carry no double-precision arithmetic for them.
  float pref20, f1bar, f2eff, inv_zbar, cff;
  int zbar_pos, z2bar_pos;
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
  const float4* tw;      // stage-major compensated twiddles of length nx
  AxisTab ax;
  VoxelArgs vox;
  PlasmaArgs pl;
  PointSrcArgs ps;
  float2* aux;           // ROW_STORE_U: the fields entering the slice; adjoint: read from here
  float* grad;           // adjoint: dL/d(delta, beta) of the slice, float pairs per voxel
  int axis_rows;         // stacked fields: rows per field (the y tables repeat); 0 = ny
  // split-pair passes (row_x2_kernel): this slice's dithered tables and DFT constants for the
  // inverse and the forward transform
  const float4* twd_inv;
  const float4* twd_fwd;
  DftConsts k_inv, k_fwd;
  // the same dithered tables as (wr, wi) entries, for the single-sequence dithered row kernel
  const float2* twd1_inv;
  const float2* twd1_fwd;
};

// Box of the tensor maps a pipelined column pass reads and writes: columns per box (the strip
// width) and rows per copy. A launcher runs only when it equals its kernel's strip geometry, so
// a copy can never deliver more bytes than the strip buffer it lands in.
struct StripBox {
  int w = 0, bh = 0;
};

struct ColArgs {
  const float2* in;
  float2* out;
  float2* spec;
  int nx;
  int flags;
  float scale;
  const float4* tw;      // stage-major compensated twiddles of length ny
  const float2* ex;      // nx entries: exp(-i pi wl dz kx^2)
  const float2* ey;      // ny entries: exp(2 pi i dz/wl) * exp(-i pi wl dz ky^2)
  const int* ylim;       // nx entries: largest |signed y index| kept by the cutoff, -1 = none
  const float4* tw2;     // two-level twiddle table of length ny (Fft2L), when ny has one
  // Batched and strided transforms (the per-block kernel only; all zero for a plain field):
  long long pitch;       // elements between consecutive rows of a transform; 0 = nx
  long long bstride;     // elements between the transforms of consecutive blockIdx.y
  int batches;           // blockIdx.y range (0 = 1)
  int ey_bstride;        // ey / kyi entries between consecutive blockIdx.y
  const int* kyi;        // signed y-frequency index per storage row (null: natural order)
  // Four-step twiddle W_L^{p*q} (W_L = exp(-2 pi i/L)), p = the transform position of the value,
  // q = the column (tw4q = 0) or blockIdx.y (tw4q = 1): multiplied after a forward transform,
  // conjugated before an inverse one. L = tw4, a power of two <= 32768; 0 = none. tw4t holds
  // W_L^m for m < L, compensated (hi, lo) like the stage tables; null: computed with sincospif.
  int tw4;
  int tw4q;
  const float4* tw4t;
  // Test hook of the pipelined pass: wait (with a short bound) on a barrier that nothing completes,
  // record the timeout in the status word and return before any copy is issued.
  int test_stall;
  // split-pair column pass (col_x2_pipe_kernel): this slice's dithered two-level table and constants
  const float4* twd;
  DftConsts kc;
  // the same table as (wr, wi) entries, for the dithered column pass one column per thread group
  const float2* twd1;
};

// ----------------------------------------------------------------------------- physics
// sin(pi h) and cos(pi h). For |h| < 1/16 (|pi h| < 0.2, the usual thin-slice half angle) by
// their Taylor series through x^9 and x^8 (first omitted terms below 5e-16 and 3e-14 of the
// result) with x = pi h formed from a two-float pi; otherwise sincospif.
constexpr float kPiHi = 3.14159274101257324219f;
constexpr float kPiLo = -8.74227766e-08f;
// The library sine/cosine and expm1 of the rarely taken branches below, kept out of line so that
// the fully unrolled transmission loops of the row passes carry one call instead of one inlined
// copy per pixel (the same functions, so the same bits).
static __device__ __noinline__ void sincospif_ool(float h, float* s, float* c) { sincospif(h, s, c); }
static __device__ __noinline__ float expm1f_ool(float x) { return expm1f(x); }

__device__ __forceinline__ void sincospi_small(float h, float* s, float* c) {
  if (fabsf(h) < 0.0625f) {
    const float x = fmaf(h, kPiHi, h * kPiLo);
    const float x2 = x * x;
    *s = x * fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 2.7557319e-06f, -1.9841270e-04f), 8.3333333e-03f),
                           -1.6666667e-01f), 1.0f);
    *c = fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 2.4801587e-05f, -1.3888889e-03f), 4.1666667e-02f), -0.5f), 1.0f);
  } else {
    sincospif_ool(h, s, c);
  }
}

__device__ __forceinline__ float2 material_factor(float delta, float beta, float a) {
  // exp(-2*pi*i*a*conj(delta + i*beta)) = exp(-2*pi*a*beta) * exp(-2*pi*i*a*delta)
  // (big-wave/optical_element.py:39-42)
  // Both factors are close to 1 for the usual thin slices, and their rounding repeats in every
  // slice of similar material, so each is formed so that its only large rounding is the final,
  // unbiased one to nearest: cos(phi) = 1 - 2 sin^2(phi/2), sin(phi) = 2 sin(phi/2) cos(phi/2)
  // from the half angle phi/2 = pi*a*delta, and exp(x) = 1 + expm1(x).
  float sh, ch;
  sincospi_small(a * delta, &sh, &ch);
  const float c = fmaf(-2.0f * sh, sh, 1.0f);
  const float s = 2.0f * sh * ch;
  const float x = -6.283185307179586f * a * beta;
  // expm1 by its Taylor series through x^4 when |x| < 1/64 (remainder below x^5/120 < 1e-11 |x|),
  // the library expm1f otherwise
  const float em1 = fabsf(x) < 0.015625f
                        ? x * fmaf(x, fmaf(x, fmaf(x, 0.041666666666666667f, 0.16666666666666667f), 0.5f), 1.0f)
                        : expm1f_ool(x);
  const float amp = 1.0f + em1;
  return make_float2(amp * c, -amp * s);
}

// exp(-2 pi i a conj(delta + i beta)) of two pixels at once, formed as material_factor does
// (half-angle cosine and sine, amplitude 1 + expm1) with each pixel's result the bits
// material_factor gives it: returns (Re, Re) and (Im, Im) pairs.
__device__ __forceinline__ cp2 material_factor2(float2 dA, float2 dB, float a) {
  const float2 h = make_float2(a * dA.x, a * dB.x);
  float2 sh, ch;
  if (fabsf(h.x) < 0.0625f && fabsf(h.y) < 0.0625f) {
    // the Taylor series of sincospi_small on both pixels at once
    const float2 x = p_fma(h, make_float2(kPiHi, kPiHi), p_mul(h, make_float2(kPiLo, kPiLo)));
    const float2 x2 = p_mul(x, x);
    const float2 ps = p_fma(x2, p_fma(x2, p_fma(x2, p_fma(x2, make_float2(2.7557319e-06f, 2.7557319e-06f),
                                                          make_float2(-1.9841270e-04f, -1.9841270e-04f)),
                                                make_float2(8.3333333e-03f, 8.3333333e-03f)),
                                      make_float2(-1.6666667e-01f, -1.6666667e-01f)),
                            make_float2(1.f, 1.f));
    sh = p_mul(x, ps);
    ch = p_fma(x2, p_fma(x2, p_fma(x2, p_fma(x2, make_float2(2.4801587e-05f, 2.4801587e-05f),
                                             make_float2(-1.3888889e-03f, -1.3888889e-03f)),
                                   make_float2(4.1666667e-02f, 4.1666667e-02f)),
                         make_float2(-0.5f, -0.5f)),
               make_float2(1.f, 1.f));
  } else {
    sincospi_small(h.x, &sh.x, &ch.x);
    sincospi_small(h.y, &sh.y, &ch.y);
  }
  const float2 c = p_fma(p_mul(make_float2(-2.f, -2.f), sh), sh, make_float2(1.f, 1.f));
  const float2 ns = p_mul(p_mul(make_float2(-2.f, -2.f), sh), ch);  // -sin(phi)
  const float k = -6.283185307179586f * a;
  const float2 x = make_float2(k * dA.y, k * dB.y);
  // expm1: the Taylor series through x^4 where |x| < 1/64 (remainder below x^5/120 < 1e-11 |x|),
  // expm1f elsewhere, chosen per pixel so that a pixel's factor does not depend on its partner's
  const float2 q = p_fma(x, make_float2(0.041666666666666667f, 0.041666666666666667f),
                         make_float2(0.16666666666666667f, 0.16666666666666667f));
  float2 em1 = p_mul(x, p_fma(x, p_fma(x, q, make_float2(0.5f, 0.5f)), make_float2(1.f, 1.f)));
  if (!(fabsf(x.x) < 0.015625f)) em1.x = expm1f_ool(x.x);
  if (!(fabsf(x.y) < 0.015625f)) em1.y = expm1f_ool(x.y);
  const float2 amp = p_add(make_float2(1.f, 1.f), em1);
  return {p_mul(amp, c), p_mul(amp, ns)};
}

// (delta, beta) of one raw voxel id (the 32-bit word as stored in the grid).
__device__ __forceinline__ float2 db_of_id(const VoxelArgs& p, uint32_t raw) {
  int id;
  if (p.grid_signed) {
    id = static_cast<int>(raw);
    if (id < 0) id += p.n_db;  // numpy negative indexing of db_list
  } else {
    id = raw > 0x7fffffffu ? p.n_db : static_cast<int>(raw);
  }
  id = min(max(id, 0), p.n_db - 1);  // ids are validated on the host; clamp keeps reads in bounds
  return __ldg(&p.db[id]);
}

__device__ __forceinline__ float2 db_lookup(const VoxelArgs& p, const void* slice, int lin) {
  if (p.dbv) return __ldg(&p.dbv[lin]);
  return db_of_id(p, static_cast<const uint32_t*>(slice)[lin]);
}

// a*(1-f) + b*f with the rounding spelled out (one product, one fused multiply-add), so that
// every kernel that blends the same values gets the same bits whatever the compiler contracts.
__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float f) {
  const float g = __fsub_rn(1.0f, f);
  return make_float2(__fmaf_rn(b.x, f, __fmul_rn(a.x, g)), __fmaf_rn(b.y, f, __fmul_rn(a.y, g)));
}

// Bilinear (delta, beta) at sim pixel with voxel corner (xi, yi) and fractions (fx, fy),
// in the reference's order: rows blended in x first, then in y (optical_element.py:576-580).
// Corners whose weight is exactly zero are not read (their contribution is exactly zero).
__device__ __forceinline__ float2 voxel_db(const VoxelArgs& p, int xi, float fx, int yi, float fy) {
  const int l0 = yi * p.nxv + xi;
  const float2 d00 = db_lookup(p, p.slice, l0);
  float2 y0 = d00;
  if (fx != 0.0f) y0 = lerp2(d00, db_lookup(p, p.slice, l0 + 1), fx);
  if (fy == 0.0f) return y0;
  const int l1 = l0 + p.nxv;
  const float2 d10 = db_lookup(p, p.slice, l1);
  float2 y1 = d10;
  if (fx != 0.0f) y1 = lerp2(d10, db_lookup(p, p.slice, l1 + 1), fx);
  return lerp2(y0, y1, fy);
}

// Voxel column j of grid row yi blended in y with weight fy (zero-weight rows are not read).
__device__ __forceinline__ float2 voxel_col_blend(const VoxelArgs& p, int j, int yi, float fy) {
  const float2 d0 = db_lookup(p, p.slice, yi * p.nxv + j);
  if (fy == 0.0f) return d0;
  return lerp2(d0, db_lookup(p, p.slice, (yi + 1) * p.nxv + j), fy);
}

// A grid value as float (float64 grids are rounded once; 1e21-scale densities fit in float).
__device__ __forceinline__ float plasma_load(const void* g, int f64, int lin) {
  return f64 ? __double2float_rn(__ldg(static_cast<const double*>(g) + lin))
             : __ldg(static_cast<const float*>(g) + lin);
}

// delta, beta of one plasma voxel (big-wave/plasma.py:380-434), FP32 arithmetic on
// pre-scaled densities (ne, ni times 1e-20) so that n_e*n_i (~1e42 cm^-6) never overflows.
__device__ __forceinline__ float2 plasma_db_vals(const PlasmaArgs& p, float ne, float ni, float te, float zs) {
  float q = p.zbar_pos ? zs * p.inv_zbar : 0.0f;
  q = fminf(fmaxf(q, 0.0f), 1.0f);
  const float fb = 1.0f - q;
  float delta = ne * p.pref20;
  float beta = 0.0f;
  if (fb > 0.0f && ni > 0.0f) {
    const float bs = ni * p.pref20 * fb;
    delta += bs * p.f1bar;
    beta += bs * p.f2eff;
  }
  if (ne > 0.0f && ni > 0.0f && q > 0.0f && p.z2bar_pos && te > 0.0f) {
    beta += p.cff * ne * ni * q * q * rsqrtf(te);
  }
  return make_float2(delta, beta);
}

__device__ __forceinline__ float2 plasma_db_voxel(const PlasmaArgs& p, int lin) {
  return plasma_db_vals(p, plasma_load(p.ne, p.f64, lin) * 1e-20f, plasma_load(p.ni, p.f64, lin) * 1e-20f,
                        plasma_load(p.te, p.f64, lin), plasma_load(p.zs, p.f64, lin));
}

// ------------------------------------------------------------- voxel-row prefetch
// The row pass copies the two voxel rows (yi, yi + 1) its transmission needs into shared memory
// with asynchronous 4-byte copies issued before the inverse row transform, so the gathers'
// latency hides behind that transform. The rows are contiguous in every grid, so each source
// is one range of 2 * nxv elements.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// 4-byte words of one source's two rows: ids (4 B), per-voxel (delta, beta) (8 B), plasma
// fields (4 or 8 B each, four sources).
__device__ __forceinline__ int prefetch_words(bool vox, const VoxelArgs& v, const PlasmaArgs& pl) {
  const int nxv = vox ? v.nxv : pl.nxv;
  if (vox) return 2 * nxv * (v.dbv ? 2 : 1);
  return 4 * 2 * nxv * (pl.f64 ? 2 : 1);
}

// Issue the copies of rows yi, yi + 1 into pf (uint32 words); src order: ids or dbv, or the
// plasma fields ne, ni, te, zs one after the other.
__device__ __forceinline__ void prefetch_rows(uint32_t* pf, bool vox, const VoxelArgs& v, const PlasmaArgs& pl,
                                              int yi, int t, int nthreads) {
  if (vox) {
    const int w = v.dbv ? 2 : 1;
    const int words = 2 * v.nxv * w;
    const uint32_t* src = v.dbv ? reinterpret_cast<const uint32_t*>(v.dbv) + static_cast<size_t>(yi) * v.nxv * 2
                                : static_cast<const uint32_t*>(v.slice) + static_cast<size_t>(yi) * v.nxv;
    for (int i = t; i < words; i += nthreads) cp_async4(pf + i, src + i);
  } else {
    const int w = pl.f64 ? 2 : 1;
    const int words = 2 * pl.nxv * w;
    const void* f[4] = {pl.ne, pl.ni, pl.te, pl.zs};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t* src = static_cast<const uint32_t*>(f[k]) + static_cast<size_t>(yi) * pl.nxv * w;
      for (int i = t; i < words; i += nthreads) cp_async4(pf + k * words + i, src + i);
    }
  }
}

__device__ __forceinline__ float pf_plasma(const uint32_t* pf, int f64, int idx) {
  return f64 ? __double2float_rn(reinterpret_cast<const double*>(pf)[idx]) : __uint_as_float(pf[idx]);
}

// Voxel column j of the prefetched rows blended in y with weight fy.
__device__ __forceinline__ float2 pf_col_blend(const uint32_t* pf, bool vox, const VoxelArgs& v,
                                               const PlasmaArgs& pl, int j, float fy) {
  if (vox) {
    const int nxv = v.nxv;
    float2 d0, d1;
    if (v.dbv) {
      const float2* r = reinterpret_cast<const float2*>(pf);
      d0 = r[j];
      if (fy == 0.0f) return d0;
      d1 = r[nxv + j];
    } else {
      d0 = db_of_id(v, pf[j]);
      if (fy == 0.0f) return d0;
      d1 = db_of_id(v, pf[nxv + j]);
    }
    return lerp2(d0, d1, fy);
  }
  const int nxv = pl.nxv;
  const int words = 2 * nxv * (pl.f64 ? 2 : 1);
  const uint32_t* ne = pf;
  const uint32_t* ni = pf + words;
  const uint32_t* te = pf + 2 * words;
  const uint32_t* zs = pf + 3 * words;
  auto at = [&](int k) {
    return plasma_db_vals(pl, pf_plasma(ne, pl.f64, k) * 1e-20f, pf_plasma(ni, pl.f64, k) * 1e-20f,
                          pf_plasma(te, pl.f64, k), pf_plasma(zs, pl.f64, k));
  };
  const float2 d0 = at(j);
  if (fy == 0.0f) return d0;
  return lerp2(d0, at(nxv + j), fy);
}

__device__ __forceinline__ float2 plasma_db(const PlasmaArgs& p, int xi, float fx, int yi, float fy) {
  const int l0 = yi * p.nxv + xi;
  const float2 d00 = plasma_db_voxel(p, l0);
  const float2 d01 = plasma_db_voxel(p, l0 + 1);
  const float2 d10 = plasma_db_voxel(p, l0 + p.nxv);
  const float2 d11 = plasma_db_voxel(p, l0 + p.nxv + 1);
  return lerp2(lerp2(d00, d01, fx), lerp2(d10, d11, fx), fy);
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
#define RS_ROW_MINB 4
#endif
// blocks per SM the row pass's registers are sized for (one 256-thread row block: 4 -> <= 64
// registers; the few spilled values cost less than the warps a fourth block adds)
template <int N, int ROWS>
#ifndef RS_ROW_MINB_POW3
#define RS_ROW_MINB_POW3 3
#endif
constexpr int row_minb() {
  // sized for 256-thread blocks; smaller blocks of short rows get proportionally more of them
  return ROWS * FftPlan<N>::T <= 256
             ? (FftPlan<N>::E == 16 ? RS_ROW_MINB : RS_ROW_MINB_POW3) * (256 / (ROWS * FftPlan<N>::T))
             : 1;
}

// Shared memory of a row block: the exchange buffers (S per row), then a voxel-row prefetch
// area of PF_WORDS 4-byte words per row (at most 4 KB: two rows of up to 512 ids; larger rows
// are gathered without it). It is kept small so that L1 keeps room for the twiddle and
// coordinate tables (at 4096, 4 KB instead of 8 KB per block: 141.8 -> 138.5 us per pass), and
// PF_WORDS <= 2*S, so whatever fits it also fits the staging buffer.
template <int N, int ROWS>
struct RowGeom {
  static constexpr size_t BUF = static_cast<size_t>(ROWS) * FftPlan<N>::S * sizeof(float2);
#ifndef RS_ROW_PF_WORDS
#define RS_ROW_PF_WORDS 1024
#endif
  static constexpr int PF_WORDS = 2 * FftPlan<N>::S < RS_ROW_PF_WORDS ? 2 * FftPlan<N>::S : RS_ROW_PF_WORDS;
  static constexpr bool PF = BUF + static_cast<size_t>(ROWS) * PF_WORDS * 4 <= 200 * 1024;
  static constexpr size_t SMEM = PF ? BUF + static_cast<size_t>(ROWS) * PF_WORDS * 4 : BUF;
};

// VOX = true: the multislice hot path and plain row transforms only (optional row IFFT, optional
// voxel transmission, row FFT, the optional field store and scale), so the point-source and
// plasma code is not in the kernel.
// DITH = true (with VOX): the transforms use the slice's dithered tables
// (twd1_inv / twd1_fwd, k_inv / k_fwd) in the single-sequence form of the split-pair arithmetic,
// and the transmission is applied as the split-pair row kernel applies it, so the result is that
// of row_x2_kernel with one row per thread group.
template <int N, int ROWS, bool VOX = false, bool DITH = false>
__global__ void __launch_bounds__(ROWS * FftPlan<N>::T, row_minb<N, ROWS>()) row_pass_kernel(const RowArgs a) {
  static_assert(!DITH || VOX, "dithered rows: the voxel hot path");
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

  // Transmission row coordinates, and the prefetch of its two voxel rows (block-uniform decision).
  const bool tmode = (flags & (ROW_TVOX | ROW_TPLASMA)) != 0;  // VOX: also plain transforms
  const bool vox = VOX || (flags & ROW_TVOX);
  int yi = -1;
  float fy = 0.0f;
  bool pf_on = false;
  uint32_t* pf = reinterpret_cast<uint32_t*>(smem + ROWS * P::S) + lr * RowGeom<N, ROWS>::PF_WORDS;
  if (tmode) {
    if (valid) {
      const int ar = a.axis_rows ? row % a.axis_rows : row;  // row of its own field
      yi = __ldg(&a.ax.yi[ar]);
      if (yi >= 0) fy = __ldg(&a.ax.yf[ar]);
    }
    if constexpr (RowGeom<N, ROWS>::PF) {
      pf_on = prefetch_words(vox, a.vox, a.pl) <= RowGeom<N, ROWS>::PF_WORDS;
      if (pf_on && yi >= 0) prefetch_rows(pf, vox, a.vox, a.pl, yi, t, T);
    }
  }

  if (flags & ROW_INV) {
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = valid ? a.in[rbase + slot_pos<N, RX>(t, e)] : make_float2(0.f, 0.f);
    if constexpr (DITH) {
      fft_seq2x<N, true>(v, buf, t, a.twd1_inv, dft_k1(a.k_inv));
    } else {
      fft_seq<N, true>(v, buf, t, a.tw);
    }
  } else if (!VOX && (flags & ROW_SRC)) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = point_source_value(a.ps, slot_pos<N, RF>(t, e), row);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = valid ? a.in[rbase + slot_pos<N, RF>(t, e)] : make_float2(0.f, 0.f);
  }

  if ((flags & ROW_STORE_U) && valid) {
#pragma unroll
    for (int e = 0; e < E; ++e) a.aux[rbase + slot_pos<N, RF>(t, e)] = v[e];
  }

  if (tmode) {
    // The exchange buffer is idle between the two transforms: stage the voxel row blended in y
    // there (one gather per voxel column instead of four per pixel), then interpolate in x.
    const int nxv = vox ? a.vox.nxv : a.pl.nxv;
    const bool staged = nxv <= P::S;  // uniform across the block
    if (pf_on) {
      cp_async_wait_all();
      __syncthreads();
      if (yi >= 0) {
        for (int j = t; j < nxv; j += T) buf[j] = pf_col_blend(pf, vox, a.vox, a.pl, j, fy);
      }
      __syncthreads();
    } else if (staged) {
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
        const int2 xe = yi >= 0 ? __ldg(&a.ax.xp[x]) : make_int2(-1, 0);
        const int xi = xe.x;
        if (xi >= 0) {
          const float fx = __int_as_float(xe.y);
          if (staged) {
            d[i] = lerp2(buf[xi], buf[xi + 1], fx);  // exact for fx = 0; xi + 1 < nxv
          } else {
            d[i] = vox ? voxel_db(a.vox, xi, fx, yi, fy) : plasma_db(a.pl, xi, fx, yi, fy);
          }
          any |= ((__float_as_uint(d[i].x) | __float_as_uint(d[i].y)) << 1) != 0u;  // +-0 is vacuum
        }
      }
      if (__any_sync(0xffffffffu, any)) {
        const float at = vox ? a.vox.a : a.pl.a;
        // the factors two pixels at a time in packed arithmetic (each pixel's bits are those
        // material_factor gives it); RS_ROW_PAIRED_FACTORS=0: one pixel at a time
#ifndef RS_ROW_PAIRED_FACTORS
#define RS_ROW_PAIRED_FACTORS 1
#endif
#if !RS_ROW_PAIRED_FACTORS
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const float2 tr = material_factor(d[i].x, d[i].y, at);
          if constexpr (DITH) {
            v[c0 + i] = x_mul_one(v[c0 + i], tr);
          } else {
            v[c0 + i] = cmul(v[c0 + i], tr);
          }
        }
#else
#pragma unroll
        for (int i = 0; i < CH; i += 2) {
          const cp2 tr = material_factor2(d[i], d[i + 1], at);
          const float2 t0 = make_float2(tr.re.x, tr.im.x), t1 = make_float2(tr.re.y, tr.im.y);
          if constexpr (DITH) {
            v[c0 + i] = x_mul_one(v[c0 + i], t0);
            v[c0 + i + 1] = x_mul_one(v[c0 + i + 1], t1);
          } else {
            v[c0 + i] = cmul(v[c0 + i], t0);
            v[c0 + i + 1] = cmul(v[c0 + i + 1], t1);
          }
        }
#endif
      }
    }
    if (staged) __syncthreads();  // the forward transform reuses the buffer
  }

  if (flags & ROW_FWD) {
    if constexpr (DITH) {
      fft_seq2x<N, false>(v, buf, t, a.twd1_fwd, dft_k1(a.k_fwd));
    } else {
      fft_seq<N, false>(v, buf, t, a.tw);
    }
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

// ------------------------------------------------------------------ adjoint row pass
// The adjoint of one slice fused between the row transforms of the backward sweep:
// [row IFFT] -> v = P^H g' in the spatial domain; with u the field that entered the slice (aux)
// and t its transmission, accumulate dL/ddelta = 4 pi a Im(t conj(G)), dL/dbeta =
// -4 pi a Re(t conj(G)), G = conj(u) v, through the bilinear weights into `grad`, and continue
// with conj(t) v -> [row FFT]. The y-blended (delta, beta) row and the x-weighted gradient sums
// live in the exchange buffer (the host checks nxv <= S/2). Consecutive lanes hold consecutive
// pixels, several of which fall in one voxel column, so the sums are kept in up to four copies
// (lane mod copies) to spread the shared-memory atomics over distinct addresses; the copies are
// added up per voxel, and each block adds its sums to the grid with one global atomic per touched
// value. The y weights (1 - fy, fy) are the same for every pixel of the row, so they are applied
// once per voxel.
// DITH: the row transforms use dithered tables (twd1_inv / twd1_fwd, k_inv / k_fwd) in the
// single-sequence form, as the default multislice row pass does.
template <int N, int ROWS, bool DITH = false>
__global__ void __launch_bounds__(ROWS * FftPlan<N>::T, row_minb<N, ROWS>()) row_adjoint_kernel(const RowArgs a) {
  using P = FftPlan<N>;
  constexpr int T = P::T;
  constexpr int E = P::E;
  constexpr int RF = P::entry_radix(false);
  constexpr int RX = P::exit_radix(false);
  extern __shared__ float2 smem[];
  const int t = threadIdx.x % T;
  const int lr = threadIdx.x / T;
  const int row = blockIdx.x * ROWS + lr;
  const bool valid = row < a.ny;
  float2* buf = smem + lr * P::S;
  const size_t rbase = static_cast<size_t>(valid ? row : 0) * N;
  const int flags = a.flags;
  const int nxv = a.vox.nxv;
  float2 v[E];
  int yi = -1;
  float fy = 0.0f;
  if (valid) {
    const int ar = a.axis_rows ? row % a.axis_rows : row;  // row of its own field
    yi = __ldg(&a.ax.yi[ar]);
    if (yi >= 0) fy = __ldg(&a.ax.yf[ar]);
  }
  if (flags & ROW_INV) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = valid ? a.in[rbase + slot_pos<N, RX>(t, e)] : make_float2(0.f, 0.f);
    if constexpr (DITH) {
      fft_seq2x<N, true>(v, buf, t, a.twd1_inv, dft_k1(a.k_inv));
    } else {
      fft_seq<N, true>(v, buf, t, a.tw);
    }
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = valid ? a.in[rbase + slot_pos<N, RF>(t, e)] : make_float2(0.f, 0.f);
  }
  // copies of the sums: [copy][nxv + 1][delta, beta] after the nxv staged (delta, beta) values
  const int stride = 2 * (nxv + 1);
  const int copies = max(1, min(4, (P::S - nxv) / (nxv + 1)));  // one copy always fits (nxv <= S/2)
  float* acc = reinterpret_cast<float*>(buf + nxv);
  if (yi >= 0) {
    for (int j = t; j < nxv; j += T) buf[j] = voxel_col_blend(a.vox, j, yi, fy);
    for (int j = t; j < copies * stride; j += T) acc[j] = 0.0f;
  }
  __syncthreads();
  if (yi >= 0) {
    const float k = 12.566370614359172f * a.vox.a;  // 4 pi t / wl
    float* mine = acc + (threadIdx.x % copies) * stride;
    // two pixels at a time: their factors in packed arithmetic (each pixel's bits are those
    // material_factor gives it), then each pixel's gradient and conj(t) v
#pragma unroll
    for (int e0 = 0; e0 < E; e0 += 2) {
      int xs[2], xis[2];
      float fxs[2];
      float2 ds[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        xs[h] = slot_pos<N, RF>(t, e0 + h);
        const int2 xe = __ldg(&a.ax.xp[xs[h]]);
        xis[h] = xe.x;
        fxs[h] = __int_as_float(xe.y);
        ds[h] = xis[h] >= 0 ? lerp2(buf[xis[h]], buf[xis[h] + 1], fxs[h]) : make_float2(0.f, 0.f);
      }
      const cp2 trs = material_factor2(ds[0], ds[1], a.vox.a);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int xi = xis[h];
        if (xi < 0) continue;  // outside the grid: t = 1 and no voxel depends on this pixel
        const int e = e0 + h;
        const float fx = fxs[h];
        const float2 tr = h == 0 ? make_float2(trs.re.x, trs.im.x) : make_float2(trs.re.y, trs.im.y);
        const float2 uu = a.aux[rbase + xs[h]];
        const float2 G = cmulc(v[e], uu);   // conj(u) v
        const float2 q = cmulc(tr, G);      // t conj(G)
        const float gd = k * q.y, gb = -k * q.x;
        const float gx0 = 1.0f - fx;
        float* r0 = mine + 2 * xi;
        atomicAdd(r0, gx0 * gd);
        atomicAdd(r0 + 1, gx0 * gb);
        atomicAdd(r0 + 2, fx * gd);
        atomicAdd(r0 + 3, fx * gb);
        v[e] = cmulc(v[e], tr);               // conj(t) v
      }
    }
  }
  __syncthreads();
  if (yi >= 0) {
    float* g0 = a.grad + static_cast<size_t>(yi) * nxv * 2;  // rows yi and yi + 1 are contiguous
    const float gy0 = 1.0f - fy;
    for (int j = t; j < 2 * nxv; j += T) {
      float val = acc[j];
      for (int c = 1; c < copies; ++c) val += acc[c * stride + j];
      if (val != 0.0f) {
        atomicAdd(&g0[j], gy0 * val);
        if (fy != 0.0f) atomicAdd(&g0[2 * nxv + j], fy * val);
      }
    }
  }
  __syncthreads();  // the forward transform reuses the buffer
  if (flags & ROW_FWD) {
    if constexpr (DITH) {
      fft_seq2x<N, false>(v, buf, t, a.twd1_fwd, dft_k1(a.k_fwd));
    } else {
      fft_seq<N, false>(v, buf, t, a.tw);
    }
    if (valid) {
#pragma unroll
      for (int e = 0; e < E; ++e) a.out[rbase + slot_pos<N, RX>(t, e)] = v[e];
    }
  } else if (valid) {
#pragma unroll
    for (int e = 0; e < E; ++e) a.out[rbase + slot_pos<N, RF>(t, e)] = v[e];
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

// Column position held by register e of thread t after the forward column transform.
template <int N, bool L2>
__device__ __forceinline__ int col_exit_pos(int t, int e) {
  if constexpr (L2) return Fft2L<N>::exit_pos(t, e);
  else return slot_pos<N, FftPlan<N>::exit_radix(false)>(t, e);
}

#ifndef RS_COL_MINB
#define RS_COL_MINB 1
#endif
template <int N, int W>
__global__ void __launch_bounds__(W * FftPlan<N>::T, (W * FftPlan<N>::T <= 512 ? RS_COL_MINB : 1))
    col_pass_kernel(const ColArgs a) {
  using P = FftPlan<N>;
  constexpr bool L2 = Fft2L<N>::ok(W);  // two-level column transforms (one block barrier each)
  constexpr int RF = P::entry_radix(false);
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
  // batched / strided transforms: this block's transform starts at blockIdx.y * bstride
  const size_t pitch = a.pitch ? static_cast<size_t>(a.pitch) : static_cast<size_t>(nx);
  const size_t boff = static_cast<size_t>(blockIdx.y) * static_cast<size_t>(a.bstride);
  const float2* in = a.in + boff;
  float2* out = a.out + boff;
  const int yrow0 = blockIdx.y * a.ey_bstride;

  if (flags & COL_FWD) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = in[static_cast<size_t>(slot_pos<N, RF>(t, e)) * pitch + x];
    if constexpr (L2) fft2l_fwd<N, PadAddr, PadAddr, 1, TwGlobal>(v, buf, t, a.tw2);
    else fft_seq<N, false>(v, buf, t, a.tw);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = in[static_cast<size_t>(col_exit_pos<N, L2>(t, e)) * pitch + x];
  }
  if (a.tw4) {
    // registers hold transform positions fy (forward exit == inverse entry mapping)
    const int q = a.tw4q ? static_cast<int>(blockIdx.y) : x;
    if (a.tw4t) {
      // compensated table; with q = blockIdx.y every column of the strip reads the same entry
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const float4 w = __ldg(&a.tw4t[(col_exit_pos<N, L2>(t, e) * q) & (a.tw4 - 1)]);
        v[e] = (flags & COL_FWD) ? cmul_tw(v[e], w) : cmulc_tw(v[e], w);
      }
    } else {
      // per-column q would scatter table reads over the warp: sincospif of the exact reduced
      // angle -2 (fy*q mod L)/L (exact in float for L <= 2^15) instead
      const float inv_half = 2.0f / static_cast<float>(a.tw4);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int pq = (col_exit_pos<N, L2>(t, e) * q) & (a.tw4 - 1);
        float sn, cs;
        sincospif(-static_cast<float>(pq) * inv_half, &sn, &cs);
        v[e] = cmul(v[e], make_float2(cs, (flags & COL_FWD) ? sn : -sn));
      }
    }
  }

  // registers are in the forward-exit (== inverse-entry) mapping: position = fy; with H applied
  // the 1/N of the inverse is folded into ey, as in the pipelined column pass
  const bool fold = (flags & COL_H) && (flags & COL_SCALE) && !(flags & COL_SPEC);  // U stays unscaled
  if (flags & (COL_H | COL_MASK)) {
    const int lim = __ldg(&a.ylim[x]);
    const float2 exv = (flags & COL_H) ? __ldg(&a.ex[x]) : make_float2(1.f, 0.f);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int fy = col_exit_pos<N, L2>(t, e);
      const int yr = yrow0 + fy;  // storage row of the table entries
      const int m = a.kyi ? __ldg(&a.kyi[yr]) : (fy < (N + 1) / 2 ? fy : fy - N);
      const bool keep = (m < 0 ? -m : m) <= lim;
      if (!keep) {
        v[e] = make_float2(0.f, 0.f);
      } else if (flags & COL_H) {
        const float2 eyv = fold ? cscale(__ldg(&a.ey[yr]), a.scale) : __ldg(&a.ey[yr]);
        v[e] = cmul(v[e], cmul(exv, eyv));
      }
    }
  }
  if ((flags & COL_SPEC) && live) {
#pragma unroll
    for (int e = 0; e < E; ++e) a.spec[boff + static_cast<size_t>(col_exit_pos<N, L2>(t, e)) * pitch + x] = v[e];
  }
  if ((flags & COL_SCALE) && !fold) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cscale(v[e], a.scale);
  }
  if (flags & COL_INV) {
    if constexpr (L2) fft2l_inv<N, PadAddr, PadAddr, 1, TwGlobal>(v, buf, t, a.tw2);
    else fft_seq<N, true>(v, buf, t, a.tw);
    if (live) {
#pragma unroll
      for (int e = 0; e < E; ++e) out[static_cast<size_t>(slot_pos<N, RF>(t, e)) * pitch + x] = v[e];
    }
  } else if (live) {
#pragma unroll
    for (int e = 0; e < E; ++e) out[static_cast<size_t>(col_exit_pos<N, L2>(t, e)) * pitch + x] = v[e];
  }
}

// --------------------------------------------------------------------------- launchers
// Implemented in rs_rows.cu / rs_cols.cu; return cudaErrorInvalidValue for unsupported N.
// Counts kernel launches made by this library (read through rs_launch_count).
void note_launch(unsigned n = 1);

// vox = false keeps the voxel-transmission specialisation out (a schedule choice of the plan).
cudaError_t launch_row_pass(int nx, const RowArgs& a, cudaStream_t s, bool vox = true);
// Adjoint row pass (row_adjoint_kernel) for power-of-two nx; cudaErrorInvalidValue otherwise.
cudaError_t launch_row_adjoint(int nx, const RowArgs& a, cudaStream_t s);
// Compensated stage-major twiddle tables of the fused passes for length n (fast sizes only).
cudaError_t launch_stage_twiddles(int n, float4* tw, cudaStream_t s);
// W_n^m for m < n, compensated, n a power of two (the four-step twiddle table).
cudaError_t launch_power_twiddles(int n, float4* tw, cudaStream_t s);
int stage_twiddle_len(int n);
// Two-level column-transform table of length n (0 when n has none) and its builder.
int twiddles_2l_len(int n);
cudaError_t launch_twiddles_2l(int n, float4* tw, cudaStream_t s);
cudaError_t launch_col_pass(int ny, const ColArgs& a, cudaStream_t s);
bool fast_size(int n);

}  // namespace rs
