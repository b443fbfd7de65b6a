// rs_abi.cu — plan object and the extern "C" entry points declared in include/rs_fresnel.h.
//
// Fast path: both axes are powers of two in [16, 16384]; a Fresnel step is one row pass and
// one column pass (plus one row pass to return to real space at the end of a run of slices).
// Generic path: any other size up to 6144 per axis, built from the direct-DFT and
// elementwise kernels (still on the GPU; there is no CPU fallback).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "rs_fresnel.h"
#include "rs_misc.cuh"
#include "rs_pipe_api.cuh"
#include "rs_x2_api.cuh"

using namespace rs;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define RS_CK(call)                                                                    \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) return fail(RS_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define RS_TRY(expr)              \
  do {                            \
    int st_ = (expr);             \
    if (st_ != RS_OK) return st_; \
  } while (0)

constexpr int kGenericMax = 6144;

// Default pass variants: the bulk-copy pipeline pays off for the column passes (it replaces 16
// strided loads per thread); rows keep the per-block kernel, which holds more rows in flight.
#ifndef RS_DEFAULT_PIPE_ROWS
#define RS_DEFAULT_PIPE_ROWS 0
#endif
constexpr bool kDefaultPipeRows = RS_DEFAULT_PIPE_ROWS != 0;
constexpr bool kDefaultPipeCols = true;

std::atomic<unsigned long long> g_launches{0};
std::atomic<unsigned long long> g_allocs{0};  // device and pinned allocations made by this library

cudaError_t counted_malloc(void** ptr, size_t bytes) {
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  return cudaMalloc(ptr, bytes);
}

bool finite_pos(double v) { return std::isfinite(v) && v > 0.0; }

// Four-step plans split each axis as n = n1 * kFourN2.
constexpr int kFourN2 = 256;
bool four_size(int n) { return n >= 16 * kFourN2 && n <= 32768 && (n & (n - 1)) == 0; }

}  // namespace

namespace rs {
void note_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace rs

struct rs_plan {
  int nx = 0, ny = 0, dev = 0;
  bool fast = false;
  // Four-step plans (axes n = n1 * 256 up to 32768): each axis transform is a length-n1 column
  // transform with the W_n twiddle fused, then a length-256 transform; the spectrum is kept in
  // four-step storage order (frequency i / 256 + n1 * (i % 256) at entry i of an axis).
  bool four = false;
  float4* tw_256 = nullptr;   // stage-major table of the length-256 transforms (rows and columns)
  float4* tw2_256 = nullptr;  // two-level table of the length-256 column transform
  float4* tw_c1x = nullptr;   // stage-major tables of the length-n1 column transforms
  float4* tw_c1y = nullptr;
  float4* tw4y = nullptr;     // W_ny^m for the fused y twiddles (compensated; the x ones use sincospif)
  int* kyi = nullptr;         // signed y-frequency index per storage row
  // Split columns (fast plans with ny = n1 * 256 in [4096, 16384]): the fused column pass of a
  // multislice step as three passes (length-n1 forward with W_ny, length-256 forward / H /
  // inverse, length-n1 inverse), selected by RS_SCHED_SPLIT_COLS.
  bool split_ok = false;
  bool split_cols = false;
  float2* ey_s = nullptr;     // ey in four-step storage order
  void* arena = nullptr;
  float4* tws_x = nullptr;  // compensated stage-major twiddles (fast sizes)
  float4* tws_y = nullptr;
  float4* tw2_y = nullptr;  // two-level column-transform table (power-of-two ny >= 256)
  float2* tw_x = nullptr;   // plain twiddles of the direct-DFT path (other sizes)
  float2* tw_y = nullptr;
  float2* ex = nullptr;
  float2* ey = nullptr;
  int* ylim = nullptr;
  int* xi = nullptr;
  float* xf = nullptr;
  int2* xp = nullptr;
  int* yi = nullptr;
  float* yf = nullptr;
  void* det = nullptr;
  size_t det_cap = 0;
  float2* plane = nullptr;  // one slice plane of plasma (delta, beta) for the voxel row kernel
  size_t plane_cap = 0;
  // Geometry whose forward detector tables sit in `det` (valid = false after any other use of the
  // buffer). A repeated geometry needs neither the host build nor the copy; the copy matters,
  // because a pageable host->device copy first waits for all earlier work on its stream.
  struct DetCache {
    bool valid = false;
    rs_detector_geom g{};
    size_t off[8] = {};
  } det_cache;
  // Pass schedule (rs_plan_set_schedule): pipelined (bulk-copy, persistent) passes per direction,
  // and whether the voxel-only row kernel takes the multislice rows. RS_PIPELINE sets the first two
  // at plan creation.
  bool pipe_rows = true;
  bool pipe_cols = true;
  bool row_vox = true;
  int* status = nullptr;  // device word set by bounded waits that gave up
  // Pinned copy of `status`, refreshed by a 4-byte copy queued at the end of every call that ran a
  // pipelined pass (status_pending), so a host that has synchronised its stream can read it
  // without another device synchronisation (rs_plan_check).
  volatile int* status_host = nullptr;
  bool status_pending = false;
  int test_stall = 0;     // one-shot: the next pipelined column pass waits on a barrier nobody completes
  // Split-pair multislice passes (rs_x2.cuh): kDitherTables dithered copies of the row stage table
  // and of the two-level column table, and the matching DFT constants; slice k uses copy k mod K.
  // schedule: cleared by RS_SCHED_COMP_ROWS / RS_SCHED_COMP_COLS; the default runs the split-pair
  // column passes and the dithered rows one row per thread group (4096^2 row pass: 127 us against
  // 142 us with compensated twiddles and 158 us as split pairs)
  bool x2r_on = true, x2c_on = true;
  bool x2_rows = false, x2_cols = false;  // available for this plan's sizes
  bool d1_rows = true;                    // dithered rows one per thread group (RS_SCHED_SINGLE_ROWS)
  bool d1_only_rows = false;              // dithered rows exist only one per thread group (no split pairs)
  const volatile int* cancel = nullptr;   // host flag read between slices (rs_plan_set_cancel_flag)
  bool d1_cols = false;                   // dithered columns one per thread group (RS_SCHED_SINGLE_COLS)
  bool d1_only_cols = false;              // dithered columns exist only one per thread group (3*2^k)
  void* twd_arena = nullptr;
  float4* twd_x = nullptr;
  float4* twd_y2 = nullptr;
  float2* twd1_x = nullptr;               // twd_x as (wr, wi) entries, for the single-sequence rows
  float2* twd1_y2 = nullptr;              // twd_y2 likewise, for the single-sequence columns (for
                                          // d1_only_cols: the stage-major table of ny)
  int twd_x_len = 0, twd_y2_len = 0;
  DftConsts kconst[kDitherTables];
  struct MapEntry {
    const void* ptr = nullptr;
    int w = 0, bh = 0, depth = 1;
    CUtensorMap map;
  };
  MapEntry maps[4];
  int map_next = 0;
  // optional per-pass event timing of the multislice loop (rs_plan_profile)
  bool prof = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;  // 0 = row pass, 1 = column pass, per event pair
  size_t ev_used = 0;
};

namespace {

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

int check_plan(const rs_plan* p) {
  if (!p) return fail(RS_EINVAL, "plan is NULL");
  int dev = -1;
  RS_CK(cudaGetDevice(&dev));
  if (dev != p->dev) return fail(RS_EINVAL, "plan was created on device %d but device %d is current", p->dev, dev);
  return RS_OK;
}

// Entry points whose passes need the natural-order spectrum or the fused single-length passes.
int check_plan_std(const rs_plan* p, const char* name) {
  RS_TRY(check_plan(p));
  if (p->four)
    return fail(RS_EUNSUPPORTED, "%s: a four-step plan (%dx%d) supports rs_propagate, rs_point_source, "
                "rs_point_source_propagate and rs_detector only", name, p->nx, p->ny);
  return RS_OK;
}

int build_prop(rs_plan* p, double dx, double dy, double wl, double dz, double cutoff, bool with_h,
               cudaStream_t s) {
  if (!finite_pos(dx) || !finite_pos(dy)) return fail(RS_EINVAL, "dx and dy must be positive and finite (dx=%g, dy=%g)", dx, dy);
  if (with_h && (!finite_pos(wl) || !std::isfinite(dz)))
    return fail(RS_EINVAL, "wavelength must be positive and dz finite (wl=%g, dz=%g)", wl, dz);
  if (std::isnan(cutoff)) return fail(RS_EINVAL, "cutoff frequency is NaN");
  PropTabArgs a{};
  a.nx = p->nx;
  a.ny = p->ny;
  a.dx = dx;
  a.dy = dy;
  // numpy: phase_scale = -1j*np.pi*wl*dz -> imaginary part -((pi*wl)*dz);
  //        global_phase = exp(1j*2*np.pi/wl*dz) -> angle ((2*pi)/wl)*dz; freq_sq = 2.0*freq**2
  a.ps = with_h ? -((M_PI * wl) * dz) : 0.0;
  a.gphi = with_h ? ((2.0 * M_PI) / wl) * dz : 0.0;
  a.freq_sq = 2.0 * std::pow(cutoff, 2.0);
  a.with_h = with_h ? 1 : 0;
  a.ex = p->ex;
  a.ey = p->ey;
  a.ylim = p->ylim;
  if (p->four) {
    a.n2x = kFourN2;
    a.n2y = kFourN2;
    a.kyi = p->kyi;
  }
  RS_CK(launch_prop_tables(a, s));
  if (p->split_ok && with_h) {  // ey and the frequency index of each row in four-step order
    PropTabArgs b = a;
    b.ex = nullptr;
    b.ylim = nullptr;
    b.ey = p->ey_s;
    b.kyi = p->kyi;
    b.n2y = kFourN2;
    RS_CK(launch_prop_tables(b, s));
  }
  return RS_OK;
}

int build_axes(rs_plan* p, const rs_voxel_geom* g, double dx, double dy, double cs, cudaStream_t s) {
  AxisTabArgs ax{p->nx, dx, cs, g->x_pos, g->nx_v, g->pixel_size_x, p->xi, p->xf, p->xp};
  RS_CK(launch_axis_table(ax, s));
  AxisTabArgs ay{p->ny, dy, cs, g->y_pos, g->ny_v, g->pixel_size_y, p->yi, p->yf, nullptr};
  RS_CK(launch_axis_table(ay, s));
  return RS_OK;
}

AxisTab axis_tab(const rs_plan* p) { return AxisTab{p->xi, p->xf, p->yi, p->yf, p->xp}; }

// At the end of an entry point that ran pipelined passes: queue the copy of the device status
// word into the plan's pinned host word on the caller's stream (stream-ordered, no host sync).
struct StatusNote {
  rs_plan* p;
  cudaStream_t s;
  StatusNote(rs_plan* plan, void* stream) : p(plan), s(static_cast<cudaStream_t>(stream)) {}
  ~StatusNote() {
    if (p && p->status_pending && p->status_host) {
      p->status_pending = false;
      cudaMemcpyAsync(const_cast<int*>(p->status_host), p->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
  }
};

// ---- pipelined passes -------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool tensor_map_encoder() {
  static bool tried = false;
  if (!tried) {
    tried = true;
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  return g_encode != nullptr;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Tensor map of a stack of `depth` (ny, nx) complex64 fields viewed as 8-byte elements (3D: x, y,
// field), box (w columns, bh rows, one field); depth 1 for a single field.
const CUtensorMap* field_map(rs_plan* p, const void* base, int w, int bh, int depth = 1) {
  for (auto& m : p->maps)
    if (m.ptr == base && m.w == w && m.bh == bh && m.depth == depth) return &m.map;
  auto& slot = p->maps[p->map_next];
  p->map_next = (p->map_next + 1) % 4;
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(p->nx), static_cast<cuuint64_t>(p->ny),
                        static_cast<cuuint64_t>(depth)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(p->nx) * 8,
                           static_cast<cuuint64_t>(p->nx) * static_cast<cuuint64_t>(p->ny) * 8};
  cuuint32_t box[3] = {static_cast<cuuint32_t>(w), static_cast<cuuint32_t>(bh), 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = g_encode(&slot.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(base), dims, strides,
                              box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    slot.ptr = nullptr;
    return nullptr;
  }
  slot.ptr = base;
  slot.w = w;
  slot.bh = bh;
  slot.depth = depth;
  return &slot.map;
}

cudaError_t run_row(rs_plan* p, const RowArgs& r, cudaStream_t s) {
  if (p->pipe_rows && !(r.flags & ROW_STORE_U) && row_pipe_ok(p->nx) && (r.flags & ROW_SRC || aligned16(r.in)) &&
      aligned16(r.out)) {
    p->status_pending = true;
    return launch_row_pipe(p->nx, r, p->status, s);
  }
  return launch_row_pass(p->nx, r, s, p->row_vox);
}

// The fused column pass of a multislice step (FWD | H | SCALE | INV, no spectrum store) as three
// four-step passes over the y axis; rows come back in natural order.
cudaError_t run_col_split(rs_plan* p, const ColArgs& c, cudaStream_t s) {
  const int n1y = p->ny / kFourN2;
  auto ycols = [&](const float2* in, float2* out, int flags) {
    ColArgs y{};
    y.in = in; y.out = out; y.nx = p->nx; y.flags = flags; y.tw = p->tw_c1y;
    y.pitch = static_cast<long long>(kFourN2) * p->nx; y.bstride = p->nx; y.batches = kFourN2;
    y.tw4 = p->ny; y.tw4q = 1; y.tw4t = p->tw4y;
    return launch_col_pass(n1y, y, s);
  };
  cudaError_t e = ycols(c.in, c.out, COL_FWD);
  if (e != cudaSuccess) return e;
  ColArgs m{};
  m.in = c.out; m.out = c.out; m.nx = p->nx; m.tw = p->tw_256; m.tw2 = p->tw2_256;
  m.ex = c.ex; m.ey = p->ey_s; m.ylim = c.ylim; m.kyi = p->kyi; m.scale = c.scale; m.flags = c.flags;
  m.pitch = p->nx; m.bstride = static_cast<long long>(kFourN2) * p->nx; m.batches = n1y; m.ey_bstride = kFourN2;
  e = launch_col_pass(kFourN2, m, s);
  if (e != cudaSuccess) return e;
  return ycols(c.out, c.out, COL_INV);
}

cudaError_t run_col(rs_plan* p, const ColArgs& ca, cudaStream_t s) {
  const bool stacked = ca.batches > 1;  // stacked fields: a batch of equal fields, bstride apart
  if (!stacked && p->split_cols && p->split_ok && ca.flags == (COL_FWD | COL_H | COL_SCALE | COL_INV) &&
      ca.ey == p->ey)
    return run_col_split(p, ca, s);
  ColArgs c = ca;
  c.tw2 = p->tw2_y;
  int w = 0, bh = 0;
  const int depth = stacked ? ca.batches : 1;
  // the pipeline takes a stack whose fields follow each other without gaps (3D tensor maps)
  const bool dense = !stacked || ca.bstride == static_cast<long long>(p->nx) * p->ny;
  if (dense && c.pitch == 0 && c.tw4 == 0 && !c.kyi && p->pipe_cols && col_pipe_box(p->ny, &w, &bh) &&
      aligned16(c.in) && aligned16(c.out) && tensor_map_encoder()) {
    // Copy the input map before the output lookup: encoding the output may recycle its slot.
    const CUtensorMap* mi = field_map(p, c.in, w, bh, depth);
    if (mi) {
      const CUtensorMap in_copy = *mi;
      const CUtensorMap* mo = field_map(p, c.out, w, bh, depth);
      if (mo) {
        p->status_pending = true;
        c.test_stall = p->test_stall;
        p->test_stall = 0;
        return launch_col_pipe(p->ny, c, in_copy, *mo, StripBox{w, bh}, p->status, s);
      }
    }
  }
  return launch_col_pass(p->ny, c, s);
}

// The multislice column pass on split pairs with table j (rs_x2.cuh), when the plan's schedule
// and sizes allow it; otherwise the column pass of the schedule. Returns cudaErrorNotSupported
// through `used` = false so the caller can tell which ran.
cudaError_t run_col_ms(rs_plan* p, const ColArgs& ca, int j, bool* used, cudaStream_t s) {
  *used = false;
  int w = 0, bh = 0;
  const int depth = ca.batches > 1 ? ca.batches : 1;
  const bool dense = depth == 1 || ca.bstride == static_cast<long long>(p->nx) * p->ny;
  // dithered columns: split pairs (col_x2_box strips) or one column per thread group
  // (col_d1_box strips), the same values
  const bool single = p->d1_cols || p->d1_only_cols;
  const bool boxed = single ? col_d1_box(p->ny, &w, &bh) : col_x2_box(p->ny, &w, &bh);
  if (p->x2c_on && (p->x2_cols || p->d1_only_cols) && dense && ca.pitch == 0 && ca.tw4 == 0 && !ca.kyi && boxed &&
      aligned16(ca.in) && aligned16(ca.out) && tensor_map_encoder()) {
    const CUtensorMap* mi = field_map(p, ca.in, w, bh, depth);
    if (mi) {
      const CUtensorMap in_copy = *mi;
      const CUtensorMap* mo = field_map(p, ca.out, w, bh, depth);
      if (mo) {
        ColArgs c = ca;
        c.twd = p->twd_y2 + static_cast<size_t>(j) * p->twd_y2_len;
        c.twd1 = p->twd1_y2 + static_cast<size_t>(j) * p->twd_y2_len;
        c.kc = p->kconst[j];
        c.test_stall = p->test_stall;
        p->test_stall = 0;
        p->status_pending = true;
        *used = true;
        return single ? launch_col_d1(p->ny, c, in_copy, *mo, StripBox{w, bh}, p->status, s)
                      : launch_col_x2(p->ny, c, in_copy, *mo, StripBox{w, bh}, p->status, s);
      }
    }
  }
  return run_col(p, ca, s);
}

// Records a start event before a pass when profiling is on; returns the pair index or -1.
int prof_begin(rs_plan* p, int kind, cudaStream_t s) {
  if (!p->prof) return -1;
  if (p->ev_used + 2 > p->ev_pool.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return -1;
      p->ev_pool.push_back(e);
    }
  }
  const size_t i = p->ev_used;
  p->ev_used += 2;
  p->ev_kind.push_back(kind);
  cudaEventRecord(p->ev_pool[i], s);
  return static_cast<int>(i);
}

void prof_end(rs_plan* p, int idx, cudaStream_t s) {
  if (idx >= 0) cudaEventRecord(p->ev_pool[idx + 1], s);
}

// ---- buffers that grow with the geometry (sized up front by rs_plan_reserve) --------------
// Growing one frees the old buffer (cudaFree waits for the work still using it) and allocates a
// larger one; rs_plan_reserve does this before a run so that the run itself allocates nothing.
int grow_det(rs_plan* p, size_t bytes) {
  if (bytes <= p->det_cap) return RS_OK;
  p->det_cache.valid = false;
  if (p->det) RS_CK(cudaFree(p->det));
  p->det = nullptr;
  p->det_cap = 0;
  cudaError_t e = counted_malloc(&p->det, bytes);
  if (e != cudaSuccess) return fail(RS_ENOMEM, "cudaMalloc(%zu) for detector tables: %s", bytes, cudaGetErrorString(e));
  p->det_cap = bytes;
  return RS_OK;
}

int grow_plane(rs_plan* p, size_t voxels) {
  if (voxels <= p->plane_cap) return RS_OK;
  if (p->plane) RS_CK(cudaFree(p->plane));
  p->plane = nullptr;
  p->plane_cap = 0;
  cudaError_t e = counted_malloc(reinterpret_cast<void**>(&p->plane), voxels * sizeof(float2));
  if (e != cudaSuccess) return fail(RS_ENOMEM, "cudaMalloc for a plasma slice plane: %s", cudaGetErrorString(e));
  p->plane_cap = voxels;
  return RS_OK;
}


// ---- building blocks (stream-ordered, no host sync) ----------------------------------
int fft2_impl(rs_plan* p, const float2* in, float2* out, cudaStream_t s) {
  if (p->fast) {
    RowArgs r{};
    r.in = in; r.out = out; r.ny = p->ny; r.flags = ROW_FWD; r.tw = p->tws_x;
    RS_CK(run_row(p, r, s));
    ColArgs c{};
    c.in = out; c.out = out; c.nx = p->nx; c.flags = COL_FWD; c.tw = p->tws_y;
    RS_CK(run_col(p, c, s));
  } else {
    RS_CK(launch_dft_axis(in, out, p->nx, p->ny, 0, 0, p->tw_x, 1.0f, s));
    RS_CK(launch_dft_axis(out, out, p->nx, p->ny, 1, 0, p->tw_y, 1.0f, s));
  }
  return RS_OK;
}

int ifft2_impl(rs_plan* p, const float2* in, float2* out, cudaStream_t s) {
  const float inv_n = static_cast<float>(1.0 / (static_cast<double>(p->nx) * p->ny));
  if (p->fast) {
    ColArgs c{};
    c.in = in; c.out = out; c.nx = p->nx; c.flags = COL_INV | COL_SCALE; c.scale = inv_n; c.tw = p->tws_y;
    RS_CK(run_col(p, c, s));
    RowArgs r{};
    r.in = out; r.out = out; r.ny = p->ny; r.flags = ROW_INV; r.tw = p->tws_x;
    RS_CK(run_row(p, r, s));
  } else {
    RS_CK(launch_dft_axis(in, out, p->nx, p->ny, 1, 1, p->tw_y, 1.0f, s));
    RS_CK(launch_dft_axis(out, out, p->nx, p->ny, 0, 1, p->tw_x, inv_n, s));
  }
  return RS_OK;
}

// propagate_2d on a four-step plan: seven passes (rs_propagate documents the order). u -> U:
// x transforms (length-n1 columns of each row's (n1, 256) view with the W_nx twiddle, then
// length-256 rows), the length-n1 y transforms over rows 256*m1 + m2 with the W_ny twiddle;
// then one pass of length-256 y transforms, H, the spectrum store and the inverse; then the
// inverse y and x steps on u. U is left holding the spectrum in four-step storage order.
int propagate_four(rs_plan* p, float2* u, float2* U, bool skip_fft, cudaStream_t s) {
  const int n1x = p->nx / kFourN2, n1y = p->ny / kFourN2;
  const float inv_n = static_cast<float>(1.0 / (static_cast<double>(p->nx) * p->ny));
  auto xcols = [&](const float2* in, float2* out, int flags) {
    ColArgs c{};
    c.in = in; c.out = out; c.nx = kFourN2; c.flags = flags; c.tw = p->tw_c1x;
    c.pitch = kFourN2; c.bstride = p->nx; c.batches = p->ny; c.tw4 = p->nx; c.tw4q = 0;  // sincospif twiddles
    return launch_col_pass(n1x, c, s);
  };
  auto xrows = [&](float2* f, int flags) {
    RowArgs r{};
    r.in = f; r.out = f; r.ny = p->ny * n1x; r.flags = flags; r.tw = p->tw_256;
    return launch_row_pass(kFourN2, r, s);
  };
  auto ycols = [&](float2* f, int flags) {
    ColArgs c{};
    c.in = f; c.out = f; c.nx = p->nx; c.flags = flags; c.tw = p->tw_c1y;
    c.pitch = static_cast<long long>(kFourN2) * p->nx; c.bstride = p->nx; c.batches = kFourN2;
    c.tw4 = p->ny; c.tw4q = 1; c.tw4t = p->tw4y;
    return launch_col_pass(n1y, c, s);
  };
  if (!skip_fft) {
    RS_CK(xcols(u, U, COL_FWD));
    RS_CK(xrows(U, ROW_FWD));
    RS_CK(ycols(U, COL_FWD));
  }
  ColArgs c{};
  c.in = U; c.out = u; c.spec = U; c.nx = p->nx; c.tw = p->tw_256; c.tw2 = p->tw2_256;
  c.ex = p->ex; c.ey = p->ey; c.ylim = p->ylim; c.kyi = p->kyi; c.scale = inv_n;
  c.pitch = p->nx; c.bstride = static_cast<long long>(kFourN2) * p->nx; c.batches = n1y; c.ey_bstride = kFourN2;
  c.flags = (skip_fft ? 0 : COL_FWD) | COL_H | COL_SPEC | COL_SCALE | COL_INV;
  RS_CK(launch_col_pass(kFourN2, c, s));
  RS_CK(ycols(u, COL_INV));
  RS_CK(xrows(u, ROW_INV));
  RS_CK(xcols(u, u, COL_INV));
  return RS_OK;
}

// Transmission of slice s (already tabulated in the plan's axis tables) and one Fresnel step
// on the generic path: u *= T; U = FFT2(u); U *= H*mask; u = IFFT2(U).
int generic_slice(rs_plan* p, float2* u, float2* U, const VoxelArgs* vox, const PlasmaArgs* pl,
                  cudaStream_t s) {
  if (vox || pl) RS_CK(launch_transmission(u, p->nx, p->ny, axis_tab(p), vox, pl, s));
  RS_TRY(fft2_impl(p, u, U, s));
  RS_CK(launch_transfer(U, p->nx, p->ny, p->ex, p->ey, p->ylim, 1, nullptr, s));
  RS_TRY(ifft2_impl(p, U, u, s));
  return RS_OK;
}

struct SliceSource {
  // exactly one of vox / pl is used
  bool plasma = false;
  int batch = 1;               // stacked fields (same size, energy and sample; consecutive in u and U)
  const char* grid = nullptr;  // voxel ids
  const float2* dbv = nullptr; // or (delta, beta) per voxel
  int grid_signed = 0;
  const float2* db = nullptr;
  int n_db = 0;
  const char* pg[4] = {nullptr, nullptr, nullptr, nullptr};  // plasma grids
  int f64 = 1;
  PlasmaArgs pl_base{};
  float2* store = nullptr;     // optional: the field entering slice z goes to store + (z - s0) * nx * ny
  bool fields_only = false;    // with store: stop once the last field is stored (u, U left unspecified)
};

// Shared driver of the voxel and plasma multislice entry points.
int multislice(rs_plan* p, float2* u, float2* U, const SliceSource& src, const rs_voxel_geom* g,
               double dx, double dy, double wl, double cutoff, const double* slice_dz,
               const double* coord_scale, int s0, int s1, cudaStream_t s) {
  if (!u || !U) return fail(RS_EINVAL, "u and U must be device pointers");
  if (!g) return fail(RS_EINVAL, "geometry is NULL");
  if (g->nz <= 0 || g->ny_v < 2 || g->nx_v < 2)
    return fail(RS_EINVAL, "grid must be (nz>0, ny>=2, nx>=2), got (%d, %d, %d)", g->nz, g->ny_v, g->nx_v);
  if (!finite_pos(g->pixel_size_x) || !finite_pos(g->pixel_size_y) || !finite_pos(g->pixel_size_z))
    return fail(RS_EINVAL, "voxel pitches must be positive");
  if (s0 < 0 || s1 > g->nz || s0 > s1) return fail(RS_EINVAL, "slice range [%d, %d) outside [0, %d]", s0, s1, g->nz);
  if (!slice_dz) return fail(RS_EINVAL, "slice_dz is NULL");
  if (!finite_pos(wl)) return fail(RS_EINVAL, "wavelength must be positive");
  if (s0 == s1) return RS_OK;
  if (src.batch < 1) return fail(RS_EINVAL, "batch must be >= 1, got %d", src.batch);
  if (src.batch > 1 && !p->fast) return fail(RS_EUNSUPPORTED, "stacked fields need a fused-kernel plan");
  if (src.batch > 1 && static_cast<long long>(p->ny) * src.batch > (1LL << 30))
    return fail(RS_EINVAL, "batch %d x %d rows is too many", src.batch, p->ny);
  const size_t plane = static_cast<size_t>(g->ny_v) * g->nx_v;
  const float a = static_cast<float>(g->pixel_size_z / wl);
  const float inv_n = static_cast<float>(1.0 / (static_cast<double>(p->nx) * p->ny));

  // Split-pair row passes (voxel transmission only: ids, per-voxel delta/beta or a plasma plane);
  // slice z's forward transform and slice z + 1's inverse use dithered table z mod K, so every
  // transform is undone by one with the same table.
  const bool plasma_rows_vox = !src.plasma || (p->fast && p->row_vox && !src.store);
  const bool x2r = p->fast && p->x2r_on && (p->x2_rows || p->d1_only_rows) && plasma_rows_vox &&
                   g->nx_v <= row_x2_slots(p->nx);
  auto table_x = [&](int z) { return p->twd_x + static_cast<size_t>(z % kDitherTables) * p->twd_x_len; };
  auto table1_x = [&](int z) { return p->twd1_x + static_cast<size_t>(z % kDitherTables) * p->twd_x_len; };
  // the dithered rows, as split pairs or one row per thread group (the same values)
  auto launch_rows_dith = [&](RowArgs& r, int z_fwd, int z_inv, cudaStream_t st) {
    if (z_fwd >= 0) {
      r.twd_fwd = table_x(z_fwd);
      r.twd1_fwd = table1_x(z_fwd);
      r.k_fwd = p->kconst[z_fwd % kDitherTables];
    }
    if (z_inv >= 0) {
      r.twd_inv = table_x(z_inv);
      r.twd1_inv = table1_x(z_inv);
      r.k_inv = p->kconst[z_inv % kDitherTables];
    }
    return p->d1_rows || !p->x2_rows ? launch_row_d1(p->nx, r, st) : launch_row_x2(p->nx, r, st);
  };
  double cur_dz = NAN, cur_cs = NAN;
  for (int z = s0; z < s1; ++z) {
    if (p->cancel && *p->cancel) return fail(RS_ECANCELLED, "cancelled before slice %d of [%d, %d)", z, s0, s1);
    const double dz = slice_dz[z];
    const double cs = coord_scale ? coord_scale[z] : 1.0;
    if (!(dz == cur_dz)) {
      RS_TRY(build_prop(p, dx, dy, wl, dz, cutoff, true, s));
      cur_dz = dz;
    }
    if (!(cs == cur_cs)) {
      if (!std::isfinite(cs)) return fail(RS_EINVAL, "coordinate scale of slice %d is not finite", z);
      RS_TRY(build_axes(p, g, dx, dy, cs, s));
      cur_cs = cs;
    }
    VoxelArgs vox{};
    PlasmaArgs pl{};
    if (!src.plasma) {
      vox.slice = src.grid ? src.grid + plane * z * 4 : nullptr;
      vox.dbv = src.dbv ? src.dbv + plane * z : nullptr;
      vox.grid_signed = src.grid_signed;
      vox.nxv = g->nx_v;
      vox.nyv = g->ny_v;
      vox.db = src.db;
      vox.n_db = src.n_db;
      vox.a = a;
    } else {
      pl = src.pl_base;
      const size_t es = src.f64 ? 8 : 4;
      pl.ne = src.pg[0] + plane * z * es;
      pl.ni = src.pg[1] + plane * z * es;
      pl.te = src.pg[2] + plane * z * es;
      pl.zs = src.pg[3] + plane * z * es;
      pl.f64 = src.f64;
      pl.nxv = g->nx_v;
      pl.nyv = g->ny_v;
      pl.a = a;
    }
    // Plasma slices on the voxel-only row kernel: the plane's (delta, beta) first, then the row
    // pass reads them as a per-voxel volume (the same values and blends as the plasma row pass).
    const bool plasma_plane = src.plasma && p->fast && p->row_vox && !src.store;
    if (plasma_plane) {
      RS_TRY(grow_plane(p, plane));
      RS_CK(launch_plasma_plane(pl, p->plane, static_cast<int>(plane), s));
      vox = VoxelArgs{};
      vox.dbv = p->plane;
      vox.nxv = g->nx_v;
      vox.nyv = g->ny_v;
      vox.a = a;
    }
    if (p->fast) {
      RowArgs r{};
      r.in = u; r.out = u; r.ny = p->ny * src.batch; r.tw = p->tws_x; r.ax = axis_tab(p);
      r.axis_rows = src.batch > 1 ? p->ny : 0;
      const bool last_field = src.fields_only && z == s1 - 1;  // nothing after its store is needed
      r.flags = (z == s0 ? 0 : ROW_INV) |
                (last_field ? 0 : ROW_FWD | (src.plasma && !plasma_plane ? ROW_TPLASMA : ROW_TVOX));
      if (src.store) {
        r.flags |= ROW_STORE_U;
        r.aux = src.store + static_cast<size_t>(z - s0) * p->nx * p->ny;
      }
      r.vox = vox;
      r.pl = pl;
      const int er = prof_begin(p, 0, s);
      if (x2r) {
        RS_CK(launch_rows_dith(r, z, z != s0 ? z - 1 : -1, s));
      } else {
        RS_CK(run_row(p, r, s));
      }
      prof_end(p, er, s);
      if (last_field) break;
      ColArgs c{};
      c.in = u; c.out = u; c.spec = U; c.nx = p->nx; c.tw = p->tws_y;
      c.ex = p->ex; c.ey = p->ey; c.ylim = p->ylim; c.scale = inv_n;
      c.flags = COL_FWD | COL_H | COL_SCALE | COL_INV | (z == s1 - 1 ? COL_SPEC : 0);
      if (src.batch > 1) {
        c.batches = src.batch;
        c.bstride = static_cast<long long>(p->nx) * p->ny;
      }
      const int ec = prof_begin(p, 1, s);
      bool col_x2 = false;
      RS_CK(run_col_ms(p, c, z % kDitherTables, &col_x2, s));
      prof_end(p, ec, s);
    } else {
      RS_TRY(generic_slice(p, u, U, src.plasma ? nullptr : &vox, src.plasma ? &pl : nullptr, s));
    }
  }
  if (p->fast && !src.fields_only) {
    RowArgs r{};
    r.in = u; r.out = u; r.ny = p->ny * src.batch; r.tw = p->tws_x; r.flags = ROW_INV;
    if (x2r) {
      RS_CK(launch_rows_dith(r, -1, s1 - 1, s));
    } else {
      RS_CK(run_row(p, r, s));
    }
  }
  return RS_OK;
}

// ---- detector geometry (big-wave/propagation.py:766-815, 818-833, 949-992) -------------
struct DetTables {
  std::vector<double> xdet, ydet, yw;
  std::vector<float> xw;
  std::vector<int> xptr, xcell, yptr, ycell;
};


// Per-axis fractional overlap plan of the area_v1 detector (big-wave/propagation.py:949-977).
void area_axis(int out_n, double ds, int grid_n, double sp, std::vector<double>& det,
               std::vector<double>& lo, std::vector<double>& hi, std::vector<long>& ilo,
               std::vector<double>& flo, std::vector<long>& ihi, std::vector<double>& fhi) {
  det.resize(out_n); lo.resize(out_n); hi.resize(out_n);
  ilo.resize(out_n); flo.resize(out_n); ihi.resize(out_n); fhi.resize(out_n);
  const double gl = (static_cast<double>(-(grid_n / 2)) - 0.5) * sp;
  const double gr = gl + static_cast<double>(grid_n) * sp;
  for (int i = 0; i < out_n; ++i) {
    det[i] = (static_cast<double>(i) - static_cast<double>(out_n / 2)) * ds;
    lo[i] = det[i] - ds * 0.5;
    hi[i] = det[i] + ds * 0.5;
    const double clo = std::min(std::max(lo[i], gl), gr);
    double chi = std::min(std::max(hi[i], gl), gr);
    chi = std::max(chi, clo);
    const double slo = (clo - gl) / sp, shi = (chi - gl) / sp;
    ilo[i] = static_cast<long>(std::floor(slo));
    ihi[i] = static_cast<long>(std::floor(shi));
    flo[i] = slo - static_cast<double>(ilo[i]);
    fhi[i] = shi - static_cast<double>(ihi[i]);
    if (ilo[i] >= grid_n) { ilo[i] = grid_n; flo[i] = 0.0; }
    if (ihi[i] >= grid_n) { ihi[i] = grid_n; fhi[i] = 0.0; }
  }
}

// area_v1 row and column weights: separable physical overlap areas (big-wave/propagation.py:995-1110).
void build_area_v1(int nx, int ny, const rs_detector_geom& g, DetTables& t) {
  std::vector<double> xlo, xhi, ylo, yhi, fx0, fx1, fy0, fy1;
  std::vector<long> ix0, ix1, iy0, iy1;
  area_axis(g.out_x, g.ds_px, nx, g.dx, t.xdet, xlo, xhi, ix0, fx0, ix1, fx1);
  area_axis(g.out_y, g.ds_py, ny, g.dy, t.ydet, ylo, yhi, iy0, fy0, iy1, fy1);
  // x: integral = dx*(sum_{i0<=k<i1} I_k - f0*I_i0 + f1*I_i1), terms at index nx dropped
  t.xptr.assign(1, 0);
  for (int o = 0; o < g.out_x; ++o) {
    const long i0 = ix0[o], i1 = ix1[o];
    for (long k = i0; k <= i1 && k < nx; ++k) {
      double w = (k < i1) ? 1.0 : 0.0;
      if (k == i0) w -= fx0[o];
      if (k == i1) w += fx1[o];
      if (w != 0.0) {
        t.xcell.push_back(static_cast<int>(k));
        t.xw.push_back(static_cast<float>(w * g.dx));
      }
    }
    t.xptr.push_back(static_cast<int>(t.xcell.size()));
  }
  // y: per grid row, detector rows with positive overlap (searchsorted right/left as in 1035-1036)
  std::vector<std::vector<std::pair<int, double>>> per(g.out_y);
  const double gyl = (static_cast<double>(-(ny / 2)) - 0.5) * g.dy;
  for (int gy = 0; gy < ny; ++gy) {
    const double cl = gyl + static_cast<double>(gy) * g.dy;
    const double ch = cl + g.dy;
    const int first = static_cast<int>(std::upper_bound(yhi.begin(), yhi.end(), cl) - yhi.begin());
    const int end = static_cast<int>(std::lower_bound(ylo.begin(), ylo.end(), ch) - ylo.begin());
    for (int oy = first; oy < end; ++oy) {
      const double ov = std::min(ch, yhi[oy]) - std::max(cl, ylo[oy]);
      if (ov > 0) per[oy].push_back({gy, ov});
    }
  }
  t.yptr.assign(1, 0);
  for (int oy = 0; oy < g.out_y; ++oy) {
    for (auto& e : per[oy]) { t.ycell.push_back(e.first); t.yw.push_back(e.second); }
    t.yptr.push_back(static_cast<int>(t.ycell.size()));
  }
}

// legacy_fastwave truncated ranges and count map (big-wave/propagation.py:836-946).
void build_legacy(int nx, int ny, const rs_detector_geom& g, DetTables& t) {
  auto ranges = [](int out_n, int grid_n, double ds, double sp, std::vector<double>& det,
                   std::vector<long>& lo, std::vector<long>& hi) {
    det.resize(out_n); lo.resize(out_n); hi.resize(out_n);
    for (int i = 0; i < out_n; ++i) {
      det[i] = (static_cast<double>(i) - static_cast<double>(out_n / 2)) * ds;
      long l = static_cast<long>(std::trunc((det[i] - ds * 0.5) / sp)) + grid_n / 2;
      long h = static_cast<long>(std::trunc((det[i] + ds * 0.5) / sp)) + grid_n / 2;
      lo[i] = std::min<long>(std::max<long>(l, 0), grid_n);
      hi[i] = std::min<long>(std::max<long>(h, 0), grid_n);
    }
  };
  std::vector<long> lx, hx, ly, hy;
  ranges(g.out_x, nx, g.ds_px, g.dx, t.xdet, lx, hx);
  ranges(g.out_y, ny, g.ds_py, g.dy, t.ydet, ly, hy);
  t.xptr.assign(1, 0);
  for (int o = 0; o < g.out_x; ++o) {
    for (long k = lx[o]; k < hx[o]; ++k) { t.xcell.push_back(static_cast<int>(k)); t.xw.push_back(1.0f); }
    t.xptr.push_back(static_cast<int>(t.xcell.size()));
  }
  // rows gy with lo_y[oy] <= gy < hi_y[oy] (searchsorted right on both, 884-885)
  const double w = g.dx * g.dy;
  t.yptr.assign(1, 0);
  for (int oy = 0; oy < g.out_y; ++oy) {
    for (long gy = ly[oy]; gy < hy[oy]; ++gy) { t.ycell.push_back(static_cast<int>(gy)); t.yw.push_back(w); }
    t.yptr.push_back(static_cast<int>(t.ycell.size()));
  }
}

size_t align8(size_t v) { return (v + 7) & ~static_cast<size_t>(7); }

// Byte offsets of the forward detector tables in one buffer; returns the buffer size.
size_t det_layout(const DetTables& t, size_t o[8]) {
  o[0] = 0;                                     // xdet
  o[1] = o[0] + align8(t.xdet.size() * 8);      // ydet
  o[2] = o[1] + align8(t.ydet.size() * 8);      // yw
  o[3] = o[2] + align8(t.yw.size() * 8);        // xw
  o[4] = o[3] + align8(t.xw.size() * 4);        // xptr
  o[5] = o[4] + align8(t.xptr.size() * 4);      // xcell
  o[6] = o[5] + align8(t.xcell.size() * 4);     // yptr
  o[7] = o[6] + align8(t.yptr.size() * 4);      // ycell
  return o[7] + align8(t.ycell.size() * 4) + 8;
}

}  // namespace

// Dithered copies of cos(pi/8), sin(pi/8), sqrt(2)/2 (radix 8 and 16) and cos(pi/12), sin(pi/12),
// sqrt(3)/2 (radix 3 and 24) for the dithered DFTs: in copy j each
// constant is one of the two floats bracketing its exact value, the upper one in a fraction of
// the copies equal to the exact value's position between them (the rule of the twiddle tables).
void dither_consts(DftConsts* k) {
  const double exact[6] = {std::cos(M_PI / 8.0),  std::sin(M_PI / 8.0),  std::sqrt(0.5),
                           std::cos(M_PI / 12.0), std::sin(M_PI / 12.0), std::sqrt(3.0) / 2.0};
  float out[6][kDitherTables];
  for (int c = 0; c < 6; ++c) {
    const float h = static_cast<float>(exact[c]);
    const double l = exact[c] - static_cast<double>(h);
    const float other = std::nextafter(h, l > 0 ? INFINITY : -INFINITY);
    const double frac = l == 0.0 ? 0.0 : l / (static_cast<double>(other) - static_cast<double>(h));
    const int n_other = static_cast<int>(std::lround(frac * kDitherTables));
    const int off = (17 * c + 5) % kDitherTables;
    for (int j = 0; j < kDitherTables; ++j) out[c][j] = ((j + off) % kDitherTables) < n_other ? other : h;
  }
  for (int j = 0; j < kDitherTables; ++j)
    k[j] = DftConsts{out[0][j], out[1][j], out[2][j], out[3][j], out[4][j], out[5][j]};
}

// ======================================================================== extern "C"
extern "C" {

const char* rs_version(void) { return "rs_fresnel 0.1 sm_103a"; }

const char* rs_last_error(void) { return g_err.c_str(); }

int rs_plan_create(int nx, int ny, unsigned flags, rs_plan** out) {
  if (!out) return fail(RS_EINVAL, "out is NULL");
  *out = nullptr;
  if (flags & ~RS_PLAN_FOURSTEP) return fail(RS_EINVAL, "unknown plan flags 0x%x", flags);
  if (nx <= 0 || ny <= 0) return fail(RS_EINVAL, "nx and ny must be positive, got nx=%d, ny=%d", nx, ny);
  // four-step when asked for, and for axes beyond the single-pass transforms (32768)
  const bool four = four_size(nx) && four_size(ny) && ((flags & RS_PLAN_FOURSTEP) || nx > 16384 || ny > 16384);
  if ((flags & RS_PLAN_FOURSTEP) && !four)
    return fail(RS_EUNSUPPORTED, "size %dx%d: four-step plans need power-of-two axes in [4096, 32768]", nx, ny);
  const bool fast = !four && fast_size(nx) && fast_size(ny);
  if (!fast && !four && (nx > kGenericMax || ny > kGenericMax))
    return fail(RS_EUNSUPPORTED, "size %dx%d: axes must be powers of two in [16, 32768] or at most %d",
                nx, ny, kGenericMax);
  rs_plan* p = new rs_plan();
  p->nx = nx;
  p->ny = ny;
  p->fast = fast;
  p->four = four;
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) { delete p; return fail(RS_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e)); }
  // One arena per plan. Fast sizes: compensated stage-major twiddles per axis (float4) and the
  // two-level column table; other sizes: plain twiddles per axis (float2) for the direct DFT.
  // Then ex, ey, ylim, the sample-coordinate tables and the status word.
  const size_t twx = fast ? std::max(stage_twiddle_len(nx), 1) : 0;
  const size_t twy = fast ? std::max(stage_twiddle_len(ny), 1) : 0;
  const size_t tw2y = fast ? static_cast<size_t>(twiddles_2l_len(ny)) : 0;
  const size_t gx = (fast || four) ? 0 : nx, gy = (fast || four) ? 0 : ny;
  const bool split = fast && four_size(ny) && ny <= 16384;  // split columns available
  const bool fy4 = four || split;                              // four-step y tables
  const size_t n1x = four ? nx / kFourN2 : 0, n1y = fy4 ? ny / kFourN2 : 0;
  const size_t f256 = fy4 ? std::max(stage_twiddle_len(kFourN2), 1) : 0;
  const size_t f2l = fy4 ? static_cast<size_t>(twiddles_2l_len(kFourN2)) : 0;
  const size_t f1x = four ? std::max(stage_twiddle_len(static_cast<int>(n1x)), 1) : 0;
  const size_t f1y = fy4 ? std::max(stage_twiddle_len(static_cast<int>(n1y)), 1) : 0;
  size_t bytes = 0;
  auto take = [&](size_t n) { const size_t at = bytes; bytes += (n + 15) & ~static_cast<size_t>(15); return at; };
  const size_t o_twx = take(sizeof(float4) * twx), o_twy = take(sizeof(float4) * twy);
  const size_t o_tw2y = take(sizeof(float4) * tw2y);
  const size_t o_gx = take(sizeof(float2) * gx), o_gy = take(sizeof(float2) * gy);
  const size_t o_ex = take(sizeof(float2) * nx), o_ey = take(sizeof(float2) * ny);
  const size_t o_ylim = take(sizeof(int) * nx), o_xi = take(sizeof(int) * nx), o_xf = take(sizeof(float) * nx);
  const size_t o_yi = take(sizeof(int) * ny), o_yf = take(sizeof(float) * ny), o_xp = take(sizeof(int2) * nx);
  const size_t o_status = take(sizeof(int));
  const size_t o_f256 = take(sizeof(float4) * f256), o_f2l = take(sizeof(float4) * f2l);
  const size_t o_f1x = take(sizeof(float4) * f1x), o_f1y = take(sizeof(float4) * f1y);
  const size_t o_kyi = take(fy4 ? sizeof(int) * ny : 0);
  const size_t o_p4y = take(fy4 ? sizeof(float4) * ny : 0);
  const size_t o_eys = take(split ? sizeof(float2) * ny : 0);
  e = counted_malloc(&p->arena, bytes);
  if (e != cudaSuccess) { delete p; return fail(RS_ENOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e)); }
  {
    void* h = nullptr;
    g_allocs.fetch_add(1, std::memory_order_relaxed);
    e = cudaHostAlloc(&h, sizeof(int), cudaHostAllocDefault);
    if (e != cudaSuccess) {
      cudaFree(p->arena);
      delete p;
      return fail(RS_ENOMEM, "cudaHostAlloc of the status word: %s", cudaGetErrorString(e));
    }
    p->status_host = static_cast<volatile int*>(h);
    *p->status_host = 0;
  }
  char* c = static_cast<char*>(p->arena);
  if (fast) {
    p->tws_x = reinterpret_cast<float4*>(c + o_twx);
    p->tws_y = reinterpret_cast<float4*>(c + o_twy);
    if (tw2y) p->tw2_y = reinterpret_cast<float4*>(c + o_tw2y);
  } else if (!four) {
    p->tw_x = reinterpret_cast<float2*>(c + o_gx);
    p->tw_y = reinterpret_cast<float2*>(c + o_gy);
  }
  if (fy4) {
    p->tw_256 = reinterpret_cast<float4*>(c + o_f256);
    if (f2l) p->tw2_256 = reinterpret_cast<float4*>(c + o_f2l);
    p->tw_c1y = reinterpret_cast<float4*>(c + o_f1y);
    p->tw4y = reinterpret_cast<float4*>(c + o_p4y);
    p->kyi = reinterpret_cast<int*>(c + o_kyi);
  }
  if (four) {
    p->tw_c1x = reinterpret_cast<float4*>(c + o_f1x);
  }
  if (split) {
    p->split_ok = true;
    p->ey_s = reinterpret_cast<float2*>(c + o_eys);
  }
  p->ex = reinterpret_cast<float2*>(c + o_ex);
  p->ey = reinterpret_cast<float2*>(c + o_ey);
  p->ylim = reinterpret_cast<int*>(c + o_ylim);
  p->xi = reinterpret_cast<int*>(c + o_xi);
  p->xf = reinterpret_cast<float*>(c + o_xf);
  p->yi = reinterpret_cast<int*>(c + o_yi);
  p->yf = reinterpret_cast<float*>(c + o_yf);
  p->xp = reinterpret_cast<int2*>(c + o_xp);
  p->status = reinterpret_cast<int*>(c + o_status);
  // RS_PIPELINE: unset -> default; "0" none; "1" both; "rows" / "cols" one direction
  const char* env = std::getenv("RS_PIPELINE");
  p->pipe_rows = kDefaultPipeRows;
  p->pipe_cols = kDefaultPipeCols;
  if (env) {
    const std::string v(env);
    p->pipe_rows = v == "1" || v == "rows";
    p->pipe_cols = v == "1" || v == "cols";
  }
  e = cudaSuccess;
  if (!four) {
    e = fast ? launch_stage_twiddles(nx, p->tws_x, 0) : launch_twiddles(p->tw_x, nx, 0);
    if (e == cudaSuccess) e = fast ? launch_stage_twiddles(ny, p->tws_y, 0) : launch_twiddles(p->tw_y, ny, 0);
    if (e == cudaSuccess && p->tw2_y) e = launch_twiddles_2l(ny, p->tw2_y, 0);
  }
  if (split || four) {
    if (e == cudaSuccess) e = launch_stage_twiddles(kFourN2, p->tw_256, 0);
    if (e == cudaSuccess && p->tw2_256) e = launch_twiddles_2l(kFourN2, p->tw2_256, 0);
    if (e == cudaSuccess) e = launch_stage_twiddles(static_cast<int>(n1y), p->tw_c1y, 0);
    if (e == cudaSuccess) e = launch_power_twiddles(ny, p->tw4y, 0);
  }
  if (four) {
    if (e == cudaSuccess) e = launch_stage_twiddles(static_cast<int>(n1x), p->tw_c1x, 0);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(p->status, 0, sizeof(int), 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    cudaFree(p->arena);
    cudaFreeHost(const_cast<int*>(p->status_host));
    delete p;
    return fail(RS_ECUDA, "twiddle setup: %s", cudaGetErrorString(e));
  }
  // dithered multislice passes: tables derived from the compensated ones (rows of 2^k and 3*2^k,
  // split-pair columns of 2^k from the two-level table, single columns of 3*2^k from the stage table)
  if (fast) {
    int w = 0, bh = 0;
    p->x2_rows = row_x2_ok(nx);
    p->d1_only_rows = !p->x2_rows && row_d1_only(nx);
    p->x2_cols = col_x2_box(ny, &w, &bh) && p->tw2_y != nullptr;
    p->d1_only_cols = !p->x2_cols && col_d1_only(ny);
    p->twd_x_len = p->x2_rows || p->d1_only_rows ? static_cast<int>(twx) : 0;
    p->twd_y2_len = p->x2_cols ? static_cast<int>(tw2y) : p->d1_only_cols ? static_cast<int>(twy) : 0;
    const size_t n = static_cast<size_t>(p->twd_x_len + p->twd_y2_len) * kDitherTables;
    if (n > 0) {
      // the split-pair (wr, wr, wi, wi) tables, then the same entries as (wr, wi)
      e = counted_malloc(&p->twd_arena, n * (sizeof(float4) + sizeof(float2)));
      if (e == cudaSuccess) {
        p->twd_x = static_cast<float4*>(p->twd_arena);
        p->twd_y2 = p->twd_x + static_cast<size_t>(p->twd_x_len) * kDitherTables;
        p->twd1_x = reinterpret_cast<float2*>(p->twd_x + n);
        p->twd1_y2 = p->twd1_x + static_cast<size_t>(p->twd_x_len) * kDitherTables;
        if (p->twd_x_len > 0) e = launch_dither_tables(p->tws_x, p->twd_x, p->twd_x_len, 0);
        if (e == cudaSuccess && p->twd_y2_len > 0)
          e = launch_dither_tables(p->x2_cols ? p->tw2_y : p->tws_y, p->twd_y2, p->twd_y2_len, 0);
        if (e == cudaSuccess) e = launch_single_tables(p->twd_x, p->twd1_x, n, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
      }
      if (e != cudaSuccess) {
        if (p->twd_arena) cudaFree(p->twd_arena);
        cudaFree(p->arena);
        cudaFreeHost(const_cast<int*>(p->status_host));
        delete p;
        return fail(RS_ECUDA, "dithered table setup: %s", cudaGetErrorString(e));
      }
    }
    dither_consts(p->kconst);
  }
  *out = p;
  return RS_OK;
}

int rs_plan_destroy(rs_plan* p) {
  if (!p) return RS_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != p->dev) cudaSetDevice(p->dev);
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  cudaError_t e1 = cudaFree(p->arena);
  cudaError_t e2 = p->det ? cudaFree(p->det) : cudaSuccess;
  if (p->plane && cudaFree(p->plane) != cudaSuccess) e2 = cudaErrorUnknown;
  if (p->status_host && cudaFreeHost(const_cast<int*>(p->status_host)) != cudaSuccess) e2 = cudaErrorUnknown;
  if (p->twd_arena && cudaFree(p->twd_arena) != cudaSuccess) e2 = cudaErrorUnknown;
  if (dev != p->dev) cudaSetDevice(dev);
  delete p;
  if (e1 != cudaSuccess || e2 != cudaSuccess) return fail(RS_ECUDA, "cudaFree failed during plan destroy");
  return RS_OK;
}

int rs_plan_is_fast(const rs_plan* p) { return p && p->fast ? 1 : 0; }

int rs_plan_is_four_step(const rs_plan* p) { return p && p->four ? 1 : 0; }

int rs_plan_set_cancel_flag(rs_plan* p, const volatile int* flag) {
  RS_TRY(check_plan(p));
  p->cancel = flag;
  return RS_OK;
}

int rs_plan_set_pipeline(rs_plan* p, int mask) {
  RS_TRY(check_plan(p));
  p->pipe_rows = (mask & RS_SCHED_PIPE_ROWS) != 0;
  p->pipe_cols = (mask & RS_SCHED_PIPE_COLS) != 0;
  return RS_OK;
}

int rs_plan_set_schedule(rs_plan* p, int mask) {
  RS_TRY(check_plan(p));
  if (mask & ~(RS_SCHED_PIPE_ROWS | RS_SCHED_PIPE_COLS | RS_SCHED_ROW_GENERAL | RS_SCHED_SPLIT_COLS |
               RS_SCHED_COMP_ROWS | RS_SCHED_COMP_COLS | RS_SCHED_SINGLE_ROWS | RS_SCHED_SINGLE_COLS))
    return fail(RS_EINVAL, "unknown schedule bits 0x%x", mask);
  p->x2r_on = (mask & RS_SCHED_COMP_ROWS) == 0;
  p->d1_rows = (mask & RS_SCHED_SINGLE_ROWS) != 0;
  p->d1_cols = (mask & RS_SCHED_SINGLE_COLS) != 0;
  p->x2c_on = (mask & RS_SCHED_COMP_COLS) == 0;
  p->pipe_rows = (mask & RS_SCHED_PIPE_ROWS) != 0;
  p->pipe_cols = (mask & RS_SCHED_PIPE_COLS) != 0;
  p->row_vox = (mask & RS_SCHED_ROW_GENERAL) == 0;
  p->split_cols = (mask & RS_SCHED_SPLIT_COLS) != 0;
  return RS_OK;
}

int rs_plan_get_schedule(const rs_plan* p, int* mask) {
  RS_TRY(check_plan(p));
  if (!mask) return fail(RS_EINVAL, "mask is NULL");
  *mask = (p->pipe_rows ? RS_SCHED_PIPE_ROWS : 0) | (p->pipe_cols ? RS_SCHED_PIPE_COLS : 0) |
          (p->row_vox ? 0 : RS_SCHED_ROW_GENERAL) | (p->split_cols ? RS_SCHED_SPLIT_COLS : 0) |
          (p->x2r_on ? 0 : RS_SCHED_COMP_ROWS) | (p->x2c_on ? 0 : RS_SCHED_COMP_COLS) |
          (p->d1_rows ? RS_SCHED_SINGLE_ROWS : 0) | (p->d1_cols ? RS_SCHED_SINGLE_COLS : 0);
  return RS_OK;
}

int rs_plan_schedules(const rs_plan* p, int* masks, int cap, int* count) {
  RS_TRY(check_plan(p));
  if (!count || (cap > 0 && !masks)) return fail(RS_EINVAL, "count/masks is NULL");
  // Distinct pass schedules for this plan's sizes: a bit whose variant does not exist for the
  // size (no pipelined kernel, or the direct-DFT path of a generic size) would change nothing.
  int w = 0, bh = 0;
  const bool rows_pipe = p->fast && row_pipe_ok(p->nx);
  const bool cols_pipe = p->fast && col_pipe_box(p->ny, &w, &bh);
  int n = 0;
  for (int m = 0; m < 256; ++m) {
    // one row (column) per thread group is a variant of the dithered (split-pair) rows (columns) only
    if ((m & RS_SCHED_SINGLE_ROWS) && ((m & RS_SCHED_COMP_ROWS) || !p->x2_rows)) continue;
    if ((m & RS_SCHED_SINGLE_COLS) && ((m & RS_SCHED_COMP_COLS) || !p->x2_cols)) continue;
    // a direction without split-pair passes has only its single-sequence kernels; where the
    // split-pair passes run, the bits that choose among that direction's other kernels change nothing
    if ((m & RS_SCHED_COMP_ROWS) && !p->x2_rows && !p->d1_only_rows) continue;
    if ((m & RS_SCHED_COMP_COLS) && !p->x2_cols && !p->d1_only_cols) continue;
    if (!(m & RS_SCHED_COMP_ROWS) && (p->x2_rows || p->d1_only_rows) && (m & (RS_SCHED_PIPE_ROWS | RS_SCHED_ROW_GENERAL)))
      continue;
    if (!(m & RS_SCHED_COMP_COLS) && (p->x2_cols || p->d1_only_cols) && (m & (RS_SCHED_PIPE_COLS | RS_SCHED_SPLIT_COLS)))
      continue;
    if ((m & RS_SCHED_SPLIT_COLS) && !p->split_ok) continue;
    if ((m & RS_SCHED_PIPE_ROWS) && !rows_pipe) continue;
    if ((m & RS_SCHED_PIPE_COLS) && !cols_pipe) continue;
    if ((m & RS_SCHED_ROW_GENERAL) && (!p->fast || (m & RS_SCHED_PIPE_ROWS))) continue;
    if (n < cap) masks[n] = m;
    ++n;
  }
  *count = n;
  return RS_OK;
}

int rs_plan_status(rs_plan* p, int* device_status) {
  RS_TRY(check_plan(p));
  if (!device_status) return fail(RS_EINVAL, "device_status is NULL");
  RS_CK(cudaDeviceSynchronize());
  RS_CK(cudaMemcpy(device_status, p->status, sizeof(int), cudaMemcpyDeviceToHost));
  *p->status_host = *device_status;
  if (*device_status != 0) return fail(RS_ETIMEOUT, "a pipelined pass gave up waiting for a bulk copy");
  return RS_OK;
}

int rs_plan_check(const rs_plan* p, int* device_status) {
  if (!p) return fail(RS_EINVAL, "plan is NULL");
  const int st = *p->status_host;
  if (device_status) *device_status = st;
  if (st != 0)
    return fail(RS_ETIMEOUT, "a pipelined pass of this plan gave up waiting for a bulk copy; the field it "
                "wrote is not valid");
  return RS_OK;
}

int rs_plan_clear_status(rs_plan* p, void* stream) {
  RS_TRY(check_plan(p));
  RS_CK(cudaMemsetAsync(p->status, 0, sizeof(int), as_stream(stream)));
  RS_CK(cudaStreamSynchronize(as_stream(stream)));
  *p->status_host = 0;
  return RS_OK;
}

int rs_plan_test_stall(rs_plan* p, int enable) {
  if (!p) return fail(RS_EINVAL, "plan is NULL");
  p->test_stall = enable ? 1 : 0;
  return RS_OK;
}

int rs_detector_table_bytes(int nx, int ny, const rs_detector_geom* g, size_t* bytes) {
  if (!g || !bytes) return fail(RS_EINVAL, "NULL pointer argument");
  if (nx <= 0 || ny <= 0) return fail(RS_EINVAL, "nx and ny must be positive");
  if (g->out_x <= 0 || g->out_y <= 0) return fail(RS_EINVAL, "detector output must be non-empty");
  if (!finite_pos(g->dx) || !finite_pos(g->dy) || !finite_pos(g->ds_px) || !finite_pos(g->ds_py))
    return fail(RS_EINVAL, "detector and grid spacings must be positive");
  if (!std::isfinite(g->detector_z) || g->detector_z == 0.0) return fail(RS_EINVAL, "detector z must be finite and non-zero");
  DetTables t;
  if (g->integrator == 0) build_area_v1(nx, ny, *g, t);
  else if (g->integrator == 1) build_legacy(nx, ny, *g, t);
  else return fail(RS_EINVAL, "unknown integrator %d", g->integrator);
  size_t o[8];
  *bytes = det_layout(t, o);
  return RS_OK;
}

int rs_plan_reserve(rs_plan* p, size_t detector_table_bytes, size_t plasma_plane_voxels) {
  RS_TRY(check_plan(p));
  RS_TRY(grow_det(p, detector_table_bytes));
  RS_TRY(grow_plane(p, plasma_plane_voxels));
  return RS_OK;
}

int rs_alloc_count(unsigned long long* out) {
  if (!out) return fail(RS_EINVAL, "out is NULL");
  *out = g_allocs.load(std::memory_order_relaxed);
  return RS_OK;
}

int rs_launch_count(unsigned long long* out) {
  if (!out) return fail(RS_EINVAL, "out is NULL");
  *out = g_launches.load(std::memory_order_relaxed);
  return RS_OK;
}

int rs_plan_profile(rs_plan* p, int enable) {
  RS_TRY(check_plan(p));
  p->prof = enable != 0;
  p->ev_used = 0;
  p->ev_kind.clear();
  return RS_OK;
}

int rs_plan_profile_read(rs_plan* p, double* row_ms, double* col_ms, int* n_row, int* n_col) {
  RS_TRY(check_plan(p));
  if (!row_ms || !col_ms || !n_row || !n_col) return fail(RS_EINVAL, "NULL output pointer");
  *row_ms = *col_ms = 0.0;
  *n_row = *n_col = 0;
  for (size_t k = 0; k < p->ev_kind.size(); ++k) {
    RS_CK(cudaEventSynchronize(p->ev_pool[2 * k + 1]));
    float ms = 0.f;
    RS_CK(cudaEventElapsedTime(&ms, p->ev_pool[2 * k], p->ev_pool[2 * k + 1]));
    if (p->ev_kind[k] == 0) { *row_ms += ms; ++*n_row; } else { *col_ms += ms; ++*n_col; }
  }
  p->ev_used = 0;
  p->ev_kind.clear();
  return RS_OK;
}

// NumpyVector.fft2 / ifft2 (big-wave/vector.py:341-347).
int rs_fft2(rs_plan* p, const void* in, void* out, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_fft2"));
  if (!in || !out) return fail(RS_EINVAL, "NULL field pointer");
  return fft2_impl(p, static_cast<const float2*>(in), static_cast<float2*>(out), as_stream(stream));
}

int rs_ifft2(rs_plan* p, const void* in, void* out, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_ifft2"));
  if (!in || !out) return fail(RS_EINVAL, "NULL field pointer");
  return ifft2_impl(p, static_cast<const float2*>(in), static_cast<float2*>(out), as_stream(stream));
}

// apply_frequency_cutoff_2d (big-wave/propagation.py:298-326).
int rs_apply_cutoff(rs_plan* p, void* U, double freq, double dx, double dy, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_apply_cutoff"));
  if (!U) return fail(RS_EINVAL, "NULL field pointer");
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_prop(p, dx, dy, 1.0, 0.0, freq, false, s));
  RS_CK(launch_transfer(static_cast<float2*>(U), p->nx, p->ny, p->ex, p->ey, p->ylim, 0, nullptr, s));
  return RS_OK;
}

int rs_apply_transfer(rs_plan* p, void* U, double dx, double dy, double wl, double dz, double cutoff,
                      void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_apply_transfer"));
  if (!U) return fail(RS_EINVAL, "NULL field pointer");
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_prop(p, dx, dy, wl, dz, cutoff, true, s));
  RS_CK(launch_transfer(static_cast<float2*>(U), p->nx, p->ny, p->ex, p->ey, p->ylim, 1, nullptr, s));
  return RS_OK;
}

// propagate_2d (big-wave/propagation.py:396-442).
int rs_propagate(rs_plan* p, void* u_, void* U_, double dx, double dy, double wl, double dz,
                 double cutoff, int skip_fft, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan(p));
  if (!u_ || !U_) return fail(RS_EINVAL, "NULL field pointer");
  float2* u = static_cast<float2*>(u_);
  float2* U = static_cast<float2*>(U_);
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_prop(p, dx, dy, wl, dz, cutoff, true, s));
  if (p->four) return propagate_four(p, u, U, skip_fft != 0, s);
  if (p->fast) {
    const float inv_n = static_cast<float>(1.0 / (static_cast<double>(p->nx) * p->ny));
    if (!skip_fft) {
      RowArgs r{};
      r.in = u; r.out = U; r.ny = p->ny; r.flags = ROW_FWD; r.tw = p->tws_x;
      RS_CK(run_row(p, r, s));
    }
    ColArgs c{};
    c.in = U; c.out = u; c.spec = U; c.nx = p->nx; c.tw = p->tws_y;
    c.ex = p->ex; c.ey = p->ey; c.ylim = p->ylim; c.scale = inv_n;
    c.flags = (skip_fft ? 0 : COL_FWD) | COL_H | COL_SPEC | COL_SCALE | COL_INV;
    RS_CK(run_col(p, c, s));
    RowArgs r{};
    r.in = u; r.out = u; r.ny = p->ny; r.flags = ROW_INV; r.tw = p->tws_x;
    RS_CK(run_row(p, r, s));
  } else {
    if (!skip_fft) RS_TRY(fft2_impl(p, u, U, s));
    RS_CK(launch_transfer(U, p->nx, p->ny, p->ex, p->ey, p->ylim, 1, nullptr, s));
    RS_TRY(ifft2_impl(p, U, u, s));
  }
  return RS_OK;
}

static int point_args(rs_plan* p, double dx, double dy, double xs, double ys, double z, double wl,
                      PointSrcArgs& a) {
  if (!finite_pos(dx) || !finite_pos(dy) || !finite_pos(wl))
    return fail(RS_EINVAL, "dx, dy and wavelength must be positive");
  if (!std::isfinite(z) || !std::isfinite(xs) || !std::isfinite(ys)) return fail(RS_EINVAL, "non-finite source geometry");
  a.dx = dx; a.dy = dy; a.xs = xs; a.ys = ys;
  a.z2 = z * z;
  a.k = (2.0 * M_PI) / wl;  // imaginary part of numpy's 2j*np.pi/wl
  a.half_nx = static_cast<double>(p->nx) / 2.0;
  a.half_ny = static_cast<double>(p->ny) / 2.0;
  return RS_OK;
}

// propagate_analytically_2d (big-wave/propagation.py:458-484).
int rs_point_source(rs_plan* p, void* u, double dx, double dy, double xs, double ys, double z,
                    double wl, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan(p));
  if (!u) return fail(RS_EINVAL, "NULL field pointer");
  PointSrcArgs a{};
  RS_TRY(point_args(p, dx, dy, xs, ys, z, wl, a));
  RS_CK(launch_point_source(static_cast<float2*>(u), p->nx, p->ny, a, as_stream(stream)));
  return RS_OK;
}

static int source_propagate(rs_plan* p, void* u_, void* U_, const PointSrcArgs& a, double dx, double dy,
                            double wl, double cutoff, void* stream);

// PointSource.propagate_to without Fresnel scaling (big-wave/source.py:97-107).
int rs_point_source_propagate(rs_plan* p, void* u_, void* U_, double dx, double dy, double xs,
                              double ys, double z, double wl, double cutoff, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan(p));
  if (!u_ || !U_) return fail(RS_EINVAL, "NULL field pointer");
  PointSrcArgs a{};
  RS_TRY(point_args(p, dx, dy, xs, ys, z, wl, a));
  if (p->four) {
    // the source field, then FFT -> cutoff -> IFFT as a four-step propagation of dz = 0 (its
    // transfer tables are exactly 1); U is left in four-step storage order
    cudaStream_t s = as_stream(stream);
    RS_CK(launch_point_source(static_cast<float2*>(u_), p->nx, p->ny, a, s));
    RS_TRY(build_prop(p, dx, dy, wl, 0.0, cutoff, true, s));
    return propagate_four(p, static_cast<float2*>(u_), static_cast<float2*>(U_), false, s);
  }
  return source_propagate(p, u_, U_, a, dx, dy, wl, cutoff, stream);
}

// Fresnel-scaled source plane (big-wave/source.py:62-95).
int rs_fresnel_plane(rs_plan* p, void* u, double dx, double dy, double xs, double ys, double dz, double wl,
                     void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan(p));
  if (!u) return fail(RS_EINVAL, "NULL field pointer");
  if (!(dz > 0.0) || !std::isfinite(dz)) return fail(RS_EINVAL, "Fresnel source-to-sample distance must be positive");
  PointSrcArgs a{};
  RS_TRY(point_args(p, dx, dy, xs, ys, 0.0, wl, a));
  a.fresnel_plane = 1;
  a.dz = dz;
  RS_CK(launch_point_source(static_cast<float2*>(u), p->nx, p->ny, a, as_stream(stream)));
  return RS_OK;
}

int rs_fresnel_plane_propagate(rs_plan* p, void* u_, void* U_, double dx, double dy, double xs, double ys,
                               double dz, double wl, double cutoff, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_fresnel_plane_propagate"));
  if (!u_ || !U_) return fail(RS_EINVAL, "NULL field pointer");
  if (!(dz > 0.0) || !std::isfinite(dz)) return fail(RS_EINVAL, "Fresnel source-to-sample distance must be positive");
  PointSrcArgs a{};
  RS_TRY(point_args(p, dx, dy, xs, ys, 0.0, wl, a));
  a.fresnel_plane = 1;
  a.dz = dz;
  return source_propagate(p, u_, U_, a, dx, dy, wl, cutoff, stream);
}

static int source_propagate(rs_plan* p, void* u_, void* U_, const PointSrcArgs& a, double dx, double dy,
                            double wl, double cutoff, void* stream) {
  float2* u = static_cast<float2*>(u_);
  float2* U = static_cast<float2*>(U_);
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_prop(p, dx, dy, wl, 0.0, cutoff, false, s));
  if (p->fast) {
    RowArgs r{};
    r.out = U; r.ny = p->ny; r.flags = ROW_SRC | ROW_FWD; r.tw = p->tws_x; r.ps = a;
    RS_CK(run_row(p, r, s));
    ColArgs c{};
    c.in = U; c.out = u; c.spec = U; c.nx = p->nx; c.tw = p->tws_y; c.ylim = p->ylim;
    c.scale = static_cast<float>(1.0 / (static_cast<double>(p->nx) * p->ny));
    c.flags = COL_FWD | COL_MASK | COL_SPEC | COL_SCALE | COL_INV;
    RS_CK(run_col(p, c, s));
    RowArgs r2{};
    r2.in = u; r2.out = u; r2.ny = p->ny; r2.flags = ROW_INV; r2.tw = p->tws_x;
    RS_CK(run_row(p, r2, s));
  } else {
    RS_CK(launch_point_source(u, p->nx, p->ny, a, s));
    RS_TRY(fft2_impl(p, u, U, s));
    RS_CK(launch_transfer(U, p->nx, p->ny, p->ex, p->ey, p->ylim, 0, nullptr, s));
    RS_TRY(ifft2_impl(p, U, u, s));
  }
  return RS_OK;
}

// Sample._apply_2d (big-wave/optical_element.py:502-596).
int rs_multislice_voxel(rs_plan* p, void* u, void* U, const void* grid, int grid_signed, const float* db,
                        int n_db, const rs_voxel_geom* geom, double dx, double dy, double wl,
                        double cutoff, const double* slice_dz, const double* coord_scale,
                        int slice_begin, int slice_end, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_voxel"));
  if (!grid || !db) return fail(RS_EINVAL, "grid and db must be device pointers");
  if (n_db < 1) return fail(RS_EINVAL, "n_db must be >= 1");
  SliceSource src;
  src.grid = static_cast<const char*>(grid);
  src.grid_signed = grid_signed;
  src.db = reinterpret_cast<const float2*>(db);
  src.n_db = n_db;
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

int rs_multislice_voxel_stacked(rs_plan* p, int batch, void* u, void* U, const void* grid, int grid_signed,
                                const float* db, int n_db, const rs_voxel_geom* geom, double dx, double dy,
                                double wl, double cutoff, const double* slice_dz, const double* coord_scale,
                                int slice_begin, int slice_end, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_voxel_stacked"));
  if (!grid || !db) return fail(RS_EINVAL, "grid and db must be device pointers");
  if (n_db < 1) return fail(RS_EINVAL, "n_db must be >= 1");
  SliceSource src;
  src.grid = static_cast<const char*>(grid);
  src.grid_signed = grid_signed;
  src.db = reinterpret_cast<const float2*>(db);
  src.n_db = n_db;
  src.batch = batch;
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

// PlasmaSample._apply_2d (big-wave/plasma_sample.py:126-233).
int rs_multislice_plasma(rs_plan* p, void* u, void* U, const void* ne, const void* ni, const void* te,
                         const void* zstar, int grid_f64, const rs_plasma_consts* pc,
                         const rs_voxel_geom* geom, double dx, double dy, double wl, double cutoff,
                         const double* slice_dz, const double* coord_scale, int slice_begin,
                         int slice_end, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_plasma"));
  if (!ne || !ni || !te || !zstar) return fail(RS_EINVAL, "plasma grids must be device pointers");
  if (!pc || !finite_pos(pc->energy_ev)) return fail(RS_EINVAL, "energy must be positive");
  SliceSource src;
  src.plasma = true;
  src.pg[0] = static_cast<const char*>(ne);
  src.pg[1] = static_cast<const char*>(ni);
  src.pg[2] = static_cast<const char*>(te);
  src.pg[3] = static_cast<const char*>(zstar);
  src.f64 = grid_f64 ? 1 : 0;
  // big-wave/plasma.py:407-433 with densities pre-scaled by 1e-20 inside the kernel
  const double lamb_cm = 1.0e-8 * pc->planck_hc / pc->energy_ev;
  const double pref = pc->r_electron_cm * lamb_cm * lamb_cm / (2.0 * M_PI);
  const double nu = pc->energy_ev / 4.135667e-15;
  PlasmaArgs& b = src.pl_base;
  b.pref20 = static_cast<float>(pref * 1e20);
  b.f1bar = static_cast<float>(pc->f1bar);
  b.f2eff = static_cast<float>(pc->f2eff_bar);
  b.zbar_pos = pc->zbar > 0.0 ? 1 : 0;
  b.inv_zbar = pc->zbar > 0.0 ? static_cast<float>(1.0 / pc->zbar) : 0.0f;
  b.z2bar_pos = pc->z2bar > 0.0 ? 1 : 0;
  b.cff = static_cast<float>(3.7e8 * pc->z2bar / (std::sqrt(11604.5) * nu * nu * nu) * lamb_cm / (4.0 * M_PI) * 1e40);
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

int rs_multislice_dbgrid(rs_plan* p, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                         double dx, double dy, double wl, double cutoff, const double* slice_dz,
                         const double* coord_scale, int slice_begin, int slice_end, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_dbgrid"));
  if (!db_grid) return fail(RS_EINVAL, "db_grid must be a device pointer");
  SliceSource src;
  src.dbv = reinterpret_cast<const float2*>(db_grid);
  src.n_db = 1;
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

int rs_multislice_dbgrid_store(rs_plan* p, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                               double dx, double dy, double wl, double cutoff, const double* slice_dz,
                               const double* coord_scale, int slice_begin, int slice_end, void* fields,
                               void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_dbgrid_store"));
  if (!db_grid || !fields) return fail(RS_EINVAL, "db_grid and fields must be device pointers");
  if (!p->fast) return fail(RS_EUNSUPPORTED, "field storing needs the fused passes (fast sizes)");
  SliceSource src;
  src.dbv = reinterpret_cast<const float2*>(db_grid);
  src.n_db = 1;
  src.store = static_cast<float2*>(fields);
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

int rs_multislice_dbgrid_fields(rs_plan* p, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                                double dx, double dy, double wl, double cutoff, const double* slice_dz,
                                const double* coord_scale, int slice_begin, int slice_end, void* fields,
                                void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_multislice_dbgrid_fields"));
  if (!db_grid || !fields) return fail(RS_EINVAL, "db_grid and fields must be device pointers");
  if (!p->fast) return fail(RS_EUNSUPPORTED, "field storing needs the fused passes (fast sizes)");
  SliceSource src;
  src.dbv = reinterpret_cast<const float2*>(db_grid);
  src.n_db = 1;
  src.store = static_cast<float2*>(fields);
  src.fields_only = true;
  return multislice(p, static_cast<float2*>(u), static_cast<float2*>(U), src, geom, dx, dy, wl, cutoff,
                    slice_dz, coord_scale, slice_begin, slice_end, as_stream(stream));
}

int rs_adjoint_multislice_dbgrid(rs_plan* p, void* g, const float* db_grid, const rs_voxel_geom* geom, double dx,
                                 double dy, double wl, double cutoff, const double* slice_dz,
                                 const double* coord_scale, int slice_begin, int slice_end, const void* fields,
                                 float* grad_grid, void* stream) {
  return rs_adjoint_multislice_dbgrid_ex(p, g, db_grid, geom, dx, dy, wl, cutoff, slice_dz, coord_scale, slice_begin,
                                         slice_end, fields, grad_grid, 0u, stream);
}

int rs_adjoint_multislice_dbgrid_ex(rs_plan* p, void* g, const float* db_grid, const rs_voxel_geom* geom, double dx,
                                    double dy, double wl, double cutoff, const double* slice_dz,
                                    const double* coord_scale, int slice_begin, int slice_end, const void* fields,
                                    float* grad_grid, unsigned gflags, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_adjoint_multislice_dbgrid"));
  if (gflags & ~(RS_ADJ_G_XSPEC_IN | RS_ADJ_G_XSPEC_OUT)) return fail(RS_EINVAL, "unknown flags 0x%x", gflags);
  if (!g || !db_grid || !fields || !grad_grid || !geom || !slice_dz) return fail(RS_EINVAL, "NULL pointer argument");
  if (geom->nz <= 0 || geom->ny_v < 2 || geom->nx_v < 2) return fail(RS_EINVAL, "bad grid shape");
  if (slice_begin < 0 || slice_end > geom->nz || slice_begin > slice_end)
    return fail(RS_EINVAL, "slice range [%d, %d) outside [0, %d]", slice_begin, slice_end, geom->nz);
  if (!finite_pos(wl)) return fail(RS_EINVAL, "wavelength must be positive");
  const bool pow2 = (p->nx & (p->nx - 1)) == 0;
  if (!p->fast || !pow2 || 2 * geom->nx_v > p->nx + p->nx / 16)
    return fail(RS_EUNSUPPORTED, "fused adjoint needs power-of-two rows with nx_v <= (nx + nx/16)/2");
  if (slice_begin == slice_end) return RS_OK;
  cudaStream_t s = as_stream(stream);
  float2* gv = static_cast<float2*>(g);
  const size_t plane = static_cast<size_t>(geom->ny_v) * geom->nx_v;
  const size_t n = static_cast<size_t>(p->nx) * p->ny;
  const float a = static_cast<float>(geom->pixel_size_z / wl);
  const float inv_n = static_cast<float>(1.0 / static_cast<double>(n));
  double cur_dz = NAN, cur_cs = NAN;
  for (int z = slice_end - 1; z >= slice_begin; --z) {
    const double dz = slice_dz[z];
    const double cs = coord_scale ? coord_scale[z] : 1.0;
    if (!(dz == cur_dz)) {
      RS_TRY(build_prop(p, dx, dy, wl, -dz, cutoff, true, s));  // P^H: the step of -dz, same cutoff
      cur_dz = dz;
    }
    if (!(cs == cur_cs)) {
      if (!std::isfinite(cs)) return fail(RS_EINVAL, "coordinate scale of slice %d is not finite", z);
      RS_TRY(build_axes(p, geom, dx, dy, cs, s));
      cur_cs = cs;
    }
    if (z == slice_end - 1 && !(gflags & RS_ADJ_G_XSPEC_IN)) {
      RowArgs r{};
      r.in = gv; r.out = gv; r.ny = p->ny; r.tw = p->tws_x; r.flags = ROW_FWD;
      RS_CK(run_row(p, r, s));
    }
    ColArgs c{};
    c.in = gv; c.out = gv; c.spec = nullptr; c.nx = p->nx; c.tw = p->tws_y;
    c.ex = p->ex; c.ey = p->ey; c.ylim = p->ylim; c.scale = inv_n;
    c.flags = COL_FWD | COL_H | COL_SCALE | COL_INV;
    bool col_x2 = false;
    RS_CK(run_col_ms(p, c, z % kDitherTables, &col_x2, s));
    RowArgs r{};
    r.in = gv; r.out = gv; r.ny = p->ny; r.tw = p->tws_x; r.ax = axis_tab(p);
    r.flags = ROW_INV | (z > slice_begin || (gflags & RS_ADJ_G_XSPEC_OUT) ? ROW_FWD : 0);
    r.vox.dbv = reinterpret_cast<const float2*>(db_grid) + plane * z;
    r.vox.nxv = geom->nx_v;
    r.vox.nyv = geom->ny_v;
    r.vox.n_db = 1;
    r.vox.a = a;
    r.aux = const_cast<float2*>(static_cast<const float2*>(fields)) + static_cast<size_t>(z - slice_begin) * n;
    r.grad = grad_grid + plane * z * 2;
    if (p->x2r_on && (p->x2_rows || p->d1_only_rows)) {
      // dithered tables: slice z's inverse undoes slice z + 1's forward, both with table z + 1
      const int ti = (z + 1) % kDitherTables, tf = z % kDitherTables;
      r.twd1_inv = p->twd1_x + static_cast<size_t>(ti) * p->twd_x_len;
      r.twd1_fwd = p->twd1_x + static_cast<size_t>(tf) * p->twd_x_len;
      r.k_inv = p->kconst[ti];
      r.k_fwd = p->kconst[tf];
      RS_CK(launch_row_adjoint_d1(p->nx, r, s));
    } else {
      RS_CK(launch_row_adjoint(p->nx, r, s));
    }
  }
  return RS_OK;
}

int rs_adjoint_slice(rs_plan* p, void* v, const void* u, const float* db_grid, const rs_voxel_geom* g,
                     double dx, double dy, double wl, int slice, double coord_scale, float* grad_grid,
                     void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_adjoint_slice"));
  if (!v || !u || !db_grid || !grad_grid || !g) return fail(RS_EINVAL, "NULL pointer argument");
  if (slice < 0 || slice >= g->nz) return fail(RS_EINVAL, "slice %d outside [0, %d)", slice, g->nz);
  if (g->ny_v < 2 || g->nx_v < 2) return fail(RS_EINVAL, "bad grid shape");
  if (!finite_pos(wl)) return fail(RS_EINVAL, "wavelength must be positive");
  if (static_cast<size_t>(g->nx_v) * 16 > 200 * 1024) return fail(RS_EUNSUPPORTED, "voxel rows wider than 12800");
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_axes(p, g, dx, dy, coord_scale, s));
  const size_t plane = static_cast<size_t>(g->ny_v) * g->nx_v;
  AdjointSliceArgs a{};
  a.v = static_cast<float2*>(v);
  a.u = static_cast<const float2*>(u);
  a.dbv = reinterpret_cast<const float2*>(db_grid) + plane * slice;
  a.grad = reinterpret_cast<float2*>(grad_grid) + plane * slice;
  a.nx = p->nx;
  a.ny = p->ny;
  a.nxv = g->nx_v;
  a.nyv = g->ny_v;
  a.ax = axis_tab(p);
  a.a = static_cast<float>(g->pixel_size_z / wl);
  RS_CK(launch_adjoint_slice(a, s));
  return RS_OK;
}

int rs_detector_adjoint(rs_plan* p, const void* u, void* g_out, const double* r, const rs_detector_geom* g,
                        void* stream) {
  RS_TRY(check_plan_std(p, "rs_detector_adjoint"));
  if (!u || !g_out || !r || !g) return fail(RS_EINVAL, "NULL pointer argument");
  if (g->out_x <= 0 || g->out_y <= 0) return fail(RS_EINVAL, "detector output must be non-empty");
  if (!finite_pos(g->dx) || !finite_pos(g->dy) || !finite_pos(g->ds_px) || !finite_pos(g->ds_py))
    return fail(RS_EINVAL, "detector and grid spacings must be positive");
  if (!std::isfinite(g->detector_z) || g->detector_z == 0.0) return fail(RS_EINVAL, "detector z must be finite and non-zero");
  DetTables t;
  if (g->integrator == 0) build_area_v1(p->nx, p->ny, *g, t);
  else if (g->integrator == 1) build_legacy(p->nx, p->ny, *g, t);
  else return fail(RS_EINVAL, "unknown integrator %d", g->integrator);
  // invert the per-detector-pixel lists into per-grid-cell lists
  std::vector<int> xptr(p->nx + 1, 0), yptr(p->ny + 1, 0);
  for (int c : t.xcell) ++xptr[c + 1];
  for (int c : t.ycell) ++yptr[c + 1];
  for (int i = 0; i < p->nx; ++i) xptr[i + 1] += xptr[i];
  for (int i = 0; i < p->ny; ++i) yptr[i + 1] += yptr[i];
  std::vector<int> xdet(t.xcell.size()), ydet(t.ycell.size());
  std::vector<float> xw(t.xcell.size());
  std::vector<double> yw(t.ycell.size());
  {
    std::vector<int> fill(xptr.begin(), xptr.end() - 1);
    for (int o = 0; o < g->out_x; ++o)
      for (int k = t.xptr[o]; k < t.xptr[o + 1]; ++k) {
        const int pos = fill[t.xcell[k]]++;
        xdet[pos] = o;
        xw[pos] = t.xw[k];
      }
    std::vector<int> filly(yptr.begin(), yptr.end() - 1);
    for (int o = 0; o < g->out_y; ++o)
      for (int k = t.yptr[o]; k < t.yptr[o + 1]; ++k) {
        const int pos = filly[t.ycell[k]]++;
        ydet[pos] = o;
        yw[pos] = t.yw[k];
      }
  }
  const size_t o_xpos = 0;
  const size_t o_ypos = o_xpos + align8(t.xdet.size() * 8);
  const size_t o_yw = o_ypos + align8(t.ydet.size() * 8);
  const size_t o_xw = o_yw + align8(yw.size() * 8);
  const size_t o_xptr = o_xw + align8(xw.size() * 4);
  const size_t o_xdet = o_xptr + align8(xptr.size() * 4);
  const size_t o_yptr = o_xdet + align8(xdet.size() * 4);
  const size_t o_ydet = o_yptr + align8(yptr.size() * 4);
  const size_t total = o_ydet + align8(ydet.size() * 4) + 8;
  std::vector<char> host(total, 0);
  auto put = [&](size_t off, const void* src, size_t n) { if (n) std::memcpy(host.data() + off, src, n); };
  put(o_xpos, t.xdet.data(), t.xdet.size() * 8);
  put(o_ypos, t.ydet.data(), t.ydet.size() * 8);
  put(o_yw, yw.data(), yw.size() * 8);
  put(o_xw, xw.data(), xw.size() * 4);
  put(o_xptr, xptr.data(), xptr.size() * 4);
  put(o_xdet, xdet.data(), xdet.size() * 4);
  put(o_yptr, yptr.data(), yptr.size() * 4);
  put(o_ydet, ydet.data(), ydet.size() * 4);
  cudaStream_t s = as_stream(stream);
  p->det_cache.valid = false;  // the buffer now holds the transposed tables
  RS_TRY(grow_det(p, total));
  char* d = static_cast<char*>(p->det);
  RS_CK(cudaMemcpyAsync(d, host.data(), total, cudaMemcpyHostToDevice, s));
  DetAdjArgs a{};
  a.u = static_cast<const float2*>(u);
  a.g = static_cast<float2*>(g_out);
  a.r = r;
  a.nx = p->nx;
  a.ny = p->ny;
  a.out_x = g->out_x;
  a.xpos = reinterpret_cast<const double*>(d + o_xpos);
  a.ypos = reinterpret_cast<const double*>(d + o_ypos);
  a.yw = reinterpret_cast<const double*>(d + o_yw);
  a.xw = reinterpret_cast<const float*>(d + o_xw);
  a.xptr = reinterpret_cast<const int*>(d + o_xptr);
  a.xdet = reinterpret_cast<const int*>(d + o_xdet);
  a.yptr = reinterpret_cast<const int*>(d + o_yptr);
  a.ydet = reinterpret_cast<const int*>(d + o_ydet);
  a.z = g->detector_z;
  RS_CK(launch_detector_adjoint(a, s));
  return RS_OK;
}

int rs_apply_transmission_voxel(rs_plan* p, void* u, const void* grid, int grid_signed, const float* db,
                                int n_db, const rs_voxel_geom* g, double dx, double dy, double wl,
                                int slice, double coord_scale, void* stream) {
  StatusNote sn_(p, stream);
  RS_TRY(check_plan_std(p, "rs_apply_transmission_voxel"));
  if (!u || !grid || !db || !g) return fail(RS_EINVAL, "NULL pointer argument");
  if (slice < 0 || slice >= g->nz) return fail(RS_EINVAL, "slice %d outside [0, %d)", slice, g->nz);
  if (g->ny_v < 2 || g->nx_v < 2 || n_db < 1) return fail(RS_EINVAL, "bad grid shape or table");
  if (!finite_pos(wl)) return fail(RS_EINVAL, "wavelength must be positive");
  cudaStream_t s = as_stream(stream);
  RS_TRY(build_axes(p, g, dx, dy, coord_scale, s));
  VoxelArgs vox{};
  vox.slice = static_cast<const char*>(grid) + static_cast<size_t>(g->ny_v) * g->nx_v * slice * 4;
  vox.grid_signed = grid_signed;
  vox.nxv = g->nx_v;
  vox.nyv = g->ny_v;
  vox.db = reinterpret_cast<const float2*>(db);
  vox.n_db = n_db;
  vox.a = static_cast<float>(g->pixel_size_z / wl);
  RS_CK(launch_transmission(static_cast<float2*>(u), p->nx, p->ny, axis_tab(p), &vox, nullptr, s));
  return RS_OK;
}

// square_and_downsample_2d (big-wave/propagation.py:1113-1130).
int rs_detector(rs_plan* p, const void* u, double* out, const rs_detector_geom* g, void* stream) {
  RS_TRY(check_plan(p));
  if (!u || !out || !g) return fail(RS_EINVAL, "NULL pointer argument");
  if (g->out_x <= 0 || g->out_y <= 0) return fail(RS_EINVAL, "detector output must be non-empty");
  if (!finite_pos(g->dx) || !finite_pos(g->dy) || !finite_pos(g->ds_px) || !finite_pos(g->ds_py))
    return fail(RS_EINVAL, "detector and grid spacings must be positive");
  if (!std::isfinite(g->detector_z) || g->detector_z == 0.0) return fail(RS_EINVAL, "detector z must be finite and non-zero");
  if (g->integrator != 0 && g->integrator != 1) return fail(RS_EINVAL, "unknown integrator %d", g->integrator);
  cudaStream_t s = as_stream(stream);
  rs_detector_geom key = *g;
  key.accumulate = 0;  // does not enter the tables
  auto& dc = p->det_cache;
  if (!(dc.valid && std::memcmp(&dc.g, &key, sizeof(key)) == 0)) {
    dc.valid = false;
    DetTables t;
    if (g->integrator == 0) build_area_v1(p->nx, p->ny, *g, t);
    else build_legacy(p->nx, p->ny, *g, t);
    size_t* o = dc.off;
    const size_t total = det_layout(t, o);
    std::vector<char> host(total, 0);
    auto put = [&](size_t off, const void* src, size_t n) { if (n) std::memcpy(host.data() + off, src, n); };
    put(o[0], t.xdet.data(), t.xdet.size() * 8);
    put(o[1], t.ydet.data(), t.ydet.size() * 8);
    put(o[2], t.yw.data(), t.yw.size() * 8);
    put(o[3], t.xw.data(), t.xw.size() * 4);
    put(o[4], t.xptr.data(), t.xptr.size() * 4);
    put(o[5], t.xcell.data(), t.xcell.size() * 4);
    put(o[6], t.yptr.data(), t.yptr.size() * 4);
    put(o[7], t.ycell.data(), t.ycell.size() * 4);
    RS_TRY(grow_det(p, total));
    // Pageable host->device copies are staged before cudaMemcpyAsync returns, so `host` may be
    // released now; the kernel is ordered after the copy on the same stream.
    RS_CK(cudaMemcpyAsync(p->det, host.data(), total, cudaMemcpyHostToDevice, s));
    dc.g = key;
    dc.valid = true;
  }
  const size_t* o = dc.off;
  char* d = static_cast<char*>(p->det);
  DetArgs a{};
  a.u = static_cast<const float2*>(u);
  a.out = out;
  a.nx = p->nx;
  a.out_x = g->out_x;
  a.out_y = g->out_y;
  a.xdet = reinterpret_cast<const double*>(d + o[0]);
  a.ydet = reinterpret_cast<const double*>(d + o[1]);
  a.yw = reinterpret_cast<const double*>(d + o[2]);
  a.xw = reinterpret_cast<const float*>(d + o[3]);
  a.xptr = reinterpret_cast<const int*>(d + o[4]);
  a.xcell = reinterpret_cast<const int*>(d + o[5]);
  a.yptr = reinterpret_cast<const int*>(d + o[6]);
  a.ycell = reinterpret_cast<const int*>(d + o[7]);
  a.z = g->detector_z;
  a.accumulate = g->accumulate;
  RS_CK(launch_detector(a, s));
  return RS_OK;
}

}  // extern "C"

// ===================================================================== no-allocation detector
// rs_detector_noalloc: the detector of rs_detector for callers that must not allocate device
// memory. Its overlap tables live in this fixed device array instead of a plan-owned buffer.
namespace {

constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB: enough for 16384 x 16384 fields
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};
std::mutex g_noalloc_mu;  // guards the look-up; only a successful address is kept

}  // namespace

extern "C" int rs_detector_noalloc(const void* u, int nx, int ny, double* out, const rs_detector_geom* g,
                                   void* stream) {
  if (!u || !out || !g) return fail(RS_EINVAL, "NULL pointer argument");
  if (nx <= 0 || ny <= 0) return fail(RS_EINVAL, "nx and ny must be positive, got nx=%d, ny=%d", nx, ny);
  if (g->out_x <= 0 || g->out_y <= 0) return fail(RS_EINVAL, "detector output must be non-empty");
  if (!finite_pos(g->dx) || !finite_pos(g->dy) || !finite_pos(g->ds_px) || !finite_pos(g->ds_py))
    return fail(RS_EINVAL, "detector and grid spacings must be positive");
  if (!std::isfinite(g->detector_z) || g->detector_z == 0.0) return fail(RS_EINVAL, "detector z must be finite and non-zero");
  int dev = -1;
  RS_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(RS_EUNSUPPORTED, "device ordinal %d above %d", dev, kMaxDevices - 1);
  // Per device, with that device current: the device address of the scratch array (the
  // host-side symbol is only a stand-in and must never reach a kernel). A failed look-up (e.g. one
  // made during a stream capture) is not remembered: the next call tries again.
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr)
        return fail(RS_ECUDA, "cudaGetSymbolAddress of the detector scratch failed: %s", cudaGetErrorString(e));
      g_noalloc_addr[dev] = ptr;
    }
    scratch = g_noalloc_addr[dev];
  }
  DetTables t;
  if (g->integrator == 0) build_area_v1(nx, ny, *g, t);
  else if (g->integrator == 1) build_legacy(nx, ny, *g, t);
  else return fail(RS_EINVAL, "unknown integrator %d", g->integrator);
  const size_t o_xdet = 0;
  const size_t o_ydet = o_xdet + align8(t.xdet.size() * 8);
  const size_t o_yw = o_ydet + align8(t.ydet.size() * 8);
  const size_t o_xw = o_yw + align8(t.yw.size() * 8);
  const size_t o_xptr = o_xw + align8(t.xw.size() * 4);
  const size_t o_xcell = o_xptr + align8(t.xptr.size() * 4);
  const size_t o_yptr = o_xcell + align8(t.xcell.size() * 4);
  const size_t o_ycell = o_yptr + align8(t.yptr.size() * 4);
  const size_t total = o_ycell + align8(t.ycell.size() * 4) + 8;
  if (total > kNoAllocScratchBytes)
    return fail(RS_EINVAL,
                "detector tables need %zu bytes but rs_detector_noalloc has a fixed %zu-byte scratch "
                "(fields up to about 16384 x 16384); use rs_detector for larger fields",
                total, kNoAllocScratchBytes);
  std::vector<char> host(total, 0);
  auto put = [&](size_t off, const void* src, size_t n) { if (n) std::memcpy(host.data() + off, src, n); };
  put(o_xdet, t.xdet.data(), t.xdet.size() * 8);
  put(o_ydet, t.ydet.data(), t.ydet.size() * 8);
  put(o_yw, t.yw.data(), t.yw.size() * 8);
  put(o_xw, t.xw.data(), t.xw.size() * 4);
  put(o_xptr, t.xptr.data(), t.xptr.size() * 4);
  put(o_xcell, t.xcell.data(), t.xcell.size() * 4);
  put(o_yptr, t.yptr.data(), t.yptr.size() * 4);
  put(o_ycell, t.ycell.data(), t.ycell.size() * 4);
  cudaStream_t s = as_stream(stream);
  char* d = static_cast<char*>(scratch);
  // Every entry the kernel reads is rewritten here, so nothing left by an earlier call is used.
  RS_CK(cudaMemcpyAsync(d, host.data(), total, cudaMemcpyHostToDevice, s));
  DetArgs a{};
  a.u = static_cast<const float2*>(u);
  a.out = out;
  a.nx = nx;
  a.out_x = g->out_x;
  a.out_y = g->out_y;
  a.xdet = reinterpret_cast<const double*>(d + o_xdet);
  a.ydet = reinterpret_cast<const double*>(d + o_ydet);
  a.yw = reinterpret_cast<const double*>(d + o_yw);
  a.xw = reinterpret_cast<const float*>(d + o_xw);
  a.xptr = reinterpret_cast<const int*>(d + o_xptr);
  a.xcell = reinterpret_cast<const int*>(d + o_xcell);
  a.yptr = reinterpret_cast<const int*>(d + o_yptr);
  a.ycell = reinterpret_cast<const int*>(d + o_ycell);
  a.z = g->detector_z;
  a.accumulate = g->accumulate;
  RS_CK(launch_detector(a, s));
  return RS_OK;
}
