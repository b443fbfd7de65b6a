/*
 * rs_fresnel.h — C ABI of the GB300 (sm_103a) multislice Fresnel propagation library.
 *
 * This is the drop-in boundary for big-wave's 2D hot path (RAVE-SIM). Every entry
 * point below replaces one function of big-wave's Python API; the citation after
 * each declaration names the reference function (file:line, paths relative to the
 * RAVE-SIM repository root) whose semantics it reproduces.
 *
 * Conventions
 *  - Fields are complex64 (interleaved float re, im), row-major (ny rows of nx
 *    columns), exactly the memory order of big-wave's NumpyVector
 *    (big-wave/vector.py:319-347: vec.reshape(ny, nx)). All field, grid and
 *    output pointers are DEVICE pointers owned by the caller.
 *  - Scalars (dx, dy, wl, dz, cutoff, ...) are in metres / 1 per metre, FP64, with
 *    the same meaning as the reference arguments.
 *  - Every call is stream-ordered on `stream` (a cudaStream_t passed as void*;
 *    NULL = legacy default stream) and never synchronises the device.
 *  - Every call returns an rs_status; on failure rs_last_error() returns a
 *    thread-local message. Nothing calls exit() (contrast fast-wave's
 *    fwcuda/types.hpp:226-238).
 *  - A plan owns its twiddle/transfer/geometry tables (allocated once in
 *    rs_plan_create). A plan must not be used concurrently from two streams.
 */
#ifndef RS_FRESNEL_H
#define RS_FRESNEL_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rs_status {
  RS_OK = 0,
  RS_EINVAL = 1,      /* bad argument / shape (Python maps to ValueError)        */
  RS_ENOMEM = 2,      /* device allocation failed                                  */
  RS_ECUDA = 3,       /* a CUDA runtime call failed                                */
  RS_EUNSUPPORTED = 4,/* size/dtype outside what this library implements             */
  RS_ETIMEOUT = 5,    /* a bounded device wait gave up                             */
  RS_ECANCELLED = 6   /* host cancel flag observed between slices                  */
} rs_status;

typedef struct rs_plan rs_plan;

/* Library version string, e.g. "rs_fresnel 0.1 sm_103a". */
const char* rs_version(void);

/* Thread-local message describing the last failed call on this host thread. */
const char* rs_last_error(void);

/* Create a plan for fields of nx columns by ny rows on the current CUDA device.
 * Replaces the per-call setup of big-wave/propagation.py:396-442 (fftfreq tables,
 * chunk validation) and fast-wave's FFT<S> plan (fast-wave/src/fft.cpp:6-28).
 * Axes of 2^k in [16, 16384] or 3*2^k in [24, 12288] get the single-pass fused transforms;
 * other axes up to 6144 the direct DFT. Axes of 32768 (both axes powers of two in
 * [4096, 32768]) get a four-step plan: each axis transform runs as a length-n/256 transform
 * with the W_n twiddle fused, then a length-256 transform, and the spectrum is kept in
 * four-step storage order (entry i of an axis holds frequency i/256 + (n/256)*(i%256)).
 * A four-step plan serves rs_propagate (U is left in that order; skip_fft expects it),
 * rs_point_source, rs_point_source_propagate and rs_detector; the other entry points return
 * RS_EUNSUPPORTED.
 * flags: 0, or RS_PLAN_FOURSTEP to ask for a four-step plan at 4096..16384 as well. */
#define RS_PLAN_FOURSTEP 1u
int rs_plan_create(int nx, int ny, unsigned flags, rs_plan** out);
int rs_plan_destroy(rs_plan* plan);
/* 1 when both axes use the fused Stockham kernels, 0 when the generic DFT path is used. */
int rs_plan_is_fast(const rs_plan* plan);
/* 1 if the plan is a four-step plan (see rs_plan_create), else 0. */
int rs_plan_is_four_step(const rs_plan* plan);

/* Unnormalised forward 2D DFT, out may equal in.
 * Replaces NumpyVector.fft2 = scipy.fft.fft2 (big-wave/vector.py:341-343). */
int rs_fft2(rs_plan* plan, const void* in, void* out, void* stream);

/* Inverse 2D DFT with 1/(nx*ny) normalisation, out may equal in.
 * Replaces NumpyVector.ifft2 = scipy.fft.ifft2 (big-wave/vector.py:345-347). */
int rs_ifft2(rs_plan* plan, const void* in, void* out, void* stream);

/* Zero spectrum bins with kx^2+ky^2 > 2*freq^2 (kx = fftfreq(nx)/dx, FP64 test).
 * Replaces apply_frequency_cutoff_2d (big-wave/propagation.py:298-326). */
int rs_apply_cutoff(rs_plan* plan, void* U, double freq, double dx, double dy,
                    void* stream);

/* One Fresnel step: u <- IFFT2[mask * exp(2 pi i dz/wl) * exp(-i pi wl dz (kx^2+ky^2)) * FFT2[u]];
 * afterwards U holds the spectrum of the new u. skip_fft != 0 means U already holds
 * FFT2(u) and the forward transform is skipped.
 * Replaces propagate_2d (big-wave/propagation.py:396-442). */
int rs_propagate(rs_plan* plan, void* u, void* U, double dx, double dy, double wl,
                 double dz, double cutoff, int skip_fft, void* stream);

/* Spherical wave u = exp(2 pi i r/wl)/r from a point source at (xs, ys) a distance z
 * upstream; x = (ix - nx/2)*dx - xs. The phase is reduced in FP64 (carrier split).
 * Replaces propagate_analytically_2d (big-wave/propagation.py:458-484). */
int rs_point_source(rs_plan* plan, void* u, double dx, double dy, double xs,
                    double ys, double z, double wl, void* stream);

/* PointSource.propagate_to in 2D without Fresnel scaling: analytic init, FFT2, circular
 * cutoff, IFFT2; U is left holding the cut-off spectrum.
 * Replaces big-wave/source.py:97-107 (after grid_density_check_2d, done by the caller). */
int rs_point_source_propagate(rs_plan* plan, void* u, void* U, double dx, double dy,
                              double xs, double ys, double z, double wl, double cutoff,
                              void* stream);

/* Fresnel-scaled source plane u = exp(-2 pi i (x xs + y ys)/(wl dz)) / dz, x = (ix - nx/2) dx (FP64
 * phase reduced to cycles), and the same followed by FFT2, circular cutoff and IFFT2 (U left
 * holding the cut-off spectrum). Replace the Fresnel-scaling branch of PointSource.propagate_to
 * (big-wave/source.py:62-95), after its geometry checks. */
int rs_fresnel_plane(rs_plan* plan, void* u, double dx, double dy, double xs, double ys, double dz,
                     double wl, void* stream);
int rs_fresnel_plane_propagate(rs_plan* plan, void* u, void* U, double dx, double dy, double xs,
                               double ys, double dz, double wl, double cutoff, void* stream);

/* Geometry of a voxel Sample (big-wave/optical_element.py:383-412, 502-546). */
typedef struct rs_voxel_geom {
  int nz, ny_v, nx_v;        /* grid shape (z, y, x)                                   */
  double pixel_size_x;       /* voxel pitch x [m]                                       */
  double pixel_size_y;       /* voxel pitch y [m] (already resolved: 0 -> pixel_size_x) */
  double pixel_size_z;       /* slice thickness [m] (material_factor thickness)        */
  double x_pos, y_pos;       /* phase-stepping offsets for this iteration [m]          */
} rs_voxel_geom;

/* Fused multislice through a voxel Sample, slices [slice_begin, slice_end):
 * per slice u *= material_factor(bilinear(db[grid[z]]), pixel_size_z, wl), then one
 * Fresnel step of slice_dz[s] with circular cutoff. grid is uint32/int32 material ids
 * (device), db is (n_db) x (delta, beta) float32 pairs (device, index 0 = vacuum).
 * slice_dz (host, nz entries) are the effective step lengths; coord_scale (host, nz
 * entries, or NULL for all 1.0) are the transverse coordinate scales of each slice.
 * u_spectral != 0 is not supported (u is spatial on entry). Afterwards u is spatial and
 * U holds FFT2(u).
 * Replaces Sample._apply_2d (big-wave/optical_element.py:502-596) together with
 * material_factor (39-42) and the propagate_2d call per slice (585-592). */
int rs_multislice_voxel(rs_plan* plan, void* u, void* U, const void* grid, int grid_signed,
                        const float* db, int n_db, const rs_voxel_geom* geom,
                        double dx, double dy, double wl, double cutoff,
                        const double* slice_dz, const double* coord_scale,
                        int slice_begin, int slice_end, void* stream);

/* rs_multislice_voxel over `batch` fields stacked in u and U (field k at u + k*nx*ny) that share
 * the plan's size, the wavelength, the sample and its placement, and differ only in their
 * content (e.g. the point sources of one energy in a multisim batch): each launch processes
 * all of them, so small fields fill the GPU. The column passes run the per-block kernel
 * batched over the fields; each field's result equals a separate rs_multislice_voxel call on it
 * bit for bit unless the plan's schedule splits its columns. No reference counterpart
 * (big-wave runs one source per process). */
int rs_multislice_voxel_stacked(rs_plan* plan, int batch, void* u, void* U, const void* grid, int grid_signed,
                                const float* db, int n_db, const rs_voxel_geom* geom,
                                double dx, double dy, double wl, double cutoff,
                                const double* slice_dz, const double* coord_scale,
                                int slice_begin, int slice_end, void* stream);

/* Plasma model scalars per energy (big-wave/plasma_sample.py:68-83, plasma.py:241-266).
 * planck_hc [eV*Angstrom] and r_electron_cm [cm] are the CODATA values the caller's
 * nist_lookup uses (nist_lookup/nist_lookup/physical_constants.py: PLANCK_HC, R_ELECTRON_CM). */
typedef struct rs_plasma_consts {
  double f1bar, f2eff_bar, zbar, z2bar;
  double energy_ev;
  double planck_hc, r_electron_cm;
} rs_plasma_consts;

/* Fused multislice through a PlasmaSample: per voxel corner, delta/beta come from
 * (n_e, n_i, T_e, Z*) grids (float64 or float32, device; grid_f64 selects) by the
 * free-electron + bound-electron + Kramers model, then bilinear interpolation, zero
 * outside the grid, material_factor, Fresnel step.
 * Replaces PlasmaSample._apply_2d (big-wave/plasma_sample.py:126-233) and
 * plasma_delta_beta_grid_multi (big-wave/plasma.py:380-434). */
int rs_multislice_plasma(rs_plan* plan, void* u, void* U, const void* ne, const void* ni,
                         const void* te, const void* zstar, int grid_f64,
                         const rs_plasma_consts* pc, const rs_voxel_geom* geom,
                         double dx, double dy, double wl, double cutoff,
                         const double* slice_dz, const double* coord_scale,
                         int slice_begin, int slice_end, void* stream);

/* Multislice through a voxel volume of (delta, beta) float32 pairs per voxel (device,
 * (nz, ny_v, nx_v, 2)) instead of material ids + table: the same interpolation, transmission
 * and Fresnel step as rs_multislice_voxel (big-wave/optical_element.py:502-596 with a per-voxel
 * delta+i*beta). This is the forward model of the adjoint below. */
int rs_multislice_dbgrid(rs_plan* plan, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                         double dx, double dy, double wl, double cutoff, const double* slice_dz,
                         const double* coord_scale, int slice_begin, int slice_end, void* stream);

/* rs_multislice_dbgrid that also writes the field entering each slice z of [slice_begin,
 * slice_end) to fields + (z - slice_begin) * nx * ny (complex64, device): the recomputation
 * step of a checkpointed adjoint. Fast sizes only (RS_EUNSUPPORTED otherwise). */
int rs_multislice_dbgrid_store(rs_plan* plan, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                               double dx, double dy, double wl, double cutoff, const double* slice_dz,
                               const double* coord_scale, int slice_begin, int slice_end, void* fields,
                               void* stream);

/* The fields of rs_multislice_dbgrid_store alone: the same slices and the same field written for
 * each, but the work after the last field's store (its transmission, its Fresnel step and the
 * return of u to real space) is skipped, so u and U are left unspecified. The recomputation step
 * of a checkpointed adjoint, which only reads the fields. No counterpart in the reference. */
int rs_multislice_dbgrid_fields(rs_plan* plan, void* u, void* U, const float* db_grid, const rs_voxel_geom* geom,
                                double dx, double dy, double wl, double cutoff, const double* slice_dz,
                                const double* coord_scale, int slice_begin, int slice_end, void* fields,
                                void* stream);

/* Backward sweep of rs_multislice_dbgrid over slices [slice_begin, slice_end) in two fused passes
 * per slice. On entry g = dL/dconj(u_end), the gradient with respect to the field leaving
 * slice_end - 1; on exit g = dL/dconj(u_begin). fields holds the fields entering each slice as
 * written by rs_multislice_dbgrid_store; dL/d(delta, beta) of every slice's voxels is added to
 * grad_grid (same layout as db_grid). Needs power-of-two rows and nx_v <= (nx + nx/16)/2
 * (RS_EUNSUPPORTED otherwise; rs_adjoint_slice covers the rest). No counterpart in the reference
 * (big-wave has no gradients). */
int rs_adjoint_multislice_dbgrid(rs_plan* plan, void* g, const float* db_grid, const rs_voxel_geom* geom, double dx,
                                 double dy, double wl, double cutoff, const double* slice_dz,
                                 const double* coord_scale, int slice_begin, int slice_end, const void* fields,
                                 float* grad_grid, void* stream);
/* The same sweep with g kept transformed along x between segments of a checkpointed backward:
 * RS_ADJ_G_XSPEC_IN, g arrives as row spectra (the previous segment's output, not real space);
 * RS_ADJ_G_XSPEC_OUT, g is left as row spectra for the next segment instead of being returned to
 * real space. A backward over segments passes OUT on every segment but the last and IN on every
 * segment but the first, which saves one row transform pair per segment boundary. */
#define RS_ADJ_G_XSPEC_IN 1u
#define RS_ADJ_G_XSPEC_OUT 2u
int rs_adjoint_multislice_dbgrid_ex(rs_plan* plan, void* g, const float* db_grid, const rs_voxel_geom* geom,
                                    double dx, double dy, double wl, double cutoff, const double* slice_dz,
                                    const double* coord_scale, int slice_begin, int slice_end, const void* fields,
                                    float* grad_grid, unsigned flags, void* stream);

/* Adjoint of one slice u' = P (t * u) of rs_multislice_dbgrid. On entry v holds P^H g' (g' =
 * dL/dconj(u'), P^H = a Fresnel step of -dz with the same cutoff); u is the field that entered
 * the slice. Accumulates dL/d(delta, beta) of the slice's voxels into grad_grid (float32 pairs,
 * same layout as db_grid) and leaves v = conj(t) * v = dL/dconj(u). No counterpart in the
 * reference (big-wave has no gradients). */
int rs_adjoint_slice(rs_plan* plan, void* v, const void* u, const float* db_grid, const rs_voxel_geom* geom,
                     double dx, double dy, double wl, int slice, double coord_scale, float* grad_grid,
                     void* stream);

/* Detector geometry (big-wave/propagation.py:766-815 _detector_geometry). */
typedef struct rs_detector_geom {
  double dx, dy;             /* grid spacings [m]                                      */
  double ds_px, ds_py;       /* effective detector pixel sizes [m]                     */
  double detector_z;         /* effective distance for the obliquity cosine [m]        */
  int out_x, out_y;          /* detector shape (columns, rows)                          */
  int integrator;            /* 0 = area_v1, 1 = legacy_fastwave                        */
  int accumulate;            /* 1: out += image (incoherent sum), 0: out = image        */
} rs_detector_geom;

/* |u|^2 integrated over detector pixels times the obliquity cosine; out is float64
 * (out_y x out_x, device). area_v1 = separable exact overlap areas; legacy_fastwave =
 * truncated index ranges. Replaces square_and_downsample_2d
 * (big-wave/propagation.py:1113-1130) -> _area_v1_stream (995-1110) and
 * _legacy_fastwave_stream (836-946). */
int rs_detector(rs_plan* plan, const void* u, double* out, const rs_detector_geom* g,
                void* stream);

/* Cancellation of the multislice loops (rs_multislice_voxel, _stacked, _plasma, _dbgrid and its
 * store / fields forms): with a flag set, each loop reads *flag (host memory, written by any host
 * thread) before it enqueues a slice's passes and, when it is non-zero, returns RS_ECANCELLED
 * (Python: InterruptedError) without enqueueing more. The passes already enqueued still run; the
 * field is then part-way through the element and not a result. NULL (the default) turns the
 * check off. Reference counterpart: the cancel tokens big-wave's long-running steps poll on the
 * host (big-wave/propagation.py:669-680, checkpoint.py:22-30). */
int rs_plan_set_cancel_flag(rs_plan* plan, const volatile int* flag);

/* Pass variants: bulk-copy staged, persistent versions of the fused passes. mask bit 0 selects
 * them for the row passes, bit 1 for the column passes (default: columns only). RS_PIPELINE in
 * the environment ("0", "1", "rows", "cols") overrides the default at plan creation. */
int rs_plan_set_pipeline(rs_plan* plan, int mask);

/* Pass schedule of a plan (the autotuner's choices; every variant computes the same transform):
 *   RS_SCHED_PIPE_ROWS   row passes as the persistent bulk-copy pipeline (tiles of rows staged
 *                        through shared memory by a producer warp);
 *   RS_SCHED_PIPE_COLS   column passes as the persistent tensor-copy pipeline (strips of columns
 *                        loaded by TMA boxes, NB buffers) instead of one block per strip;
 *   RS_SCHED_ROW_GENERAL the multislice rows run the general row kernel instead of the
 *                        voxel-only specialisation;
 *   RS_SCHED_SPLIT_COLS  (ny = n1*256 in [4096, 16384]) the column pass of a multislice step runs
 *                        as three shorter passes: length-n1 transforms with the W_ny twiddle,
 *                        length-256 transform / H / inverse, length-n1 inverse. Rounding differs
 *                        from the single pass at the FP32 level (the other bits reproduce it
 *                        exactly).
 * rs_plan_schedules lists the masks that are distinct for the plan's sizes (it writes at most
 * `cap` of them and the total to *count). Where the split-pair passes run (no
 * RS_SCHED_COMPENSATED), the bits that pick among the single-sequence kernels of that direction
 * are not listed. No reference function: big-wave has one FFT schedule. */
#define RS_SCHED_PIPE_ROWS 1
#define RS_SCHED_PIPE_COLS 2
#define RS_SCHED_ROW_GENERAL 4
#define RS_SCHED_SPLIT_COLS 8
/*   RS_SCHED_COMP_ROWS,  the multislice row (resp. column) passes run the single-sequence kernels
 *   RS_SCHED_COMP_COLS   with compensated (float + residual) twiddles, as every other entry point
 *                        does, instead of the split-pair passes: two rows (or two columns) per
 *                        thread group in packed f32x2 arithmetic with 64 dithered twiddle tables,
 *                        slice k using table k mod 64 (their rounding errors average out over
 *                        slices instead of adding up). Both keep the FP64-vs-FP32 intensity error of
 *                        a 514-slice run within 2e-5; their results differ at the FP32 rounding level. */
#define RS_SCHED_COMP_ROWS 16
#define RS_SCHED_COMP_COLS 32
#define RS_SCHED_COMPENSATED (RS_SCHED_COMP_ROWS | RS_SCHED_COMP_COLS)
/*   RS_SCHED_SINGLE_ROWS (without RS_SCHED_COMP_ROWS) the dithered row passes hold one row per
 *                        thread group instead of two, in the single-sequence form of the same
 *                        arithmetic: the same results (up to the sign of zero) with half the
 *                        registers per thread. Rows of 16384 (a row pair does not fit shared
 *                        memory) and rows of 3*2^k in [384, 6144] (a radix-24 first stage) have
 *                        only this form, so there the bit changes nothing. */
#define RS_SCHED_SINGLE_ROWS 64
/*   RS_SCHED_SINGLE_COLS (without RS_SCHED_COMP_COLS) the same for the dithered column passes:
 *                        one column per thread group (the strips of the pipelined single-sequence
 *                        column pass), the split-pair columns' results. Columns of 3*2^k in
 *                        [384, 6144] have only this form, so there the bit changes nothing. */
#define RS_SCHED_SINGLE_COLS 128
int rs_plan_set_schedule(rs_plan* plan, int mask);
int rs_plan_get_schedule(const rs_plan* plan, int* mask);
int rs_plan_schedules(const rs_plan* plan, int* masks, int cap, int* count);
/* Synchronises the device and returns the plan's device status word: 0, or non-zero (with
 * RS_ETIMEOUT) if a pipelined pass gave up waiting for a bulk copy. */
int rs_plan_status(rs_plan* plan, int* device_status);
/* The same answer without a device synchronisation: every call that ran a pipelined pass queues
 * a 4-byte copy of the status word into pinned host memory on its stream, so once the caller has
 * synchronised that stream (as it does to read a detector image) this reads the word as of its
 * last call. Returns RS_ETIMEOUT when it is set: the field that pass wrote is not valid. A status
 * stays set until rs_plan_clear_status (which synchronises `stream`). No reference counterpart:
 * big-wave's NumPy path has no device waits. */
int rs_plan_check(const rs_plan* plan, int* device_status);
int rs_plan_clear_status(rs_plan* plan, void* stream);
/* Test hook: the next pipelined column pass of the plan waits (with a short bound, about 2^14
 * polls) on a barrier that nothing completes, records the timeout in the status word and returns
 * without touching the field, as a pass whose bulk copy never landed would. One-shot. */
int rs_plan_test_stall(rs_plan* plan, int enable);

/* Buffers that grow with the geometry: the detector tables of rs_detector and the plasma slice
 * plane of rs_multislice_plasma. Growing one mid-run frees and reallocates device memory (and
 * so synchronises the device); a caller that knows its run reserves both first.
 * rs_detector_table_bytes gives the table bytes rs_detector needs for a geometry (host only);
 * rs_plan_reserve grows the buffers to at least the given sizes now. rs_alloc_count returns the
 * number of device and pinned-host allocations this library has made in the process (plans,
 * tables, status words), so a caller can check that a run allocated nothing.
 * Reference counterpart: none (big-wave allocates NumPy arrays per call). */
int rs_detector_table_bytes(int nx, int ny, const rs_detector_geom* geom, size_t* bytes);
int rs_plan_reserve(rs_plan* plan, size_t detector_table_bytes, size_t plasma_plane_voxels);
int rs_alloc_count(unsigned long long* out);

/* Tracing (counterpart of fast-wave's CudaTimerSection, fast-wave/src/simulation.cpp:14-33):
 * total number of kernels this library has launched in the process ... */
int rs_launch_count(unsigned long long* out);
/* ... and optional CUDA-event timing of every row / column pass of the multislice loops.
 * rs_plan_profile(plan, 1) starts recording (clearing earlier records); rs_plan_profile_read
 * waits for the recorded passes and returns their summed milliseconds and counts, then clears. */
int rs_plan_profile(rs_plan* plan, int enable);
int rs_plan_profile_read(rs_plan* plan, double* row_ms, double* col_ms, int* n_row, int* n_col);

/* Adjoint of rs_detector: given r = dL/dI (float64, out_y x out_x, device) and the field u,
 * writes g = dL/dconj(u) = (D^T r) * u, D the detector integration (area_v1 or legacy). */
int rs_detector_adjoint(rs_plan* plan, const void* u, void* g, const double* r, const rs_detector_geom* geom,
                        void* stream);

/* The detector of rs_detector for callers that must not allocate device memory: code that
 * runs where the device memory is owned by someone else (a framework's caching pool, a
 * fixed memory budget) or that cannot afford rs_detector's cudaMalloc/cudaFree, which grows
 * its table buffer and synchronises the whole device when it does. This entry point needs no
 * plan and allocates nothing: its overlap tables (built on the host, copied with one
 * cudaMemcpyAsync) live in a fixed 4 MiB device array compiled into the library, which is
 * enough for fields up to about 16384 x 16384; larger requests fail with RS_EINVAL. u is the
 * (ny, nx) complex64 field, out the float64 (out_y, out_x) image, both device pointers owned
 * by the caller. The first call on a device looks up that array's device address (with the
 * caller's device current); make it before any stream capture. All calls share the one
 * array, so two calls whose work overlaps on the GPU (other streams, other host threads)
 * race; serialise them. Every table entry is rewritten on each call.
 * No counterpart in the reference: big-wave allocates its detector output on the host
 * (propagation.py:700-733). */
int rs_detector_noalloc(const void* u, int nx, int ny, double* out, const rs_detector_geom* g,
                        void* stream);

/* Plain (unfused) forms used as the in-repo comparator: T multiply, H multiply. */
int rs_apply_transmission_voxel(rs_plan* plan, void* u, const void* grid, int grid_signed,
                                const float* db, int n_db, const rs_voxel_geom* geom,
                                double dx, double dy, double wl, int slice, double coord_scale,
                                void* stream);
int rs_apply_transfer(rs_plan* plan, void* U, double dx, double dy, double wl, double dz,
                      double cutoff, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RS_FRESNEL_H */
