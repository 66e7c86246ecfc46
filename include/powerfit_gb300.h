/*
 * powerfit_gb300 — C ABI of the GB300 (sm_103a) exhaustive 6D local
 * cross-correlation search.
 *
 * Every entry point takes plain pointers and sizes (no framework types),
 * returns 0 on success and a negative PF_E* code on failure; a failing call
 * never aborts the process.  The message of the last failure is available
 * from pf_last_error() (per context) or pf_global_error() (calls without a
 * context).  Arrays are C-order (z, y, x), host memory unless the name says
 * otherwise.
 *
 * Reference interfaces replaced (file:line in haddocking/powerfit v3.0.2):
 *   correlator object  src/powerfit_em/powerfitter.py:166-393 (BaseCorrelator,
 *                      CPUCorrelator) and :396-555 (GPUCorrelator)
 *   native helpers     src/powerfit_em/_extensions.c:7-196 (rotate_grid3d),
 *                      src/powerfit_em/_powerfit.pyx:45-72 (conj_multiply,
 *                      calc_lcc)
 *   shard merge        src/powerfit_em/powerfitter.py:146-163 (_combine)
 */
#ifndef POWERFIT_GB300_H
#define POWERFIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF_OK 0
#define PF_E_ARG (-1)       /* bad argument (shape, size, pointer, order of calls) */
#define PF_E_CUDA (-2)      /* CUDA runtime error */
#define PF_E_NOMEM (-3)     /* device allocation failed */
#define PF_E_STATE (-4)     /* target / template / rotations not set */
#define PF_E_SHAPE (-5)     /* grid size not supported (prime factor > 7, plane too large) */
#define PF_E_UNSUPPORTED (-6) /* not available in this variant of the library */

/* pf_scan flags */
#define PF_FLAG_FP64_NORM 1   /* local variance and LCC in float64 (default: float-float) */
#define PF_FLAG_NO_PRUNE 2    /* do not skip rotated rows known to be zero */
#define PF_FLAG_ACCUMULATE 4  /* keep the running best of earlier scans (do not reset) */
#define PF_FLAG_GENERIC 8     /* use the runtime-planned kernels even where a specialised path exists */
#define PF_FLAG_ROT_MAX 16    /* also keep, per rotation, the best LCC over the lcc-mask voxels (pf_get_rotation_max) */
#define PF_FLAG_TENSOR_DFT 32 /* precision study: the DFT stages of the search on the tensor cores in split-bf16x3
                                 (mma.sync bf16, float32 accumulation; runtime-planned kernels, edges <= 256) */
#define PF_FLAG_TENSOR_TC05 64 /* with PF_FLAG_TENSOR_DFT: the plane pass's DFT stages with tcgen05.mma (operands
                                  in shared memory, accumulators in tensor memory) instead of mma.sync; planes that
                                  fit one block with the operand area (PF_E_ARG otherwise) */

typedef struct pf_ctx pf_ctx;

/* --- correlator context: one per (grid shape, device); replaces the
 *     constructor of CPUCorrelator/GPUCorrelator (powerfitter.py:262-277,
 *     :399-424) ------------------------------------------------------------ */
pf_ctx *pf_create(int nz, int ny, int nx, int device, int *status);
int pf_destroy(pf_ctx *ctx);
int pf_last_error(const pf_ctx *ctx, char *buf, size_t len);
int pf_global_error(char *buf, size_t len);

/* Target, already normalised by its maximum and Laplace-filtered if the
 * search uses the Laplace pre-filter (powerfitter.py:268-277), and the lcc
 * mask (target > 0.05 max of the unfiltered target, powerfitter.py:178-180).
 * Computes FT(target) and FT(target^2) on the device. */
int pf_set_target(pf_ctx *ctx, const double *target, const uint8_t *lcc_mask);

/* Template after the mask setter's preprocessing (Laplace, mask, normalise,
 * mask again: powerfitter.py:190-220), the mask, the number of mask voxels
 * (norm_factor, :199) and the rotation radius rmax (min(shape)//2, :176). */
int pf_set_template_mask(pf_ctx *ctx, const double *tmpl, const double *mask, double norm_factor, int rmax);

/* One-shot scan of nrot row-major 3x3 rotation matrices (powerfitter.py:
 * 317-333): per voxel the best LCC (strict >, initial 0, lowest index wins
 * ties) and the index of the rotation that gave it, plus rot_offset.
 * out_lcc/out_rot: nz*ny*nx float32 / int32 (GPUCorrelator.lcc/.rot types). */
int pf_scan(pf_ctx *ctx, const double *rotmats, int64_t nrot, int64_t rot_offset,
            float *out_lcc, int32_t *out_rot, int flags);

/* Resident variant (inputs and outputs stay in device memory):
 * upload a rotation set once, scan slices of it, read the results. */
int pf_set_rotations(pf_ctx *ctx, const double *rotmats, int64_t nrot);
int pf_reset_results(pf_ctx *ctx);
int pf_scan_resident(pf_ctx *ctx, int64_t first, int64_t count, int64_t rot_offset, int flags);
int pf_get_results(pf_ctx *ctx, float *out_lcc, int32_t *out_rot);
/* Checkpoint / resume: load a running best saved with pf_get_results (lcc,
 * rot of nz*ny*nx voxels); a later pf_scan_resident with PF_FLAG_ACCUMULATE
 * over the remaining rotations continues the search as if never stopped
 * (the partial maxima merge with _combine semantics, powerfitter.py:146-163). */
int pf_set_results(pf_ctx *ctx, const float *lcc, const int32_t *rot);
/* After scans with PF_FLAG_ROT_MAX: for rotations first .. first+count-1 of
 * the uploaded set, the best LCC over the voxels inside the lcc mask (-inf
 * for a rotation not scanned since its range was last reset).  The per-rotation
 * score the learned proposal trains on and ranks by; the reference keeps only
 * the per-voxel best (powerfitter.py:317-333). */
int pf_get_rotation_max(pf_ctx *ctx, float *out, int64_t first, int64_t count);
/* The same maxima and, per rotation, the voxel (C-order index) holding it
 * (-1 where none); either output may be NULL.  Of equal maxima, the higher
 * voxel index is reported. */
int pf_get_rotation_best(pf_ctx *ctx, float *value, int32_t *voxel, int64_t first, int64_t count);
int pf_synchronize(pf_ctx *ctx);
/* Launch on the caller's cudaStream_t (NULL: back to the context's own
 * non-blocking stream -- so the legacy default stream cannot be selected;
 * pass a created stream); lets a host framework order the search with its
 * own work and time it with events on that stream. */
int pf_set_stream(pf_ctx *ctx, void *stream);

/* Tuning: rotation pairs per batch, rows per tile of passes 1 and 3
 * (0 keeps the current value). */
int pf_set_tuning(pf_ctx *ctx, int pairs_per_batch, int rows_pass1, int rows_pass3);
int pf_get_tuning(const pf_ctx *ctx, int *pairs_per_batch, int *rows_pass1, int *rows_pass3);
/* Autotuner: times short scans (trial_rotations of the uploaded set) over
 * candidate batch and tile sizes and keeps the fastest; resets the results.
 * No reference counterpart (the reference has no tunables). */
int pf_autotune(pf_ctx *ctx, int64_t trial_rotations, int *pairs_per_batch, int *rows_pass1,
                int *rows_pass3, double *best_ms);
/* Radius beyond which rotated data is zero (pruning), planes kept, rmax. */
int pf_get_geometry(const pf_ctx *ctx, int *reff, int *valid_planes, int *rmax);

/* Kernel timing (CUDA events around every launch while enabled):
 * accumulated milliseconds and launch counts of pass 1, 2, 3. */
int pf_set_profiling(pf_ctx *ctx, int enable);
int pf_get_kernel_times(pf_ctx *ctx, double *ms, int64_t *launches);

/* Diagnostic: forward 3D FFT of a real grid through the library's own
 * transforms; out = (nz, ny, nx) complex64 interleaved in natural order.
 * No reference counterpart (the reference calls FFTW / clFFT). */
int pf_fft3d(pf_ctx *ctx, const float *in, float *out);

/* Scan that allocates no device memory, for callers that cannot allocate
 * while they run: a host that gives all device memory to its own allocator
 * at start-up and forbids later cudaMalloc, or a plugin that may only use
 * the buffers its host hands it.  No counterpart in the reference.
 *
 * All pointers are device pointers the caller owns: target (already
 * normalised and filtered, N float32), lcc mask (N uint8), template and mask
 * (N float32 each, after the mask setter's preprocessing), rotations (nrot x 9
 * float64, row-major); outputs lcc (N float32) and rot (N int32), zeroed by
 * the call.  Results equal pf_scan's for the same inputs within float32
 * rounding.  The target spectra, one rotation pair's intermediate spectra,
 * the twiddle tables (built on the device by the call) and the converted
 * rotations live in one file-scope device array of about 10.1 MiB (grids up
 * to 64^3 voxels, edges <= 256, (z, y) plane within shared memory); larger
 * grids return PF_E_SHAPE.  Every GPU that loads the library holds that array
 * until the process exits.
 *
 * The first call on each device does a one-time set-up with that device
 * current: it looks up the array's device address (cudaGetSymbolAddress) and
 * sets the kernels' shared-memory limits.  Make that first call before any
 * stream capture.  Every call queues its work on `stream` and returns
 * without waiting for it.  All calls share the one array and it keeps the
 * last call's contents (each call rebuilds what it reads): calls that overlap
 * on the GPU (different streams, or a second call before the first has
 * finished on another stream) race and corrupt each other's results. */
int pf_scan_noalloc(int nz, int ny, int nx, const float *d_target, const uint8_t *d_lcc_mask,
                    const float *d_template, const float *d_mask, double norm_factor, int rmax,
                    const double *d_rotmats, int64_t nrot, int64_t rot_offset,
                    float *d_lcc, int32_t *d_rot, void *stream);

/* --- unit-level mirrors of the reference's native helpers (run on the
 *     current CUDA device) -------------------------------------------------- */
/* _extensions.c:7-196: out[p] = grid(R^T p) for |p| <= radius, periodic wrap;
 * trilinear (nearest == 0) or nearest; voxels outside the sphere untouched. */
int pf_rotate_grid3d(const double *grid, int nz, int ny, int nx, const double *rotmat,
                     int radius, double *out, int nearest);
/* _powerfit.pyx:45-53: out = conj(in1) * in2, n complex128 (interleaved). */
int pf_conj_multiply(const double *in1, const double *in2, double *out, int64_t n);
/* _powerfit.pyx:56-72: lcc = gcc / sqrt(ave2 - ave^2) where mask != 0. */
int pf_calc_lcc(const double *gcc, const double *ave, const double *ave2, const uint8_t *mask,
                double *lcc, int64_t n);
/* powerfitter.py:146-163: merge one rotation shard into (lcc, rot):
 * where part_lcc > lcc: lcc = part_lcc, rot = part_rot + rot_add. */
int pf_combine(float *lcc, int32_t *rot, const float *part_lcc, const int32_t *part_rot,
               int64_t n, int64_t rot_add);

/* --- preprocessing on the GPU (run once per search; host arrays) -------- */
/* _powerfit.pyx:75-140 (blur_points): out += w exp(-d^2 / 2 sigma^2) within
 * 4 sigma of each point; points are (3, n) rows x, y, z in voxel units; with
 * wraparound negative indices wrap once (as the reference's Cython indexing). */
int pf_blur_points(const double *points, const double *weights, int64_t n, double sigma, double *out,
                   int nz, int ny, int nx, int wraparound);
/* _powerfit.pyx:143-206 (dilate_points): out = 1 within radii[i] of each point. */
int pf_dilate_points(const double *points, const double *radii, int64_t n, double *out,
                     int nz, int ny, int nx, int wraparound);
/* powerfitter.py:212-215: scipy.ndimage.laplace(in, mode='wrap'). */
int pf_laplace_wrap(const double *in, double *out, int nz, int ny, int nx);
/* helpers.py:26-34 (determine_core_indices): number of 6-connected binary
 * erosions (border 0) each voxel of mask > 0 survives, counting itself. */
int pf_core_indices(const double *mask, double *out, int nz, int ny, int nx);
/* message of the last failing preprocessing call */
int pf_prep_error(char *buf, size_t len);

/* --- learned rotation proposal (device pointers; no reference counterpart) --
 * The scoring network y = w3 . relu(W2 relu(W1 x + b1) + b2) + b3 with nin
 * inputs and nh hidden units (16, 32 or 64), bfloat16 weights and float32
 * accumulation.  Parameters are one flat vector [W1 (nh*nin), b1 (nh),
 * W2 (nh*nh), b2 (nh), w3 (nh), b3 (1)]: pf_mlp_param_count entries, float32
 * master copy and bfloat16 copy.  x is row-major (n, nin) float32.  stream:
 * a cudaStream_t, or NULL for the legacy default stream. */
int64_t pf_mlp_param_count(int nin, int nh);
int pf_mlp_forward(const float *x, int64_t n, int nin, int nh, const void *params_bf16, float *y, void *stream);
/* Adds the gradient of L = sum_i c_i (y_i - t_i)^2, c_i = scale * w_i (w
 * may be NULL: w_i = 1), into grad (param_count floats) and L into *loss. */
int pf_mlp_grad(const float *x, const float *t, const float *w, int64_t n, int nin, int nh,
                const void *params_bf16, float scale, float *grad, float *loss, void *stream);
/* One Adam step (bias-corrected, step >= 1) on the float32 master
 * parameters; rewrites the bfloat16 copy. */
int pf_mlp_adam(float *params, void *params_bf16, const float *grad, float *m, float *v, int64_t count,
                float lr, float beta1, float beta2, float eps, int step, void *stream);
/* message of the last failing pf_mlp_* call */
int pf_mlp_error(char *buf, size_t len);

/* --- error-path testing --------------------------------------------------
 * Make the after-th device allocation of the library from now on (0: the
 * next) fail as if the device were out of memory, once; -1 turns it off.
 * The failing call returns PF_E_NOMEM and leaves no partial state behind. */
int pf_debug_fail_alloc(int64_t after);

/* --- bounds-checked build ------------------------------------------------
 * Built with -DPF_BOUNDS_CHECK (libpowerfit_gb300_checked.so), the search
 * kernels check every index into global, shared and distributed shared
 * memory against the extent of its array; an index outside is recorded and
 * the access skipped (a load reads zero, a store does nothing), never
 * trapped.  The other build returns PF_E_UNSUPPORTED from these calls.
 *
 * 1 when this library was built with bounds checks, else 0. */
int pf_bounds_checked(void);
/* Waits for the device, then returns the violations recorded on it since the
 * last call and clears them: *count violations, *first the code of one of
 * them ((site << 48) | (index & (2^48 - 1)); 0 when none).  Sites: 1 twiddle
 * table, 2 shared-memory array, 3 template/mask gather, 4 pass-1 row list,
 * 5 spectra store, 6 spectra load, 7 target spectrum, 8 output spectra,
 * 9 cluster push, 10 voxel array, 11 pass-3 voxel list, 12 per-rotation
 * maximum. */
int pf_debug_bounds(int device, uint64_t *first, uint64_t *count);
/* Tell the kernels of this context that the intermediate spectra buffer
 * holds only `elements` complex values (less than allocated; -1: all), so
 * that the accesses beyond -- still inside the allocation -- show up as
 * violations (a test of the checks themselves). */
int pf_debug_buffer_extent(pf_ctx *ctx, int64_t elements);

#ifdef __cplusplus
}
#endif
#endif /* POWERFIT_GB300_H */
