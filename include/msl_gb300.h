/*
 * msl_gb300.h -- C ABI of the GB300 skeleton library (libmsl_gb300.so).
 *
 * The Muesli reference (NinaHerrmann/muesli4) is a header-only C++ template
 * API with no C ABI; this header is the boundary its skeleton hot path would
 * bind through an FFI. Every entry point names the reference function it
 * replaces (path:line inside the reference project).
 *
 * Conventions
 *  - Every function returns an int status: MSL_OK (0) or a negative MSL_ERR_*.
 *    The reference prints exceptions and continues (src/muesli.cpp:292-294) or
 *    exit()s on CUDA errors (include/muesli.h:70-77); this ABI never exits and
 *    never throws. msl_last_error_string() describes the last failure of the
 *    calling thread.
 *  - Device pointers are plain addresses in the memory of the current device
 *    (msl_alloc, or any cudaMalloc'd buffer). Host pointers are plain host
 *    memory; pinned memory makes the copies faster but is not required.
 *  - All device work is enqueued on the library stream (msl_get_stream /
 *    msl_set_stream). Calls that return a value to the host (folds, residuals)
 *    synchronise that stream; the others return once the work is enqueued.
 *  - Element types: MSL_F32 (float), MSL_F64 (double), MSL_I32 (int32,
 *    two's-complement wrap-around arithmetic), MSL_BF16 (bfloat16 storage,
 *    stencils only).
 *  - Layouts (one partition, the whole container): DA is T[n]; DM is
 *    row-major T[rows][cols] (include/dm.h); DC is T[depth][rows][cols], index
 *    (z*rows + y)*cols + x (include/plcube.h:121-123).
 */
#ifndef MSL_GB300_H
#define MSL_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (names follow include/detail/exception.h) ------------- */
#define MSL_OK 0
#define MSL_ERR_INVALID_ARGUMENT (-1)   /* IllegalArgument / IllegalFunctorException */
#define MSL_ERR_NOT_INITIALIZED (-2)    /* MissingInitializationException */
#define MSL_ERR_CUDA (-3)               /* a CUDA runtime/driver call failed */
#define MSL_ERR_OUT_OF_MEMORY (-4)      /* DeviceOutOfMemory */
#define MSL_ERR_NOT_IMPLEMENTED (-5)    /* NotYetImplementedException */
#define MSL_ERR_SIZE_MISMATCH (-6)      /* SizeMismatch / NotSameSizeException / InvalidCube */
#define MSL_ERR_TIMEOUT (-7)            /* a bounded device-side wait gave up */
#define MSL_ERR_BUDGET (-8)             /* HBM budget of a batch/server exceeded */
#define MSL_ERR_UNSUPPORTED_DEVICE (-9) /* FeatureNotSupportedByDeviceException */
#define MSL_ERR_CANCELLED (-10)         /* a server request cancelled by msl_server_cancel */

/* ---- element types ------------------------------------------------------- */
#define MSL_F32 0
#define MSL_F64 1
#define MSL_I32 2
#define MSL_BF16 3
/* batch storage only (msl_batch_create): FP32 solution with bfloat16-stored
 * corrections, iterated by defect correction */
#define MSL_BF16_DC 4

/* ---- built-in map functors: out = op(x) ---------------------------------- */
#define MSL_MAP_AFFINE 0   /* p[0]*x + p[1]  (two roundings, never fused) */
#define MSL_MAP_ABS 1      /* |x| */
#define MSL_MAP_SQUARE 2   /* x*x */

/* ---- built-in zip functors: out = op(a, b) ------------------------------- */
#define MSL_ZIP_ADD 0      /* a + b */
#define MSL_ZIP_SUB 1      /* a - b */
#define MSL_ZIP_MUL 2      /* a * b */
#define MSL_ZIP_MULADD 3   /* a*b + a (two roundings) */
#define MSL_ZIP_ABSDIFF 4  /* |a - b| */
#define MSL_ZIP_MAX 5      /* a > b ? a : b */
#define MSL_ZIP_MIN 6      /* a < b ? a : b */
/* three-input zip (msl_zip3): out = op(a, b, c) */
#define MSL_ZIP3_MULADD 0  /* a*b + c (two roundings) */
#define MSL_ZIP3_SUM 1     /* (a + b) + c */

/* ---- built-in index functors ----------------------------------------------
 * Coordinates c[] in the reference's argument order: DA (i); DM (row, col);
 * DC (x=col, y=row, z=depth). v is the element of the first input, w of the
 * second (zip_index only).                                                  */
#define MSL_IDX_LINEAR 0   /* p[0]*c0 + p[1]*c1 (+ p[2]*c2) + p[nd]*v (+ p[nd+1]*w), left to right */
#define MSL_IDX_PRODUCT 1  /* c0 * c1 (* c2) * v (* w) */
#define MSL_IDX_XOR_MASK 2 /* v ^ (flat_index & p[0])   (MSL_I32 only) */
#define MSL_IDX_BORDER 3   /* DM/DC: row 0 -> p[0]; other boundary cells -> p[1]; inside -> v */

/* ---- built-in fold functors ---------------------------------------------- */
#define MSL_FOLD_SUM 0
#define MSL_FOLD_MAX 1
#define MSL_FOLD_MIN 2

/* ---- built-in stencil functors --------------------------------------------
 * view(x, y[, z]) is the input at that cell, or `neutral` outside the grid
 * (include/nplmatrix.h:123-139, include/plcube.h:105-119).                 */
#define MSL_ST2_JACOBI5 0  /* boundary cells keep view(x,y); inside: (((0+W)+E)+N)+S, /4 */
#define MSL_ST2_HEAT5 1    /* every cell: (((0+W)+E)+N)+S, /4 (examples/heatdiffusion.cpp:67-76) */
#define MSL_ST2_BOXMEAN 2  /* sum over dx outer, dy inner of view, / (2r+1)^2 */
#define MSL_ST2_BOXSUM 3   /* same sum, not divided */
#define MSL_ST2_LIFE 4     /* Conway's rule, 8 neighbours (examples/gameoflife.cpp:22-42); MSL_I32 */
#define MSL_ST3_HEAT7 0    /* ((((((0+W)+E)+N)+S)+B)+F)/6 (examples/heatdiffusion.cpp:55-65) */
#define MSL_ST3_BOXSUM 1   /* sum over dx, dy, dz (outer to inner) (examples/meanblur2.cpp:46-57) */
#define MSL_ST3_BOXMEAN 2  /* the same sum / (2r+1)^3 (examples/meanblur20.cpp) */

/* ---- runtime ------------------------------------------------------------- */
/* Bind the calling process to `device`, create the library stream and the
 * fold scratch. Replaces msl::initSkeletons (src/muesli.cpp:63-110). */
int msl_init(int device);
/* Release the stream and scratch. Replaces msl::terminateSkeletons (src/muesli.cpp:112-158). */
int msl_terminate(void);
/* Wait for all enqueued work. Replaces msl::syncStreams (src/muesli.cpp:213-223). */
int msl_sync(void);
/* Description of the calling thread's last error ("" if none). */
const char *msl_last_error_string(void);
/* Library stream as a cudaStream_t, and replacing it with a caller's stream
 * (NULL restores the library's own). No reference counterpart: the reference
 * keeps one stream per device in Muesli::streams (include/muesli.h:149-181). */
int msl_get_stream(void **stream);
int msl_set_stream(void *stream);
/* Device facts: SM count, free and total device memory. */
int msl_device_info(int *sm_count, size_t *free_bytes, size_t *total_bytes);
/* Number of kernels this library has launched since msl_init. */
int msl_launch_count(unsigned long long *count);

/* ---- failure detection ----------------------------------------------------
 * Every device-side wait of the library's kernels (on an mbarrier that a TMA
 * copy completes) is bounded: a wait that gives up sets a bit in the
 * context's device error word, lets its own copy land (a second bounded
 * wait) and the CTA returns; the next synchronising call returns
 * MSL_ERR_TIMEOUT and clears the bit, and the context stays usable. None of
 * this has a reference counterpart: the reference exit()s on CUDA errors
 * (include/muesli.h:70-77) and never waits on device-side barriers. */
/* Poll limit of those waits (0 restores the default, about seconds). */
int msl_set_wait_limit(unsigned polls);
/* One CTA waits through the same bounded poll (`polls` polls) on a barrier
 * whose phase completes only if `arrive` is non-zero; returns MSL_OK, or
 * MSL_ERR_TIMEOUT when the wait gave up. Synchronous. */
int msl_wait_selftest(unsigned polls, int arrive);
/* Host-side allocation fault injection: after `after` more allocations by
 * msl_alloc, msl_batch_create or a server's admission, every further one
 * fails with MSL_ERR_OUT_OF_MEMORY (checked before anything else, so it works
 * without a device); a negative value turns the injection off. */
int msl_debug_fail_allocs(long long after);

/* ---- partition storage (DS<T>) ------------------------------------------- */
/* Device partition of a container: DS ctor / initGPUs (src/ds.cpp:215-239). */
int msl_alloc(void **dptr, size_t bytes);
int msl_free(void *dptr);
/* Host -> device: DS::updateDevice (src/ds.cpp:442-462), setLocalPartition (:274-287). */
int msl_upload(void *dst_device, const void *src_host, size_t bytes);
/* Device -> host: DS::updateHost / gather (src/ds.cpp:465-484, 539-591). Synchronous. */
int msl_download(void *dst_host, const void *src_device, size_t bytes);
/* Stream-ordered forms of msl_upload / msl_download: enqueued on `stream` (a
 * cudaStream_t; NULL = the library stream) without waiting, so a transfer can
 * overlap kernels on other buffers. The caller orders them against its other
 * work with events and keeps the host buffer (pinned, for an asynchronous
 * copy) alive until the copy has finished. The reference copies synchronously
 * in updateDevice / updateHost (src/ds.cpp:442-484). */
int msl_upload_async(void *dst_device, const void *src_host, size_t bytes, void *stream);
int msl_download_async(void *dst_host, const void *src_device, size_t bytes, void *stream);
/* Device -> device copy kernel: copyKernel (src/copy_kernel.cu:33-43), gather(DS&) (src/ds.cpp:562-581). */
int msl_copy(void *dst_device, const void *src_device, size_t bytes);
/* DS::fill(const T&) (src/ds.cpp:290-305). */
int msl_fill(int dtype, void *dst, size_t n, double value);

/* ---- element-wise skeletons --------------------------------------------- */
/* out[i] = op(in[i]); in == out is mapInPlace.
 * DS::map / mapInPlace (src/ds.cpp:614-663), mapKernel (src/map_kernels.cu:36-43). */
int msl_map(int dtype, int op, const void *in, void *out, size_t n, const double *params);
/* out[i] = op(a[i], b[i]); a == out is zipInPlace. The argument order is the
 * reference GPU build's (src/zip_kernels.cu:37-43, launched src/ds.cpp:708-709).
 * DS::zip / zipInPlace (src/ds.cpp:669-727). */
int msl_zip(int dtype, int op, const void *a, const void *b, void *out, size_t n);
/* out[i] = op(a[i], b[i], c[i]); DA::zipInPlace3 (src/da.cpp:434-459). */
int msl_zip3(int dtype, int op, const void *a, const void *b, const void *c, void *out, size_t n);
/* Index map: out = op(coords..., in). ndim 1: DA::mapIndex/mapIndexInPlace
 * (src/da.cpp:232-255,328-355); ndim 2 (dims = rows, cols): DM::mapIndex*
 * (src/dm.cpp:372-429); ndim 3 (dims = depth, rows, cols): DC::mapIndex*
 * (src/dc.cpp:387-448). params holds up to 8 values. */
int msl_map_index(int dtype, int op, const void *in, void *out, int ndim, const long long *dims,
                  const double *params);
/* Index zip: out = op(coords..., a, b). DA::zipIndex* (src/da.cpp:375-430),
 * DM::zipIndex* (src/dm.cpp:435-501), DC::zipIndex* (src/dc.cpp:456-550),
 * in the GPU build's argument order. */
int msl_zip_index(int dtype, int op, const void *a, const void *b, void *out, int ndim,
                  const long long *dims, const double *params);

/* ---- folds ---------------------------------------------------------------- */
/* *result (host, one element of dtype) = fold of in[0..n) with op, seeded with
 * elements (no identity), single pass. n == 0 is MSL_ERR_INVALID_ARGUMENT.
 * DS::fold / foldCPU (src/ds.cpp:741-954), foldKernel (src/fold_kernels.cu:51-129). */
int msl_fold(int dtype, int op, const void *in, size_t n, void *result);
/* *result = max_i |a[i] - b[i]| computed in FP64 (a zip + fold(max) fused in
 * one pass; examples/jacobisolver.cpp:127-140 runs them as two skeletons). */
int msl_fold_absdiff_max(int dtype, const void *a, const void *b, size_t n, double *result);

/* Fold that allocates nothing, for callers that cannot allocate device memory
 * (loops that must never pay cudaMalloc's implicit synchronisation, plugins
 * running inside a host whose device memory belongs to that host's own
 * allocator). It needs no msl_init: it runs on the current
 * device and `stream` (a cudaStream_t; NULL is the default stream) and writes
 * one element of dtype to the device pointer result_device; the caller
 * synchronises. Its scratch is a static device array of 2048 CTA partials
 * (about 41 KiB, held by every device that loads the library until exit), so n
 * is limited to 2^30 elements; larger n fails with MSL_ERR_SIZE_MISMATCH
 * before anything is launched. Every call looks up the array's device address
 * in the current context (no allocation). The first call on each device (in
 * each context) also makes the CUDA runtime load this library's device code
 * into that context when lazy module loading is on (the default): that
 * one-time load may allocate device memory and synchronise. Callers that must
 * never pay either make one warm-up call during set-up, before any stream
 * capture, or run with CUDA_MODULE_LOADING=EAGER.
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. dtype MSL_F32, MSL_F64 or MSL_I32; op as msl_fold.
 * No counterpart in the reference (its fold allocates per call, src/ds.cpp:772). */
int msl_fold_noalloc(int dtype, int op, const void *in, size_t n, void *result_device, void *stream);

/* ---- row / column skeletons of a rows x cols row-major matrix (DM) -------- */
/* out[r] = fold of row r with op (MSL_FOLD_*), for every row. The fold order is
 * the reference's row-fold kernel's: L lanes per row (L = threads_per_block when
 * cols >= threads_per_block, else the next power of two >= (cols + 1) / 2);
 * lane t folds row[t], row[t+L], ... left to right, then lane values combine
 * pairwise v[t] = f(v[t], v[t+h]) for h = L/2 ... 1. threads_per_block is the
 * reference's setThreadsPerBlock value: a power of two in [1, 1024].
 * dtype MSL_F32, MSL_F64 or MSL_I32. Replaces DM::reduceRows
 * (src/dm.cpp:1596-1707, kernel src/fold_kernels.cu:215-294). */
int msl_fold_rows(int dtype, int op, const void *in, long long rows, long long cols, int threads_per_block,
                  void *out);
/* out[c] = fold of column c top to bottom (element-seeded, sequential):
 * the column counterpart of msl_fold_rows. */
int msl_fold_cols(int dtype, int op, const void *in, long long rows, long long cols, void *out);
/* out[r][c] = op(m[r][c], v[r]) with a MSL_ZIP_* op: a matrix zipped with a
 * per-row vector (the DM x DA broadcast of DM::zipIndexInPlaceA,
 * src/dm.cpp:1790-1812). out may be m. */
int msl_zip_rows(int dtype, int op, const void *m, const void *v, void *out, long long rows, long long cols);
/* out row k = in row (k - a) mod rows. |a| > rows is MSL_ERR_NOT_IMPLEMENTED,
 * as the reference's RotateRowManyNotImplementedException; out != in.
 * Replaces DM::rotateRows (src/dm.cpp:1345-1475). Any dtype (a raw copy). */
int msl_rotate_rows(int dtype, const void *in, void *out, long long rows, long long cols, long long a);
/* out[r][j] = in[r][(j + a) mod cols]; out != in. Replaces DM::rotateCols
 * (src/dm.cpp:1483-1533). */
int msl_rotate_cols(int dtype, const void *in, void *out, long long rows, long long cols, long long a);
/* dm[r][col] = da[r] for every row; col outside [0, cols) is
 * MSL_ERR_INVALID_ARGUMENT. Replaces DM::setColumn (src/dm.cpp:1856-1879). */
int msl_set_column(int dtype, void *dm, const void *da, long long rows, long long cols, long long col);

/* ---- grid results I/O --------------------------------------------------------- */
/* Append a device grid to a text file in the `;`-separated format of the
 * reference's examples: depth 1 writes one line per row (examples/
 * heatdiffusion.cpp:99-114); depth > 1 writes one line per (x, y) with z
 * innermost (examples/heatdiffusion.cpp:156-170). Values are formatted as
 * std::ostream writes them by default (%g, 6 significant digits; integers in
 * decimal); bfloat16 values as the float they hold. */
int msl_grid_dump_text(const char *path, int dtype, const void *grid, int depth, int rows, int cols);
/* Read such a file back into a device grid (exactly depth*rows*cols values,
 * else MSL_ERR_SIZE_MISMATCH). The text holds 6 significant digits: a dump
 * and load round trip is exact for integers and for values with at most 6. */
int msl_grid_load_text(const char *path, int dtype, void *grid, int depth, int rows, int cols);

/* ---- stencils ------------------------------------------------------------- */
/* Stage stencil windows with TMA tensor copies when the grid allows it (1,
 * the default) or always with plain coalesced loads (0). Results are
 * identical either way; the switch exists to test and compare the loaders.
 * No reference counterpart (the reference has no staging). */
int msl_set_tma(int enabled);
/* 3-D stencils of radius <= 3: 1 = a persistent kernel (two CTAs per SM,
 * each loading its next block with TMA while it computes the current one),
 * 0 = one CTA per 64 x 16 x 8 block, -1 = the library's default (one CTA per
 * block). Results are identical either way. */
int msl_set_stencil3d_persistent(int mode);
/* Sweeps per launch of msl_stencil3d_iterate (and of the server's large
 * cubes) for heat3D (FP32, radius 1, neutral 0) on grids TMA can address:
 * 2 (default) = the z-marching kernel, which keeps the first sweep of each
 * pair in shared memory and halves the HBM traffic per sweep; 1 = one sweep
 * per launch. Results are identical either way. */
int msl_set_stencil3d_depth(int sweeps);
/* z planes each CTA of the z-marching kernel marches through (0, the
 * default: chosen per grid so that the CTAs fill whole waves; else 1..1024).
 * A tuning knob only: results are identical for every value. */
int msl_set_stencil3d_zchunk(int planes);
/* Sweeps fused into one launch by msl_stencil2d_iterate (temporal blocking:
 * the CTA runs depth-1 sweeps on a shared-memory tile with a depth*r halo and
 * writes the last; results are identical to single sweeps). 0 (default) uses
 * the autotuner's choice for the grid, or 1 when none was recorded; at most
 * 32. Applies to Jacobi, heat2D (F32, F64, BF16) and Life. An int32 Life
 * iteration with neutral 0 runs its first generation cell by cell and then
 * `depth` generations per launch on cells packed one bit each (its cells are
 * then all 0 or 1), with identical results. No reference counterpart. */
int msl_set_temporal_depth(int depth);
/* Tile height of the temporal-blocking kernel: 16, 32 or 64 rows of 64
 * columns per CTA (128, 256 or 512 threads), or 0 (default) for the
 * autotuner's record (32 when none). Results do not depend on it. No
 * reference counterpart (the reference's tiles are tile_width x tile_width,
 * include/muesli.h:195). */
int msl_set_tile_rows(int rows);
/* out = f(view, x, y) for every cell of a rows x cols grid; `radius` is the
 * stencil size r, `neutral` the value outside the grid. in != out.
 * DM::mapStencil<f> (src/dm.cpp:1535-1591), NPLMatrix (include/nplmatrix.h:56-168). */
int msl_stencil2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int radius,
                  double neutral);
/* `iters` ping-pong sweeps a -> b -> a ... (examples/heatdiffusion.cpp:93-96).
 * On return *result_in_b says which buffer holds the last sweep; if residual is
 * not NULL it receives max |last - previous| in FP64, fused into the last sweep. */
int msl_stencil2d_iterate(int dtype, int kind, void *a, void *b, int rows, int cols, int radius,
                          double neutral, int iters, double *residual, int *result_in_b);
/* 3-D: out = f(view, x, y, z) over depth x rows x cols.
 * DC::mapStencil<f> (src/dc.cpp:559-592), PLCube (include/plcube.h:55-144). */
int msl_stencil3d(int dtype, int kind, const void *in, void *out, int depth, int rows, int cols,
                  int radius, double neutral);
int msl_stencil3d_iterate(int dtype, int kind, void *a, void *b, int depth, int rows, int cols,
                          int radius, double neutral, int iters, double *residual, int *result_in_b);

/* ---- batched solves -----------------------------------------------------------
 * Many independent plain-Jacobi grids (the MSL_ST2_JACOBI5 functor, radius 1)
 * iterated together until each one's FP64 residual max |last - previous|,
 * taken every `check_every` sweeps, is <= tol (or max_iters sweeps are done).
 * Grids whose two iterates fit in one CTA's shared memory are solved there by
 * one CTA each; the others share a tile work-list advanced by a persistent
 * kernel, `depth` fused sweeps per round, the rounds replayed from a CUDA
 * graph. Each grid's sweeps are exactly those of msl_stencil2d_iterate on that
 * grid alone, so results do not depend on the rest of the batch.
 * storage: MSL_F32, or MSL_BF16 (bfloat16 storage, FP32 arithmetic: the
 * iterates themselves are bfloat16, so a grid stalls once the updates fall
 * below half a bfloat16 ulp of its values), or MSL_BF16_DC (defect
 * correction: the solution u stays FP32; every cycle of check_every sweeps
 * applies the previous correction, u <- u + d, takes the defect
 * r = J(u) - u in FP64 -- its max-norm is the residual checked against tol --
 * and solves d = A d + r, A the Jacobi average of the four neighbours, by
 * check_every - 1 sweeps over bfloat16-stored d and r from d = r; in exact
 * arithmetic u + d equals u after check_every Jacobi sweeps. The cycle
 * (check_every) must be in [2, 64]: the bfloat16 rounding of d accumulates
 * over a cycle.)
 * hbm_budget (bytes, 0 = none): creation fails with MSL_ERR_BUDGET when the
 * batch would need more device memory. No reference counterpart (the
 * reference solves one DM at a time, examples/jacobisolver.cpp:110-145). */
int msl_batch_create(int storage, int count, const int *rows, const int *cols, size_t hbm_budget, void **batch);
/* Set grid `index` from FP32 host values (rounded to bfloat16 for MSL_BF16 storage). */
int msl_batch_set_grid(void *batch, int index, const float *host_grid);
/* Restore every grid to the values last given by msl_batch_set_grid (device
 * copy) and set its sweep count to 0. */
int msl_batch_reset(void *batch);
/* Iterate every grid until its FP64 residual (checked every check_every
 * sweeps) is <= tol or it has done max_iters sweeps in total. A grid continues
 * from its own sweep count (0 after create, set_grid or reset), which must be
 * a multiple of check_every; check_every must divide max_iters; depth 0 =
 * autotuned. */
int msl_batch_solve(void *batch, double tol, long long max_iters, int check_every, int depth);
/* Latest iterate (MSL_BF16_DC: the solution) of grid `index` as FP32, with its
 * sweep count and last residual. */
int msl_batch_get_grid(void *batch, int index, float *host_out, long long *iters, double *residual);
/* Grid count, grids solved CTA-resident, work-list tiles, device bytes (iterates and initial values). */
int msl_batch_info(void *batch, int *count, int *resident, long long *tiles, size_t *device_bytes);
/* Write the batch to a file: every grid's shape, sweep count, residual and
 * done flag, its latest iterate and its initial values. */
int msl_batch_checkpoint(void *batch, const char *path);
/* Create a batch from a checkpoint file (under hbm_budget, 0 = no limit).
 * msl_batch_solve then resumes every grid from its sweep count: with the same
 * tol and check_every the results equal those of one uninterrupted solve. */
int msl_batch_restore(const char *path, size_t hbm_budget, void **batch);
int msl_batch_destroy(void *batch);

/* ---- stencil-solve server ------------------------------------------------------
 * Continuous batching of solve requests: a worker thread admits requests in
 * arrival order while their two iterates fit in hbm_budget (0 = no limit),
 * advances all admitted requests together, check_every sweeps at a time (2-D
 * and 3-D requests on two streams, overlapping), and retires each one when its
 * FP64 residual max |last - previous| is <= tol or after max_iters sweeps
 * (check_every must divide max_iters). A request's sweeps are those of the
 * one-request path (msl_stencil2d_iterate / msl_stencil3d_iterate in chunks of
 * check_every sweeps), so its result does not depend on what else is served.
 * depth = fused sweeps per 2-D launch (0 = autotuned). No reference
 * counterpart. */
#define MSL_SERVE_JACOBI2D 0 /* plain Jacobi (MSL_ST2_JACOBI5) on rows x cols, FP32 */
#define MSL_SERVE_HEAT3D 1   /* heat3D (MSL_ST3_HEAT7), Dirichlet 0, on depth x rows x cols, FP32 */
int msl_server_start(size_t hbm_budget, double tol, long long max_iters, int check_every, int depth, void **server);
/* Queue a request; `init` (FP32 host values) is copied, *request receives its id.
 * A request larger than the whole budget fails with MSL_ERR_BUDGET. */
int msl_server_submit(void *server, int kind, int depth, int rows, int cols, const float *init, long long *request);
/* Block until the request finished (timeout_s < 0: no limit; MSL_ERR_TIMEOUT on
 * expiry). A request cancelled by msl_server_cancel returns MSL_ERR_CANCELLED;
 * one whose iterates could not be allocated at admission fails alone with
 * MSL_ERR_OUT_OF_MEMORY while the others go on. */
int msl_server_wait(void *server, long long request, double timeout_s);
/* Cancel a queued or running request: a queued one leaves the queue at once, a
 * running one is retired (its iterates freed) before the next check interval
 * and produces no result. The other requests' sweeps and results are not
 * affected. A request that has already finished cannot be cancelled
 * (MSL_ERR_INVALID_ARGUMENT). */
int msl_server_cancel(void *server, long long request);
/* Result of a finished request: values (FP32, host), sweeps, last residual,
 * latency (submit to completion) and queueing time (submit to admission). */
int msl_server_result(void *server, long long request, float *out, long long *iters, double *residual,
                      double *latency_s, double *queue_s);
/* Forget a finished, cancelled or out-of-memory request (frees its host copy of the result). */
int msl_server_release(void *server, long long request);
int msl_server_stats(void *server, long long *completed, long long *active, long long *queued, size_t *device_bytes,
                     long long *intervals);
/* Serve what was submitted, then stop the worker and free the device state. */
/* Write every request the server holds to a file -- queued ones with their
 * initial values, running ones with their latest iterate and sweep count
 * (taken between two check intervals), finished ones with their result --
 * together with the server's settings. halt != 0 stops the worker after the
 * write: requests not finished stay unfinished (msl_server_wait reports it)
 * and msl_server_stop then frees the server. */
int msl_server_checkpoint(void *server, const char *path, int halt);
/* Start a server from a checkpoint file: finished requests keep their
 * results, running ones resume from their sweep count ahead of the queued
 * ones, all under their original ids. Each result equals the one the
 * uninterrupted server would have returned. */
int msl_server_restore(const char *path, void **server);
int msl_server_stop(void *server);

/* ---- autotuner -------------------------------------------------------------
 * Times msl_stencil2d_iterate over `iters` sweeps of a rows x cols grid for
 * every launch shape that fits -- temporal depth 1, 2, 3, 4, 6, 8, 12, 16, 24
 * or 32 and, for depths >= 2, tiles of 64 x 16, 64 x 32 or 64 x 64 cells
 * (128, 256 or 512 threads per CTA) -- on scratch grids it allocates and
 * frees, records the fastest for (dtype, kind, radius, grid-size class) and
 * returns it with its rate in cell updates per second. The record is used by
 * later iterate calls when the temporal depth (tile height) setting is 0; the
 * settings themselves are left as the caller had them. No
 * reference counterpart (the reference fixes tile width 16,
 * include/muesli.h:195, and 1024-thread blocks, src/muesli.cpp:103). */
int msl_autotune_stencil2d_shape(int dtype, int kind, int rows, int cols, int radius, int iters, int *best_depth,
                                 int *best_tile_rows, double *best_rate);
/* The same, returning the depth only. */
int msl_autotune_stencil2d(int dtype, int kind, int rows, int cols, int radius, int iters, int *best_depth,
                           double *best_rate);
/* Persist / restore the autotuner's records (plain text, one record per line). */
int msl_autotune_save(const char *path);
int msl_autotune_load(const char *path);

#ifdef __cplusplus
}
#endif
#endif /* MSL_GB300_H */
