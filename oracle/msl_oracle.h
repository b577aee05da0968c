/*
 * CPU oracle for the skeleton hot path -- TEST INFRASTRUCTURE, not product code.
 *
 * A plain C++/OpenMP restatement of the Muesli reference's OpenMP (CPU) build
 * of DA/DM/DC map, zip, index map/zip, fold and DM/DC mapStencil, with the
 * built-in functors of include/msl_gb300.h. Only tests, the smoke check and
 * the CPU-baseline leg of the benchmark load it (liboracle.so, via ctypes);
 * the product library never does.
 *
 * Parity is pinned: tests/golden/ holds outputs of the reference itself
 * (oracle/_ref/ref_harness, built from the reference sources by oracle/Makefile)
 * and tests/test_oracle_golden.py checks this restatement against them.
 *
 * Every entry point takes host pointers and returns 0 or a negative
 * MSL_ERR_* code. Floating-point expressions are evaluated one IEEE operation
 * at a time in the functor's source order (compiled with -ffp-contract=off).
 */
#ifndef MSL_ORACLE_H
#define MSL_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

int oracle_set_threads(int n);  /* OpenMP threads for map/zip/stencil loops; returns the count in use */
int oracle_map(int dtype, int op, const void *in, void *out, size_t n, const double *params);
int oracle_zip(int dtype, int op, const void *a, const void *b, void *out, size_t n);
int oracle_zip3(int dtype, int op, const void *a, const void *b, const void *c, void *out, size_t n);
int oracle_map_index(int dtype, int op, const void *in, void *out, int ndim, const long long *dims,
                     const double *params);
int oracle_zip_index(int dtype, int op, const void *a, const void *b, void *out, int ndim,
                     const long long *dims, const double *params);
int oracle_fold(int dtype, int op, const void *in, size_t n, void *result);
int oracle_fold_absdiff_max(int dtype, const void *a, const void *b, size_t n, double *result);
int oracle_stencil2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int radius,
                     double neutral);
int oracle_stencil2d_iterate(int dtype, int kind, void *a, void *b, int rows, int cols, int radius,
                             double neutral, int iters, double *residual, int *result_in_b);
int oracle_stencil3d(int dtype, int kind, const void *in, void *out, int depth, int rows, int cols,
                     int radius, double neutral);
int oracle_stencil3d_iterate(int dtype, int kind, void *a, void *b, int depth, int rows, int cols,
                             int radius, double neutral, int iters, double *residual, int *result_in_b);
/* Plain Jacobi by defect correction with bfloat16-stored correction and
 * defect (the GPU batch's MSL_BF16_DC mode): u (FP32, in place) is the
 * solution; returns the sweeps done and the FP64 residual max |J(u) - u|. */
int oracle_jacobi_defect_bf16(float *u, int rows, int cols, double tol, long long max_iters, int cycle,
                              long long *iters, double *residual);
/* DM row / column skeletons: reduceRows (GPU row-fold order), column folds,
 * matrix x per-row-vector zips, rotateRows, rotateCols, setColumn. */
int oracle_fold_rows(int dtype, int op, const void *in, long long rows, long long cols, int threads_per_block,
                     void *out);
int oracle_fold_cols(int dtype, int op, const void *in, long long rows, long long cols, void *out);
int oracle_zip_rows(int dtype, int op, const void *m, const void *v, void *out, long long rows, long long cols);
int oracle_rotate_rows(int dtype, const void *in, void *out, long long rows, long long cols, long long a);
int oracle_rotate_cols(int dtype, const void *in, void *out, long long rows, long long cols, long long a);
int oracle_set_column(int dtype, void *dm, const void *da, long long rows, long long cols, long long col);
/* Text dump of a grid in the examples' `;`-separated format (appends). */
int oracle_dump_text(const char *path, int dtype, const void *grid, int depth, int rows, int cols);

#ifdef __cplusplus
}
#endif
#endif
