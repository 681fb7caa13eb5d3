/* Host BLAS-1 helpers on host arrays, kept for source compatibility with the
 * reference's src/vector.h:4-7 (callers use them to build right-hand sides and
 * check results).  The solver never calls them: its vector work runs in the
 * fused CUDA kernels. */
#ifndef VECTOR_H
#define VECTOR_H

#ifdef __cplusplus
extern "C" {
#endif

void my_daxpy(int n, double alpha, const double *x, double *y); /* y += alpha x */
double my_ddot(int n, const double *x, const double *y);        /* sum x_i y_i in index order */
void my_dscal(int n, double alpha, double *x);                  /* x *= alpha */
void my_dcopy(int n, const double *x, double *y);               /* y = x */

#ifdef __cplusplus
}
#endif
#endif /* VECTOR_H */
