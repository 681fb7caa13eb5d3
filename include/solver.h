/* Shifted BiCGStab with seed switching on one GB300 — drop-in for the
 * reference's src/solver.h:33-35.
 *
 * Solves (A + sigma_j I) x_j = b for j = 0..sigma_len-1 with one Krylov process
 * on the seed system and scalar recurrences for the others; when the seed
 * converges, the unconverged shift with the largest residual factor
 * |1/(zeta_j pi_j)| becomes the new seed.
 *
 * Contract (as the reference's, src/solver_dynamic.c:3-463):
 *   A_loc_diag   the matrix (CSR, square); A_loc_offd must be empty or is added
 *   A_info       rows/cols/nz of the matrix; a non-square matrix prints
 *                "Error: matrix is not square." and exits(1), like the reference
 *   x_loc_set    sigma_len * rows doubles, shift-major, zero on entry; the
 *                solutions on exit
 *   r_loc        b on entry; the final residual of the seed system on exit
 *   sigma        sigma_len shifts; seed = index of the first seed
 *   returns      k = iterations + 1 on convergence, MAX_ITER + 1 at the limit;
 *                a negative value if the GPU reported an error
 * All pointers are host pointers.  The three entry points compute the same
 * results; they differ in how the GPU runs the iteration:
 *   _static   one kernel per step of the reference's iteration, scalars and the
 *             switch decision on the host (the per-kernel form)
 *   _dynamic  fused kernels, scalars, convergence test and seed switch on the
 *             device, the iteration captured in CUDA graphs
 *   _normal   fused kernels launched one by one, no graph
 * EPS and MAX_ITER are the reference's defaults (src/solver.h:13-14);
 * hbicg_dropin_config() changes them at run time.
 */
#ifndef SOLVER_H
#define SOLVER_H

#include <math.h>
#include <stdbool.h>
#include <time.h>

#include "matrix.h"
#include "vector.h"

#define EPS 1.0e-12
#define MAX_ITER 2000
#define SEED_SWITCHING

#ifdef __cplusplus
extern "C" {
#endif

int shifted_lopbicg_dynamic(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                            double *r_loc, double *sigma, int sigma_len, int seed);
int shifted_lopbicg_static(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed);
int shifted_lopbicg_normal(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed);

/* Run-time replacement of EPS / MAX_ITER / SEED_SWITCHING for the three entry
 * points above (the reference fixes them at compile time). */
void hbicg_dropin_config(double tol, int max_iter, int switching);

#ifdef __cplusplus
}
#endif
#endif /* SOLVER_H */
