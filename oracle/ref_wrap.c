/* Test infrastructure (oracle build only).
 *
 * Compiles one of the reference's solver sources unmodified, with its
 * compile-time constants turned into run-time values:
 *   EPS      (src/solver.h:13)  -> hbicg_ref_tol
 *   MAX_ITER (src/solver.h:14)  -> hbicg_ref_maxit
 *   SEED_SWITCHING (src/solver.h:31) removed when REF_FIXED_SEED is defined.
 * The Makefile builds this file once per variant with -DREF_SOURCE naming the
 * solver source and -D<entry>=<renamed entry> so the variants can share one
 * library.  solver.h's include guard keeps the overrides below in force when
 * the solver source includes it again.
 */
#include "solver.h"

extern double hbicg_ref_tol;
extern int hbicg_ref_maxit;

#undef EPS
#define EPS hbicg_ref_tol
#undef MAX_ITER
#define MAX_ITER hbicg_ref_maxit
#ifdef REF_FIXED_SEED
#undef SEED_SWITCHING
#endif

#include REF_SOURCE
