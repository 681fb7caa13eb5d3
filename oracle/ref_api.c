/* Test infrastructure (oracle build only).
 *
 * Flat C entry points over the reference's own solver, built single-rank
 * through shim/mpi.h, so that tests can call it through ctypes with plain
 * arrays.  The matrix is passed as one CSR block; the off-diagonal block of
 * the reference's row-block split is empty on one rank (src/matrix.c:336-340).
 *
 * Seed tracking: the reference gathers the seed's search vector at start-up
 * (src/solver_dynamic.c:115), after every iteration and after a switch
 * (:230,:352), and gathers the residual once per iteration (:177).  The hook
 * counts the residual gathers as iterations and maps every other gathered
 * pointer back to a shift index through the first gather, which is
 * &p_loc_set[seed * n].
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "solver.h"

double hbicg_ref_tol = 1.0e-12;
int hbicg_ref_maxit = 2000;
void (*hbicg_shim_gather_hook)(const void *sendbuf, int count) = 0;

int ref_dynamic(CSR_Matrix *, CSR_Matrix *, INFO_Matrix *, double *, double *, double *, int, int);
int ref_static(CSR_Matrix *, CSR_Matrix *, INFO_Matrix *, double *, double *, double *, int, int);
int ref_normal(CSR_Matrix *, CSR_Matrix *, INFO_Matrix *, double *, double *, double *, int, int);
int ref_dynamic_fixed(CSR_Matrix *, CSR_Matrix *, INFO_Matrix *, double *, double *, double *, int, int);

static struct {
    const double *r_ptr;
    const double *p_base;
    long n;
    int cur, iters;
    int *log_k, *log_seed, cap, count;
} g_track;

static void track_hook(const void *sendbuf, int count) {
    const double *s = (const double *)sendbuf;
    (void)count;
    if (s == g_track.r_ptr) {
        g_track.iters++;
        return;
    }
    if (!g_track.p_base) {
        g_track.p_base = s - (long)g_track.cur * g_track.n;
        return;
    }
    long off = s - g_track.p_base;
    int idx = (int)(off / g_track.n);
    if (idx != g_track.cur) {
        if (g_track.count < g_track.cap) {
            g_track.log_k[g_track.count] = g_track.iters;
            g_track.log_seed[g_track.count] = idx;
        }
        g_track.count++;
        g_track.cur = idx;
    }
}

/* variant: 0 dynamic, 1 static, 2 normal, 3 dynamic with switching compiled out.
 * x: m*n zero on entry; r: b on entry, final seed residual on exit.
 * Returns the reference's k; *n_log = number of seed switches seen. */
int ref_solve(int variant, unsigned n, const unsigned *ptr, const unsigned *col, const double *val, double *x,
              double *r, const double *sigma, int m, int seed, double tol, int maxit, int *log_k, int *log_seed,
              int log_cap, int *n_log) {
    CSR_Matrix diag, offd;
    INFO_Matrix info;
    int recv = (int)n, displ = 0;
    diag.val = (double *)val;
    diag.col = (unsigned *)col;
    diag.ptr = (unsigned *)ptr;
    diag.nz = ptr[n];
    diag.rows = diag.cols = n;
    offd.val = NULL;
    offd.col = NULL;
    offd.ptr = (unsigned *)calloc((size_t)n + 1, sizeof(unsigned));
    offd.nz = 0;
    offd.rows = offd.cols = n;
    info.nz = diag.nz;
    info.rows = info.cols = n;
    memcpy(info.code, "MCRG", 4);
    info.recvcounts = &recv;
    info.displs = &displ;

    hbicg_ref_tol = tol;
    hbicg_ref_maxit = maxit;
    memset(&g_track, 0, sizeof g_track);
    g_track.r_ptr = r;
    g_track.n = n;
    g_track.cur = seed;
    g_track.log_k = log_k;
    g_track.log_seed = log_seed;
    g_track.cap = log_cap;
    hbicg_shim_gather_hook = track_hook;

    int k;
    double *sig = (double *)sigma;
    switch (variant) {
    case 1: k = ref_static(&diag, &offd, &info, x, r, sig, m, seed); break;
    case 2: k = ref_normal(&diag, &offd, &info, x, r, sig, m, seed); break;
    case 3: k = ref_dynamic_fixed(&diag, &offd, &info, x, r, sig, m, seed); break;
    default: k = ref_dynamic(&diag, &offd, &info, x, r, sig, m, seed); break;
    }
    hbicg_shim_gather_hook = 0;
    free(offd.ptr);
    if (n_log) *n_log = g_track.count;
    return k;
}

/* y = A x through the reference's own serial CSR product (src/matrix.c:498). */
void ref_mult(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x, double *y) {
    CSR_Matrix a;
    a.val = (double *)val;
    a.col = (unsigned *)col;
    a.ptr = (unsigned *)ptr;
    a.nz = ptr[n];
    a.rows = a.cols = n;
    memset(y, 0, sizeof(double) * n);
    mult(&a, (double *)x, y);
}

/* The reference's single-rank Matrix Market loader (src/matrix.c:402-419).
 * First call with out arrays NULL to learn n and nnz; second call fills them
 * (diagonal block only: the off-diagonal block is empty on one rank). */
int ref_load_block(const char *path, unsigned *n_out, unsigned *nz_out, unsigned *ptr, unsigned *col, double *val,
                   char *code_out) {
    CSR_Matrix diag, offd;
    INFO_Matrix info;
    int recv = 0, displ = 0;
    info.recvcounts = &recv;
    info.displs = &displ;
    MPI_csr_load_matrix_block((char *)path, &diag, &offd, &info);
    *n_out = diag.rows;
    *nz_out = diag.nz;
    if (code_out) memcpy(code_out, info.code, 4);
    if (ptr) memcpy(ptr, diag.ptr, sizeof(unsigned) * ((size_t)diag.rows + 1));
    if (col) memcpy(col, diag.col, sizeof(unsigned) * diag.nz);
    if (val) memcpy(val, diag.val, sizeof(double) * diag.nz);
    int offd_nz = (int)offd.nz;
    csr_free_matrix(&diag);
    csr_free_matrix(&offd);
    return offd_nz;
}

/* The reference's serial loader (src/matrix.c:234-242): real, integer and
 * pattern values; returns mm_is_symmetric of the banner. */
int ref_load_csr(const char *path, unsigned *n_out, unsigned *nz_out, unsigned *ptr, unsigned *col, double *val) {
    CSR_Matrix a;
    csr_init_matrix(&a);
    int sym = csr_load_matrix((char *)path, &a);
    *n_out = a.rows;
    *nz_out = a.nz;
    if (ptr) memcpy(ptr, a.ptr, sizeof(unsigned) * ((size_t)a.rows + 1));
    if (col) memcpy(col, a.col, sizeof(unsigned) * a.nz);
    if (val) memcpy(val, a.val, sizeof(double) * a.nz);
    csr_free_matrix(&a);
    return sym;
}

/* mm_read_banner + mm_read_mtx_crd_size (src/mmio.c:96,189) on a file. */
int ref_read_header(const char *path, char *code_out, int *m, int *n, int *nz) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    MM_typecode code;
    int rc = mm_read_banner(f, &code);
    if (rc == 0) rc = mm_read_mtx_crd_size(f, m, n, nz);
    memcpy(code_out, code, 4);
    fclose(f);
    return rc;
}
