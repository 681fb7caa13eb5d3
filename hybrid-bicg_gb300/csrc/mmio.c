/* Matrix Market coordinate I/O (see include/mmio.h).
 *
 * Behaviour follows the reference's reader where its loaders depend on it:
 * the banner's four tokens are matched case-insensitively after the
 * "%%MatrixMarket" marker (src/mmio.c:96-179); the size line is the first
 * line that does not start with '%', and if it does not hold three integers
 * the reader keeps scanning for them (src/mmio.c:189-217).
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mmio.h"

static void lower(char *s) {
    for (; *s; s++) *s = (char)tolower((unsigned char)*s);
}

int mm_read_banner(FILE *f, MM_typecode *code) {
    char line[MM_MAX_LINE_LENGTH];
    char tok[5][MM_MAX_TOKEN_LENGTH];
    mm_clear_typecode(code);
    if (!fgets(line, sizeof line, f)) return MM_PREMATURE_EOF;
    if (sscanf(line, "%63s %63s %63s %63s %63s", tok[0], tok[1], tok[2], tok[3], tok[4]) != 5)
        return MM_PREMATURE_EOF;
    if (strncmp(tok[0], MatrixMarketBanner, strlen(MatrixMarketBanner)) != 0) return MM_NO_HEADER;
    for (int i = 1; i < 5; i++) lower(tok[i]);
    if (strcmp(tok[1], MM_MTX_STR) != 0) return MM_UNSUPPORTED_TYPE;
    mm_set_matrix(code);

    if (!strcmp(tok[2], MM_SPARSE_STR)) mm_set_sparse(code);
    else if (!strcmp(tok[2], MM_DENSE_STR)) mm_set_dense(code);
    else return MM_UNSUPPORTED_TYPE;

    if (!strcmp(tok[3], MM_REAL_STR)) mm_set_real(code);
    else if (!strcmp(tok[3], MM_COMPLEX_STR)) mm_set_complex(code);
    else if (!strcmp(tok[3], MM_PATTERN_STR)) mm_set_pattern(code);
    else if (!strcmp(tok[3], MM_INT_STR)) mm_set_integer(code);
    else return MM_UNSUPPORTED_TYPE;

    if (!strcmp(tok[4], MM_GENERAL_STR)) mm_set_general(code);
    else if (!strcmp(tok[4], MM_SYMM_STR)) mm_set_symmetric(code);
    else if (!strcmp(tok[4], MM_HERM_STR)) mm_set_hermitian(code);
    else if (!strcmp(tok[4], MM_SKEW_STR)) mm_set_skew(code);
    else return MM_UNSUPPORTED_TYPE;
    return 0;
}

/* skip '%' lines; parse `count` integers from the first other line, or keep
 * scanning the stream for them */
static int read_ints(FILE *f, int count, int *a, int *b, int *c) {
    char line[MM_MAX_LINE_LENGTH];
    do {
        if (!fgets(line, sizeof line, f)) return MM_PREMATURE_EOF;
    } while (line[0] == '%');
    int got = count == 3 ? sscanf(line, "%d %d %d", a, b, c) : sscanf(line, "%d %d", a, b);
    while (got != count) {
        got = count == 3 ? fscanf(f, "%d %d %d", a, b, c) : fscanf(f, "%d %d", a, b);
        if (got == EOF) return MM_PREMATURE_EOF;
    }
    return 0;
}

int mm_read_mtx_crd_size(FILE *f, int *M, int *N, int *nz) {
    *M = *N = *nz = 0;
    return read_ints(f, 3, M, N, nz);
}

int mm_read_mtx_array_size(FILE *f, int *M, int *N) {
    int unused = 0;
    *M = *N = 0;
    return read_ints(f, 2, M, N, &unused);
}

int mm_write_mtx_crd_size(FILE *f, int M, int N, int nz) {
    return fprintf(f, "%d %d %d\n", M, N, nz) < 0 ? MM_COULD_NOT_WRITE_FILE : 0;
}

int mm_write_mtx_array_size(FILE *f, int M, int N) {
    return fprintf(f, "%d %d\n", M, N) < 0 ? MM_COULD_NOT_WRITE_FILE : 0;
}

int mm_is_valid(MM_typecode code) {
    if (!mm_is_matrix(code)) return 0;
    if (mm_is_dense(code) && mm_is_pattern(code)) return 0;
    if (mm_is_real(code) && mm_is_hermitian(code)) return 0;
    if (mm_is_pattern(code) && (mm_is_hermitian(code) || mm_is_skew(code))) return 0;
    return 1;
}

char *mm_typecode_to_str(MM_typecode code) {
    const char *storage, *field, *sym;
    if (!mm_is_matrix(code)) return NULL;
    if (mm_is_sparse(code)) storage = MM_SPARSE_STR;
    else if (mm_is_dense(code)) storage = MM_DENSE_STR;
    else return NULL;
    if (mm_is_real(code)) field = MM_REAL_STR;
    else if (mm_is_complex(code)) field = MM_COMPLEX_STR;
    else if (mm_is_pattern(code)) field = MM_PATTERN_STR;
    else if (mm_is_integer(code)) field = MM_INT_STR;
    else return NULL;
    if (mm_is_general(code)) sym = MM_GENERAL_STR;
    else if (mm_is_symmetric(code)) sym = MM_SYMM_STR;
    else if (mm_is_hermitian(code)) sym = MM_HERM_STR;
    else if (mm_is_skew(code)) sym = MM_SKEW_STR;
    else return NULL;
    size_t len = strlen(MM_MTX_STR) + strlen(storage) + strlen(field) + strlen(sym) + 4;
    char *out = malloc(len);
    if (out) snprintf(out, len, "%s %s %s %s", MM_MTX_STR, storage, field, sym);
    return out;
}

int mm_write_banner(FILE *f, MM_typecode code) {
    char *s = mm_typecode_to_str(code);
    if (!s) return MM_UNSUPPORTED_TYPE;
    int rc = fprintf(f, "%s %s\n", MatrixMarketBanner, s);
    free(s);
    return rc < 0 ? MM_COULD_NOT_WRITE_FILE : 0;
}

int mm_read_mtx_crd_entry(FILE *f, int *I, int *J, double *real, double *img, MM_typecode code) {
    if (mm_is_complex(code)) return fscanf(f, "%d %d %lg %lg", I, J, real, img) == 4 ? 0 : MM_PREMATURE_EOF;
    if (mm_is_real(code)) return fscanf(f, "%d %d %lg", I, J, real) == 3 ? 0 : MM_PREMATURE_EOF;
    if (mm_is_integer(code)) {
        int v;
        if (fscanf(f, "%d %d %d", I, J, &v) != 3) return MM_PREMATURE_EOF;
        *real = (double)v;
        return 0;
    }
    if (mm_is_pattern(code)) return fscanf(f, "%d %d", I, J) == 2 ? 0 : MM_PREMATURE_EOF;
    return MM_UNSUPPORTED_TYPE;
}

int mm_read_mtx_crd_data(FILE *f, int M, int N, int nz, int I[], int J[], double val[], MM_typecode code) {
    (void)M;
    (void)N;
    for (int i = 0; i < nz; i++) {
        double re = 0.0, im = 0.0;
        int rc = mm_read_mtx_crd_entry(f, &I[i], &J[i], &re, &im, code);
        if (rc) return rc;
        if (mm_is_complex(code)) {
            val[2 * i] = re;
            val[2 * i + 1] = im;
        } else if (!mm_is_pattern(code)) {
            val[i] = re;
        }
    }
    return 0;
}

int mm_write_mtx_crd(char fname[], int M, int N, int nz, int I[], int J[], double val[], MM_typecode code) {
    FILE *f = strcmp(fname, "stdout") == 0 ? stdout : fopen(fname, "w");
    if (!f) return MM_COULD_NOT_WRITE_FILE;
    int rc = mm_write_banner(f, code);
    if (!rc) rc = mm_write_mtx_crd_size(f, M, N, nz);
    for (int i = 0; !rc && i < nz; i++) {
        int w;
        if (mm_is_pattern(code)) w = fprintf(f, "%d %d\n", I[i], J[i]);
        else if (mm_is_complex(code)) w = fprintf(f, "%d %d %.17g %.17g\n", I[i], J[i], val[2 * i], val[2 * i + 1]);
        else w = fprintf(f, "%d %d %.17g\n", I[i], J[i], val[i]);
        if (w < 0) rc = MM_COULD_NOT_WRITE_FILE;
    }
    if (f != stdout) fclose(f);
    return rc;
}
