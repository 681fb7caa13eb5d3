/* Parallel Matrix Market coordinate reader.
 *
 * The reference reads its matrices with one fscanf per entry
 * (src/matrix.c:26-94, through src/mmio.c:96-218), which takes minutes for a
 * matrix of 10^8 entries.  This reader maps the file, splits the body into
 * line-aligned chunks, counts the entries of every chunk in parallel, and
 * parses the chunks in parallel into their final positions, so the entries
 * keep file order.  Values go through strtod, the conversion fscanf("%lg")
 * performs, so the doubles are the reference's bit for bit.
 *
 * Accepted: "%%MatrixMarket matrix coordinate {real|double|integer|pattern}
 * {general|symmetric|skew-symmetric}" (keywords in any case, as src/mmio.c
 * accepts them).  Pattern entries get the value 1.0, integer entries their
 * value.  Symmetric files are returned as stored unless expand_symmetric is
 * set; then the mirror of every off-diagonal entry (negated for
 * skew-symmetric) is appended after all stored entries, in file order.  (The
 * reference never expands them, src/matrix.c:93.)  Errors are returned, not
 * exit()ed. */
#define _GNU_SOURCE
#include <ctype.h>
#include <errno.h>
#include <fcntl.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "host_internal.h"

static void msgf(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    hbicg__set_message(buf);
}

enum { F_REAL = 0, F_INTEGER = 1, F_PATTERN = 2 };
enum { S_GENERAL = 0, S_SYMMETRIC = 1, S_SKEW = 2 };

typedef struct {
    const char *b, *e;          /* chunk [b, e), starts at a line start */
    unsigned long long first;   /* index of its first entry */
    unsigned long long count;   /* entries in the chunk */
    unsigned long long offdiag; /* off-diagonal entries (for expansion) */
    unsigned long long mirror0; /* index of its first mirrored entry */
    int field, sym, err;
    unsigned M, N;
    unsigned *row, *col;
    double *val;
    char msg[160];
} chunk_t;

static int blank_line(const char *p, const char *e) {
    for (; p < e && *p != '\n'; ++p)
        if (!isspace((unsigned char)*p)) return 0;
    return 1;
}

static void *count_chunk(void *arg) {
    chunk_t *c = arg;
    unsigned long long k = 0;
    for (const char *p = c->b; p < c->e;) {
        const char *nl = memchr(p, '\n', (size_t)(c->e - p));
        const char *le = nl ? nl : c->e;
        if (!blank_line(p, le)) ++k;
        p = nl ? nl + 1 : c->e;
    }
    c->count = k;
    return NULL;
}

/* unsigned decimal at *pp (leading blanks skipped); 0 on failure */
static int read_index(const char **pp, const char *e, unsigned long long *v) {
    const char *p = *pp;
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p >= e || !isdigit((unsigned char)*p)) return 0;
    unsigned long long x = 0;
    while (p < e && isdigit((unsigned char)*p)) {
        x = x * 10 + (unsigned)(*p - '0');
        if (x > 0xFFFFFFFFull) return 0;
        ++p;
    }
    *pp = p;
    *v = x;
    return 1;
}

static void *parse_chunk(void *arg) {
    chunk_t *c = arg;
    unsigned long long k = c->first, nd = 0;
    char buf[128];
    for (const char *p = c->b; p < c->e;) {
        const char *nl = memchr(p, '\n', (size_t)(c->e - p));
        const char *le = nl ? nl : c->e;
        if (!blank_line(p, le)) {
            unsigned long long r, q;
            const char *s = p;
            if (!read_index(&s, le, &r) || !read_index(&s, le, &q) || r < 1 || q < 1 || r > c->M || q > c->N) {
                c->err = 1;
                snprintf(c->msg, sizeof c->msg, "bad index in entry %llu", k + 1);
                return NULL;
            }
            double v = 1.0;
            if (c->field != F_PATTERN) {
                while (s < le && (*s == ' ' || *s == '\t')) ++s;
                size_t len = (size_t)(le - s);
                if (len == 0 || len >= sizeof buf) {
                    c->err = 1;
                    snprintf(c->msg, sizeof c->msg, "missing or overlong value in entry %llu", k + 1);
                    return NULL;
                }
                memcpy(buf, s, len);
                buf[len] = 0;
                char *end = NULL;
                if (c->field == F_INTEGER) {
                    errno = 0;
                    long long iv = strtoll(buf, &end, 10);
                    if (end == buf || errno) {
                        c->err = 1;
                        snprintf(c->msg, sizeof c->msg, "bad integer value in entry %llu", k + 1);
                        return NULL;
                    }
                    v = (double)iv;
                } else {
                    v = strtod(buf, &end);
                    if (end == buf) {
                        c->err = 1;
                        snprintf(c->msg, sizeof c->msg, "bad value in entry %llu", k + 1);
                        return NULL;
                    }
                }
            }
            c->row[k] = (unsigned)(r - 1);
            c->col[k] = (unsigned)(q - 1);
            c->val[k] = v;
            if (r != q) ++nd;
            ++k;
        }
        p = nl ? nl + 1 : c->e;
    }
    c->offdiag = nd;
    return NULL;
}

static void *mirror_chunk(void *arg) {
    chunk_t *c = arg;
    unsigned long long o = c->mirror0;
    const double sgn = c->sym == S_SKEW ? -1.0 : 1.0;
    for (unsigned long long k = c->first; k < c->first + c->count; ++k) {
        if (c->row[k] == c->col[k]) continue;
        c->row[o] = c->col[k];
        c->col[o] = c->row[k];
        c->val[o] = sgn * c->val[k];
        ++o;
    }
    return NULL;
}

static int run_all(chunk_t *ch, int nt, void *(*fn)(void *)) {
    pthread_t th[64];
    int started = 0;
    for (int t = 1; t < nt; ++t) {
        if (pthread_create(&th[t], NULL, fn, &ch[t]) != 0) break;
        started = t;
    }
    fn(&ch[0]);
    for (int t = started + 1; t < nt; ++t) fn(&ch[t]); /* threads that could not start */
    for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* next token of the banner/size lines */
static const char *token(const char *p, const char *e, char *out, size_t cap) {
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    size_t n = 0;
    while (p < e && !isspace((unsigned char)*p)) {
        if (n + 1 < cap) out[n++] = *p;
        ++p;
    }
    out[n] = 0;
    return p;
}

void hbicg_coo_free(hbicg_coo *c) {
    if (!c) return;
    free(c->row);
    free(c->col);
    free(c->val);
    memset(c, 0, sizeof *c);
}

int hbicg_mm_read(const char *path, int expand_symmetric, int threads, hbicg_coo *out) {
    if (!path || !out) return HBICG_E_ARG;
    memset(out, 0, sizeof *out);
    int fd = open(path, O_RDONLY);
    if (fd < 0) {
        msgf("cannot open %s: %s", path, strerror(errno));
        return HBICG_E_IO;
    }
    struct stat stt;
    if (fstat(fd, &stt) != 0 || stt.st_size == 0) {
        close(fd);
        msgf("cannot read %s", path);
        return HBICG_E_IO;
    }
    const size_t size = (size_t)stt.st_size;
    char *map = mmap(NULL, size, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    if (map == MAP_FAILED) {
        msgf("cannot map %s", path);
        return HBICG_E_IO;
    }
    const char *p = map, *e = map + size;
    int rc = HBICG_OK;
    chunk_t *ch = NULL;
    /* banner */
    const char *nl = memchr(p, '\n', size);
    const char *le = nl ? nl : e;
    char t0[64], t1[64], t2[64], t3[64], t4[64];
    const char *q = token(p, le, t0, sizeof t0);
    q = token(q, le, t1, sizeof t1);
    q = token(q, le, t2, sizeof t2);
    q = token(q, le, t3, sizeof t3);
    q = token(q, le, t4, sizeof t4);
    if (strcmp(t0, "%%MatrixMarket") != 0 || strcasecmp(t1, "matrix") != 0 || strcasecmp(t2, "coordinate") != 0) {
        msgf("%s: not a Matrix Market coordinate matrix", path);
        rc = HBICG_E_IO;
        goto done;
    }
    int field, sym;
    if (!strcasecmp(t3, "real") || !strcasecmp(t3, "double")) field = F_REAL;
    else if (!strcasecmp(t3, "integer")) field = F_INTEGER;
    else if (!strcasecmp(t3, "pattern")) field = F_PATTERN;
    else {
        msgf("%s: unsupported field '%s'", path, t3);
        rc = HBICG_E_IO;
        goto done;
    }
    if (!strcasecmp(t4, "general")) sym = S_GENERAL;
    else if (!strcasecmp(t4, "symmetric")) sym = S_SYMMETRIC;
    else if (!strcasecmp(t4, "skew-symmetric")) sym = S_SKEW;
    else {
        msgf("%s: unsupported symmetry '%s'", path, t4);
        rc = HBICG_E_IO;
        goto done;
    }
    /* comments, then the size line */
    p = nl ? nl + 1 : e;
    while (p < e && (*p == '%' || blank_line(p, e))) {
        nl = memchr(p, '\n', (size_t)(e - p));
        p = nl ? nl + 1 : e;
    }
    nl = memchr(p, '\n', (size_t)(e - p));
    le = nl ? nl : e;
    unsigned long long M, N, NZ;
    {
        const char *s = p;
        if (!read_index(&s, le, &M) || !read_index(&s, le, &N) || !read_index(&s, le, &NZ)) {
            msgf("%s: could not read the size line", path);
            rc = HBICG_E_IO;
            goto done;
        }
    }
    const char *body = nl ? nl + 1 : e;
    /* chunks */
    long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
    int nt = threads > 0 ? threads : (int)(ncpu > 0 ? ncpu : 1);
    if (nt > 64) nt = 64;
    const size_t bytes = (size_t)(e - body);
    if (bytes < (size_t)nt * 65536) nt = (int)(bytes / 65536) + 1;
    ch = calloc((size_t)nt, sizeof *ch);
    if (!ch) {
        rc = HBICG_E_NOMEM;
        goto done;
    }
    const char *cur = body;
    for (int t = 0; t < nt; ++t) {
        const char *end = t + 1 == nt ? e : body + bytes * (size_t)(t + 1) / (size_t)nt;
        if (end < cur) end = cur;
        if (t + 1 < nt) {
            const char *x = memchr(end, '\n', (size_t)(e - end));
            end = x ? x + 1 : e;
        }
        ch[t].b = cur;
        ch[t].e = end;
        ch[t].field = field;
        ch[t].sym = sym;
        ch[t].M = (unsigned)M;
        ch[t].N = (unsigned)N;
        cur = end;
    }
    run_all(ch, nt, count_chunk);
    unsigned long long total = 0;
    for (int t = 0; t < nt; ++t) {
        ch[t].first = total;
        total += ch[t].count;
    }
    if (total != NZ) {
        msgf("%s: %llu entries, the size line says %llu", path, total, NZ);
        rc = HBICG_E_IO;
        goto done;
    }
    /* room for the mirrored entries is sized after the parse: first parse
     * into arrays of NZ, then grow when expanding */
    out->row = malloc(sizeof(unsigned) * (size_t)(NZ + 1));
    out->col = malloc(sizeof(unsigned) * (size_t)(NZ + 1));
    out->val = malloc(sizeof(double) * (size_t)(NZ + 1));
    if (!out->row || !out->col || !out->val) {
        rc = HBICG_E_NOMEM;
        goto done;
    }
    for (int t = 0; t < nt; ++t) {
        ch[t].row = out->row;
        ch[t].col = out->col;
        ch[t].val = out->val;
    }
    run_all(ch, nt, parse_chunk);
    for (int t = 0; t < nt; ++t)
        if (ch[t].err) {
            msgf("%s: %s", path, ch[t].msg);
            rc = HBICG_E_IO;
            goto done;
        }
    unsigned long long nnz = NZ;
    if (expand_symmetric && sym != S_GENERAL) {
        unsigned long long extra = 0;
        for (int t = 0; t < nt; ++t) {
            ch[t].mirror0 = NZ + extra;
            extra += ch[t].offdiag;
        }
        nnz = NZ + extra;
        unsigned *r2 = realloc(out->row, sizeof(unsigned) * (size_t)(nnz + 1));
        if (r2) out->row = r2;
        unsigned *c2 = realloc(out->col, sizeof(unsigned) * (size_t)(nnz + 1));
        if (c2) out->col = c2;
        double *v2 = realloc(out->val, sizeof(double) * (size_t)(nnz + 1));
        if (v2) out->val = v2;
        if (!r2 || !c2 || !v2) {
            rc = HBICG_E_NOMEM;
            goto done;
        }
        for (int t = 0; t < nt; ++t) {
            ch[t].row = out->row;
            ch[t].col = out->col;
            ch[t].val = out->val;
        }
        run_all(ch, nt, mirror_chunk);
    }
    out->rows = (unsigned)M;
    out->cols = (unsigned)N;
    out->nnz = nnz;
    out->field = field;
    out->symmetry = sym;
    out->expanded = expand_symmetric && sym != S_GENERAL;
done:
    free(ch);
    munmap(map, size);
    if (rc != HBICG_OK) hbicg_coo_free(out);
    return rc;
}
