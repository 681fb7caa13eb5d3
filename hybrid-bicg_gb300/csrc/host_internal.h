/* Internal interface between the host-side translation units of libhbicg:
 * the context and matrix objects, the per-thread error message and the error
 * checks every host entry point uses.  Not installed; not part of the C ABI. */
#pragma once
#include <stddef.h>

#include <cuda_runtime.h>

#include "hbicg.h"
#include "hbk.h"

struct hbicg_context {
    cudaStream_t stream;
    cudaStream_t cstream;  /* copies of finished solutions to the host during a solve */
    cudaEvent_t ev0, ev1, evf0, evf1, cev;
    hbk_scalars *h_sc; /* pinned */
    double *h_dbl;     /* pinned scratch */
    int refs;          /* the caller's handle + one per live matrix or solver */
};

struct hbicg_matrix {
    hbicg_context *ctx;
    hbk_matrix k;
    unsigned *d_ptr, *d_col;
    double *d_val;
    int owns;
    int pooled; /* d_ptr, d_col, d_val came from the library's pool (hbicg__dev_alloc) */
    unsigned *d_blk_row;
    unsigned char *d_blk_kind;
    double *d_sval;
    unsigned *d_scol;
    unsigned long long *d_sptr;
    /* positions of the diagonal entries in the SELL-32 arrays (for folding a
     * shift into the diagonal); diag_state: 0 not computed, 1 ok, 2 a row has
     * no stored diagonal */
    unsigned long long *d_sdiag;
    int diag_state;
    /* HYB form (hbk.h HBK_FMT_HYB) */
    double *d_hval;
    unsigned *d_hcol, *d_srow, *d_wrow; /* d_srow: lane -> row map, then the lanes' row lengths (bytes) */
    size_t slen_off;                    /* entries of the map before the lengths */
    unsigned long long *d_hsptr;
    unsigned nslice, nwrow;
    unsigned hnw;  /* warp work lists in d_wrow (after the long rows' entry ranges and the long rows) */
    int hyb_grid;  /* blocks of the HYB kernels: one list per warp */
    unsigned hrow32, hrow16, hit16, hit4, hitl; /* HYB lane classes of the long rows (hbk.h) */
    /* MERGE form (hbk.h HBK_FMT_MERGE): block row ranges, then the long rows,
     * in one allocation */
    unsigned *d_merge;
    unsigned nmblk, nmlong;
};

/* message of the last failed call on this thread (hbicg_last_message) */
void hbicg__set_msg(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
void hbicg__set_message(const char *msg);
#define set_msg hbicg__set_msg

/* a context lives while its handle or any matrix or solver made on it does */
void hbicg__ctx_retain(hbicg_context *c);
void hbicg__ctx_release(hbicg_context *c);

/* HYB warp work lists (host only): ni items with costs dealt costliest first
 * (ties: lower item), each to the list with the least cost so far (ties:
 * lower list); hwbeg[hnw + 1] list starts, hitem[ni] the lists in order of
 * dealing.  HBICG_OK or HBICG_E_NOMEM. */
int hbicg__hyb_plan(size_t ni, const unsigned *cost, unsigned hnw, unsigned *hwbeg, unsigned *hitem);

/* positions of A's SELL-32 diagonal entries (computed once per layout) */
int hbicg__sell_diag(hbicg_matrix *A);
/* device arrays from the library's stream-ordered pool (solver.c) */
cudaError_t hbicg__dev_alloc(void **p, size_t bytes, cudaStream_t st);
void hbicg__dev_free(void *p, cudaStream_t st);
/* the shift mode a solver made with p takes for n rows and m shifts */
int hbicg__shift_mode_for(const hbicg_params *p, unsigned n, int m);
/* many families' iterations in one persistent launch (solver.c) */
typedef struct hbicg__group hbicg__group;
int hbicg__group_eligible(const hbicg_solver *s);
hbicg__group *hbicg__group_new(int cap, int max_ctas);
/* a family's first step; returns its slot (its status: hbicg__group_finish) */
int hbicg__group_add(hbicg__group *g, hbicg_solver *s, const double *b, const double *sigma, int seed, double *x,
                     hbicg_stats *st);
int hbicg__group_launch(hbicg__group *g);
int hbicg__group_finish(hbicg__group *g, int slot);
void hbicg__group_free(hbicg__group *g);
/* a context whose stream has the device's greatest priority when high = 1 */
int hbicg__context_create_prio(hbicg_context **out, int high);
const hbk_matrix *hbicg__matrix_kernel_view(const hbicg_matrix *A);
hbicg_context *hbicg__matrix_context(const hbicg_matrix *A);
/* y (+)= A x for host arrays, on a process-wide context (matrix.h's mult) */
int hbicg__host_spmv(unsigned rows, unsigned cols, unsigned nnz, const unsigned *ptr, const unsigned *col,
                     const double *val, const double *x, double *y, int accumulate);

/* leading dimension of the per-shift vectors: 256-byte aligned rows */
static inline size_t hbicg__ld_of(unsigned n) { return ((size_t)n + 31) / 32 * 32; }

#define CUDA_TRY(call)                                                                                   \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));                  \
            return e_ == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;                       \
        }                                                                                                \
    } while (0)

#define HBK_TRY(call)                                                                                    \
    do {                                                                                                 \
        int e_ = (call);                                                                                 \
        if (e_) {                                                                                        \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, hbk_error_string(e_));                    \
            return HBICG_E_CUDA;                                                                         \
        }                                                                                                \
    } while (0)

/* the same two checks for functions that own host or device scratch: set rc
 * and leave through their `out:` cleanup */
#define CUDA_GOTO(call)                                                                                  \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));                  \
            rc = e_ == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;                         \
            goto out;                                                                                    \
        }                                                                                                \
    } while (0)
#define HBK_GOTO(call)                                                                                   \
    do {                                                                                                 \
        int e_ = (call);                                                                                 \
        if (e_) {                                                                                        \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, hbk_error_string(e_));                    \
            rc = HBICG_E_CUDA;                                                                           \
            goto out;                                                                                    \
        }                                                                                                \
    } while (0)
