/*
 * oops_expv.h -- C-ABI of liboops_gb300.so, the GB300 (sm_103a) drop-in for
 * the nzhao/oops expv library (libexpv.so).
 *
 * Plain C types only: sizes are size_t, complex numbers are (re, im) double
 * pairs (std::complex<double> in C++, double _Complex in C), device buffers and
 * CUDA streams are passed as void*.  Every oops_* entry point returns an int
 * status (OOPS_OK or a negative OOPS_ERR_*); the two reference-compatible
 * void entry points record their status for oops_expv_status().
 *
 * Term-list arguments (nspin ... nspin_dim) are the flattened SumKronProd that
 * MatExpVector::runInexplicitGPU builds (src/source/math/MatExp.cpp:367-420):
 * real coefficients, bodies per term, 0-based position offsets (nterm+1),
 * spin positions, body dimensions, matrix offsets and column-major body
 * matrices.  Spin 0 is the most significant Kronecker index.
 */
#ifndef OOPS_EXPV_H
#define OOPS_EXPV_H

#include <stddef.h>

#ifdef __cplusplus
#include <complex>
typedef std::complex<double> oops_zcomplex;
extern "C" {
#else
typedef double _Complex oops_zcomplex;
#endif

/* status codes */
#define OOPS_OK 0
#define OOPS_ERR_ARG (-1)          /* null pointer / inconsistent arguments      */
#define OOPS_ERR_SIZE (-3)         /* m >= n, m == 0, sizes beyond limits        */
#define OOPS_ERR_UNSUPPORTED (-4)  /* e.g. a term with more than two bodies      */
#define OOPS_ERR_CUDA (-5)         /* CUDA runtime error (message kept)          */
#define OOPS_ERR_NOMEM (-6)        /* device allocation failed                   */
#define OOPS_ERR_NUMERIC (-7)      /* Pade denominator singular, NaN, step cap   */
#define OOPS_ERR_TIMEOUT (-8)      /* bounded device wait expired                */

/* ------------------------------------------------------------------------
 * Reference-compatible entry points (libexpv.so replacements)
 * ---------------------------------------------------------------------- */

/* Replaces main_cache_ (src/expv/include/main_cache.h:6, Fortran MAIN_CACHE in
 * src/expv/source/main_cache.f:1-136 driving ZGEXPV_CACHE,
 * src/expv/source/zgexpv_cache.f:4-690).  Computes
 *   w_seq(:, tt) = exp(-i H ta[tt]) v,  tt = 0 .. tn-1,
 * with ta increasing and measured from 0, H = sum coeff[t] (x) mats.  Host
 * pointers throughout; the whole integration is device-resident.
 * maxThreadsPerBlock / maxGridSize are accepted and ignored (launch shapes are
 * chosen for sm_103a).  k is the Lanczos length of the norm estimate (the
 * reference passes 10), m the Krylov dimension (1 <= m < ham_dim, m <= 50),
 * tol the local error tolerance.  The status is kept for oops_expv_status(). */
void main_cache_(size_t *nspin, size_t *nTerm, double *coeff_lst,
                 size_t *nbody_lst, size_t *pos_i_idx, size_t *pos_i_lst,
                 size_t *dim_i_lst, size_t *mat_i_idx, oops_zcomplex *mat_i_lst,
                 size_t *ham_dim, size_t *nspin_dim, oops_zcomplex *v,
                 size_t *pos_idx, size_t *mat_idx, size_t *k,
                 size_t *maxThreadsPerBlock, size_t *maxGridSize, size_t *tn,
                 double *ta, size_t *m, double *tol, size_t *itrace,
                 oops_zcomplex *w_seq, size_t *w_seq_len);

/* Replaces main_mkl_ (src/expv/include/main_mkl.h:6, src/expv/source/
 * main_mkl.f:1-130).  Same computation and arguments minus the two CUDA
 * geometry arguments; served by the same GPU path (there is no CPU path in
 * this library). */
void main_mkl_(size_t *nspin, size_t *nTerm, double *coeff_lst,
               size_t *nbody_lst, size_t *pos_i_idx, size_t *pos_i_lst,
               size_t *dim_i_lst, size_t *mat_i_idx, oops_zcomplex *mat_i_lst,
               size_t *ham_dim, size_t *nspin_dim, oops_zcomplex *v,
               size_t *pos_idx, size_t *mat_idx, size_t *k, size_t *tn,
               double *ta, size_t *m, double *tol, size_t *itrace,
               oops_zcomplex *w_seq, size_t *w_seq_len);

/* Status of the calling thread's last main_cache_ / main_mkl_ call (the
 * reference has no error return: it stops the process or ignores CUDA
 * errors, zgexpv_cache.f:378, hamvec_cuda3.cu:479). */
int oops_expv_status(void);
/* Message for the calling thread's last failure ("" when none). */
const char *oops_expv_error(void);

/* Status and message of the calling thread's last oops_* call of any kind
 * (no counterpart in the reference, which has no error reporting). */
int oops_last_status(void);
const char *oops_last_error(void);

/* ------------------------------------------------------------------------
 * Hamiltonian handle and device matvec
 * ---------------------------------------------------------------------- */
typedef struct oops_ham oops_ham;

/* Upload a term list (layout above) to the current device.  Terms may have 1
 * or 2 bodies (hamvec_cuda3.cu:556-619 supports the same; more bodies give
 * OOPS_ERR_UNSUPPORTED).  All-spin-1/2 systems use the bit-flip kernel, other
 * dimensions the generic mode-product kernel. */
int oops_ham_create(size_t nspin, size_t nterm, const double *coeff_lst,
                    const size_t *nbody_lst, const size_t *pos_i_idx,
                    const size_t *pos_i_lst, const size_t *dim_i_lst,
                    const size_t *mat_i_idx, const oops_zcomplex *mat_i_lst,
                    const size_t *nspin_dim, oops_ham **out);
int oops_ham_destroy(oops_ham *h);
size_t oops_ham_dim(const oops_ham *h);

/* y = alpha * H x on a block of nvec vectors held interleaved on the device
 * (element (i, b) at index i*nvec + b); nvec a power of two <= 4096.  Replaces hamvec_cuda3_
 * (src/expv/source/hamvec_cuda3.cu:661-696), which applied one term per
 * launch to a single vector. */
int oops_ham_apply(const oops_ham *h, double alpha_re, double alpha_im,
                   const void *x_dev, void *y_dev, size_t nvec, void *stream);

/* ------------------------------------------------------------------------
 * Block Krylov expv (device pointers)
 * ---------------------------------------------------------------------- */
typedef struct {
    long nmult, nexph, nscale, nstep, nreject, ibrkflag, mbrkdwn;
    double anorm, step_min, step_max, x_error, s_error, hump;
} oops_expv_stats;

/* W(tt, :, b) = exp(-i H ta[b*tn + tt]) V(:, b) for nvec columns of a block
 * (interleaved layout, V has ham_dim*nvec entries, W has tn*ham_dim*nvec),
 * each column with its own increasing time list.  Same algorithm as
 * main_cache_, one adaptive step control per column, Arnoldi in lockstep.
 * nvec <= 256 per call.  stats (optional, host) receives column 0's counters. */
int oops_expv_block(const oops_ham *h, const void *V_dev, size_t nvec,
                    size_t tn, const double *ta_host, size_t m, double tol,
                    size_t klim, void *W_dev, oops_expv_stats *stats,
                    void *stream);

#ifdef __cplusplus
}
#endif
#endif
