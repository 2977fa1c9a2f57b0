// capi.cu -- the extern "C" surface of liboops_gb300.so: the reference-compatible
// main_cache_ / main_mkl_ drop-ins, status reporting and the block expv.
#include <cuda_runtime.h>

#include <string>

#include "oops_common.cuh"
#include "oops_internal.h"

int oops_expv_run(const oops_ham *h, const zd *V_in, size_t nvec, size_t tn,
                  const double *ta_host, size_t m, double tol, size_t klim, zd *W_out,
                  oops_expv_stats *stats, cudaStream_t st);

namespace {
thread_local int g_status = OOPS_OK;
thread_local std::string g_msg;
thread_local int g_drop_status = OOPS_OK;
thread_local std::string g_drop_msg;
}  // namespace

int oops_set_status(int code, const char *msg)
{
    g_status = code;
    g_msg = msg ? msg : "";
    return code;
}

int oops_sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

extern "C" int oops_expv_status(void) { return g_drop_status; }
extern "C" const char *oops_expv_error(void) { return g_drop_msg.c_str(); }
extern "C" int oops_last_status(void) { return g_status; }
extern "C" const char *oops_last_error(void) { return g_msg.c_str(); }

extern "C" int oops_expv_block(const oops_ham *h, const void *V_dev, size_t nvec, size_t tn,
                               const double *ta_host, size_t m, double tol, size_t klim,
                               void *W_dev, oops_expv_stats *stats, void *stream)
{
    g_status = OOPS_OK;
    g_msg.clear();
    if (!h || !V_dev || !W_dev || (tn && !ta_host)) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    return oops_expv_run(h, (const zd *)V_dev, nvec, tn, ta_host, m, tol, klim, (zd *)W_dev,
                         stats, (cudaStream_t)stream);
}

// shared body of main_cache_ / main_mkl_
static int drop_in(size_t *nspin, size_t *nTerm, double *coeff_lst, size_t *nbody_lst,
                   size_t *pos_i_idx, size_t *pos_i_lst, size_t *dim_i_lst, size_t *mat_i_idx,
                   oops_zcomplex *mat_i_lst, size_t *ham_dim, size_t *nspin_dim,
                   oops_zcomplex *v, size_t *k, size_t *tn, double *ta, size_t *m, double *tol,
                   oops_zcomplex *w_seq, size_t *w_seq_len)
{
    g_status = OOPS_OK;
    g_msg.clear();
    if (!nspin || !nTerm || !ham_dim || !nspin_dim || !v || !k || !tn || !m || !tol || !w_seq ||
        !w_seq_len || (*tn && !ta))
        return oops_set_status(OOPS_ERR_ARG, "null argument");
    oops_ham *h = nullptr;
    int rc = oops_ham_create(*nspin, *nTerm, coeff_lst, nbody_lst, pos_i_idx, pos_i_lst, dim_i_lst,
                             mat_i_idx, mat_i_lst, nspin_dim, &h);
    if (rc) return rc;
    const size_t N = oops_ham_dim(h);
    if (N != *ham_dim) {
        oops_ham_destroy(h);
        return oops_set_status(OOPS_ERR_ARG, "ham_dim does not match the spin dimensions");
    }
    if (*w_seq_len < N * *tn) {
        oops_ham_destroy(h);
        return oops_set_status(OOPS_ERR_SIZE, "w_seq_len < ham_dim * tn");
    }
    zd *dv = nullptr, *dw = nullptr;
    cudaStream_t st = cudaStreamPerThread;
    if (cudaMalloc(&dv, N * sizeof(zd)) != cudaSuccess ||
        cudaMalloc(&dw, (*tn ? *tn : 1) * N * sizeof(zd)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dv);
        oops_ham_destroy(h);
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (state vectors)");
    }
    rc = OOPS_OK;
    if (cudaMemcpyAsync(dv, v, N * sizeof(zd), cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = oops_set_status(OOPS_ERR_CUDA, "H2D copy failed");
    if (!rc)
        rc = oops_expv_run(h, dv, 1, *tn, ta, *m, *tol, *k, dw, nullptr, st);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(w_seq, dw, *tn * N * sizeof(zd), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dv);
    cudaFree(dw);
    oops_ham_destroy(h);
    return rc;
}

extern "C" void main_cache_(size_t *nspin, size_t *nTerm, double *coeff_lst, size_t *nbody_lst,
                            size_t *pos_i_idx, size_t *pos_i_lst, size_t *dim_i_lst,
                            size_t *mat_i_idx, oops_zcomplex *mat_i_lst, size_t *ham_dim,
                            size_t *nspin_dim, oops_zcomplex *v, size_t *pos_idx, size_t *mat_idx,
                            size_t *k, size_t *maxThreadsPerBlock, size_t *maxGridSize,
                            size_t *tn, double *ta, size_t *m, double *tol, size_t *itrace,
                            oops_zcomplex *w_seq, size_t *w_seq_len)
{
    (void)pos_idx; (void)mat_idx; (void)maxThreadsPerBlock; (void)maxGridSize; (void)itrace;
    g_drop_status = drop_in(nspin, nTerm, coeff_lst, nbody_lst, pos_i_idx, pos_i_lst, dim_i_lst,
                            mat_i_idx, mat_i_lst, ham_dim, nspin_dim, v, k, tn, ta, m, tol, w_seq,
                            w_seq_len);
    g_drop_msg = g_drop_status ? g_msg : std::string();
}

extern "C" void main_mkl_(size_t *nspin, size_t *nTerm, double *coeff_lst, size_t *nbody_lst,
                          size_t *pos_i_idx, size_t *pos_i_lst, size_t *dim_i_lst,
                          size_t *mat_i_idx, oops_zcomplex *mat_i_lst, size_t *ham_dim,
                          size_t *nspin_dim, oops_zcomplex *v, size_t *pos_idx, size_t *mat_idx,
                          size_t *k, size_t *tn, double *ta, size_t *m, double *tol,
                          size_t *itrace, oops_zcomplex *w_seq, size_t *w_seq_len)
{
    (void)pos_idx; (void)mat_idx; (void)itrace;
    g_drop_status = drop_in(nspin, nTerm, coeff_lst, nbody_lst, pos_i_idx, pos_i_lst, dim_i_lst,
                            mat_i_idx, mat_i_lst, ham_dim, nspin_dim, v, k, tn, ta, m, tol, w_seq,
                            w_seq_len);
    g_drop_msg = g_drop_status ? g_msg : std::string();
}
