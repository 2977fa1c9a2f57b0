// cce_reduce.cu -- the CCE reduction and the whole ensemble-CCE run.
//
// Reduction (CCE::cce_coherence_reduction / compuate_final_coherence,
// src/source/app/cce.cpp:151-189):
//   Ltilde_C(t) = L_C(t) / prod_{S in closure(C)} Ltilde_S(t)   (divisions in
//                 the closure's set order, as the reference loop does)
//   each(t, o)  = prod_C Ltilde_C(t) over the clusters of order o
//   cum(t, o)   = prod_{o' <= o} each(t, o')
// The per-order product of thousands of near-1 factors is accumulated in FP64
// in the log domain (sum of log|x|, count of negative and zero factors) with a
// fixed-order two-level reduction, so the result is deterministic.
//
// oops_ensemble_cce is the EnsembleCCE run (CCE::set_bath_cluster,
// run_each_clusters, post_treatment; cce.cpp:42-80) on one GPU: enumeration on
// the host (clusters.cpp), every cluster's coherence on the device per size
// class (cce_dense.cu), reduction on the device, final curves to the host.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "oops_cce.h"
#include "oops_common.cuh"
#include "oops_internal.h"

namespace {

__global__ void k_tilde(const double *__restrict__ Lraw, int n, int nT,
                        const unsigned long long *__restrict__ off,
                        const unsigned *__restrict__ pairs, const double *const *__restrict__ til,
                        double *__restrict__ out)
{
    size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (size_t)n * nT) return;
    const int j = (int)(g / nT), t = (int)(g % nT);
    double r = Lraw[g];
    for (unsigned long long s = off[j]; s < off[j + 1]; ++s) {
        const unsigned o = pairs[2 * s], p = pairs[2 * s + 1];
        r = r / til[o][(size_t)p * nT + t];
    }
    out[g] = r;
}

struct LogAcc {
    double lsum;
    int neg, zero;
};

// partial[blk][t] over clusters [blk*chunk, (blk+1)*chunk)
__global__ void k_logprod_partial(const double *__restrict__ til, int n, int nT, int chunk,
                                  LogAcc *__restrict__ partial)
{
    const int t = blockIdx.y * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    const int j0 = blockIdx.x * chunk, j1 = min(n, j0 + chunk);
    LogAcc a = {0.0, 0, 0};
    for (int j = j0; j < j1; ++j) {
        const double x = til[(size_t)j * nT + t];
        if (x == 0.0) a.zero++;
        else {
            if (x < 0) a.neg++;
            a.lsum += log(fabs(x));
        }
    }
    partial[(size_t)blockIdx.x * nT + t] = a;
}

__global__ void k_logprod_final(const LogAcc *__restrict__ partial, int nblk, int nT, int order,
                                int max_order, double *__restrict__ each, double *__restrict__ cum,
                                double *__restrict__ cumlog)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    LogAcc a = {0.0, 0, 0};
    for (int b = 0; b < nblk; ++b) {
        LogAcc p = partial[(size_t)b * nT + t];
        a.lsum += p.lsum;
        a.neg += p.neg;
        a.zero += p.zero;
    }
    double v = a.zero ? 0.0 : ((a.neg & 1) ? -exp(a.lsum) : exp(a.lsum));
    // column-major (nT x max_order), as the reference's _final_result matrices
    each[(size_t)order * nT + t] = v;
    // running product across orders, kept as (log, sign) in cumlog[2*t..]
    double l = cumlog[2 * t] + (a.zero ? 0.0 : a.lsum);
    double sgn = cumlog[2 * t + 1] * ((a.neg & 1) ? -1.0 : 1.0) * (a.zero ? 0.0 : 1.0);
    cumlog[2 * t] = l;
    cumlog[2 * t + 1] = sgn;
    cum[(size_t)order * nT + t] = sgn == 0.0 ? 0.0 : sgn * exp(l);
}

__global__ void k_init_cumlog(double *cumlog, int nT)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nT) {
        cumlog[2 * t] = 0.0;
        cumlog[2 * t + 1] = 1.0;
    }
}

}  // namespace

// Reduction on device data: Lraw[o] / til[o] are count_o x nT (cluster-major,
// device); off[o] (count_o+1) and pairs[o] (2*total) the closure CSR (device).
int oops_cce_reduce_device(int max_order, const size_t *counts, int nT,
                           const double *const *Lraw, double *const *til,
                           const unsigned long long *const *off, const unsigned *const *pairs,
                           double *each_dev, double *cum_dev, cudaStream_t st)
{
    double **til_dev = nullptr;
    double *cumlog = nullptr;
    LogAcc *partial = nullptr;
    const int chunk = 16;
    size_t maxn = 1;
    for (int o = 0; o < max_order; ++o) maxn = std::max(maxn, counts[o]);
    const int maxblk = (int)((maxn + chunk - 1) / chunk);
    if (cudaMallocAsync((void **)&til_dev, max_order * sizeof(double *), st) != cudaSuccess ||
        cudaMallocAsync((void **)&cumlog, 2 * (size_t)nT * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&partial, (size_t)maxblk * nT * sizeof(LogAcc), st) != cudaSuccess) {
        cudaGetLastError();
        if (til_dev) cudaFreeAsync(til_dev, st);
        if (cumlog) cudaFreeAsync(cumlog, st);
        if (partial) cudaFreeAsync(partial, st);
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (reduction)");
    }
    cudaMemcpyAsync(til_dev, til, max_order * sizeof(double *), cudaMemcpyHostToDevice, st);
    k_init_cumlog<<<(nT + 255) / 256, 256, 0, st>>>(cumlog, nT);
    for (int o = 0; o < max_order; ++o) {
        const int n = (int)counts[o];
        if (n > 0) {
            size_t tot = (size_t)n * nT;
            k_tilde<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(Lraw[o], n, nT, off[o], pairs[o],
                                                                  til_dev, til[o]);
        }
        const int nblk = std::max(1, (n + chunk - 1) / chunk);
        dim3 g(nblk, (nT + 127) / 128);
        k_logprod_partial<<<g, 128, 0, st>>>(til[o], n, nT, chunk, partial);
        k_logprod_final<<<(nT + 127) / 128, 128, 0, st>>>(partial, nblk, nT, o, max_order, each_dev,
                                                        cum_dev, cumlog);
    }
    cudaFreeAsync(til_dev, st);
    cudaFreeAsync(cumlog, st);
    cudaFreeAsync(partial, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    return OOPS_OK;
}

extern "C" int oops_cce_reduce(int max_order, const size_t *counts, size_t nT,
                               const double *const *Lraw_dev, double *const *til_dev,
                               const unsigned long long *const *off_dev,
                               const unsigned *const *pairs_dev, double *each_dev, double *cum_dev,
                               void *stream)
{
    if (max_order < 1 || !counts || !Lraw_dev || !til_dev || !off_dev || !pairs_dev || !each_dev ||
        !cum_dev)
        return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    return oops_cce_reduce_device(max_order, counts, (int)nT, Lraw_dev, til_dev, off_dev, pairs_dev,
                                  each_dev, cum_dev, (cudaStream_t)stream);
}

extern "C" int oops_ensemble_cce(size_t nbath, const double *coords, double cutoff,
                                 int max_order, const oops_cce_params *p, int precision,
                                 double *final_cum, double *final_each, size_t *counts_out,
                                 double *cluster_L, size_t cluster_L_len, void *stream)
{
    if (!coords || !p || !final_cum || max_order < 1 || max_order > 6)
        return oops_set_status(OOPS_ERR_ARG, "bad arguments (max_order must be 1..6)");
    cudaStream_t st = (cudaStream_t)stream;
    oops_clusters *cl = nullptr;
    int rc = oops_clusters_enumerate(nbath, coords, cutoff, max_order, &cl);
    if (rc) return rc;
    const int nT = (int)p->nT;
    std::vector<size_t> counts(max_order);
    size_t total_cl = 0;
    for (int o = 0; o < max_order; ++o) {
        counts[o] = oops_clusters_count(cl, o);
        total_cl += counts[o];
        if (counts_out) counts_out[o] = counts[o];
    }
    double *dcoords = nullptr, *dL = nullptr, *dT = nullptr, *each = nullptr, *cum = nullptr;
    unsigned *didx = nullptr, *dpairs = nullptr;
    unsigned long long *doff = nullptr;
    size_t idx_total = 0, pair_total = 0, off_total = 0;
    for (int o = 0; o < max_order; ++o) {
        idx_total += counts[o] * (o + 1);
        pair_total += 2 * oops_clusters_subcluster_total(cl, o);
        off_total += counts[o] + 1;
    }
    auto cleanup = [&]() {
        if (dcoords) cudaFreeAsync(dcoords, st);
        if (dL) cudaFreeAsync(dL, st);
        if (dT) cudaFreeAsync(dT, st);
        if (each) cudaFreeAsync(each, st);
        if (cum) cudaFreeAsync(cum, st);
        if (didx) cudaFreeAsync(didx, st);
        if (dpairs) cudaFreeAsync(dpairs, st);
        if (doff) cudaFreeAsync(doff, st);
        cudaStreamSynchronize(st);
        oops_clusters_destroy(cl);
    };
    if (cudaMallocAsync((void **)&dcoords, (nbath ? nbath : 1) * 3 * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&dL, (total_cl ? total_cl : 1) * nT * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&dT, (total_cl ? total_cl : 1) * nT * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&each, (size_t)max_order * nT * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&cum, (size_t)max_order * nT * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&didx, (idx_total ? idx_total : 1) * sizeof(unsigned), st) != cudaSuccess ||
        cudaMallocAsync((void **)&dpairs, (pair_total ? pair_total : 1) * sizeof(unsigned), st) != cudaSuccess ||
        cudaMallocAsync((void **)&doff, off_total * sizeof(unsigned long long), st) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (ensemble CCE)");
    }
    // host staging of indices and closures (pinned by the caller's choice; plain here)
    std::vector<unsigned> hidx(idx_total ? idx_total : 1), hpairs(pair_total ? pair_total : 1);
    std::vector<unsigned long long> hoff(off_total);
    std::vector<const double *> Lraw(max_order);
    std::vector<double *> til(max_order);
    std::vector<const unsigned long long *> offp(max_order);
    std::vector<const unsigned *> pairp(max_order);
    std::vector<const unsigned *> idxp(max_order);
    size_t io = 0, po = 0, oo = 0, lo = 0;
    for (int o = 0; o < max_order; ++o) {
        oops_clusters_indices(cl, o, hidx.data() + io);
        std::vector<size_t> offs(counts[o] + 1);
        oops_clusters_subclusters(cl, o, offs.data(), hpairs.data() + po);
        for (size_t q = 0; q <= counts[o]; ++q) hoff[oo + q] = offs[q];
        idxp[o] = didx + io;
        pairp[o] = dpairs + po;
        offp[o] = doff + oo;
        Lraw[o] = dL + lo;
        til[o] = dT + lo;
        io += counts[o] * (o + 1);
        po += 2 * oops_clusters_subcluster_total(cl, o);
        oo += counts[o] + 1;
        lo += counts[o] * nT;
    }
    cudaMemcpyAsync(dcoords, coords, nbath * 3 * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(didx, hidx.data(), idx_total * sizeof(unsigned), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dpairs, hpairs.data(), pair_total * sizeof(unsigned), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(doff, hoff.data(), off_total * sizeof(unsigned long long), cudaMemcpyHostToDevice, st);
    for (int o = 0; o < max_order && !rc; ++o)
        if (counts[o])
            rc = oops_cce_coherence(dcoords, nbath, idxp[o], counts[o], o + 1, p, precision,
                                    const_cast<double *>(Lraw[o]), st);
    if (!rc)
        rc = oops_cce_reduce_device(max_order, counts.data(), nT, Lraw.data(), til.data(),
                                    offp.data(), pairp.data(), each, cum, st);
    if (!rc) {
        cudaMemcpyAsync(final_cum, cum, (size_t)max_order * nT * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (final_each)
            cudaMemcpyAsync(final_each, each, (size_t)max_order * nT * sizeof(double),
                            cudaMemcpyDeviceToHost, st);
        if (cluster_L) {
            if (cluster_L_len < total_cl * nT) rc = oops_set_status(OOPS_ERR_SIZE, "cluster_L too small");
            else cudaMemcpyAsync(cluster_L, dL, total_cl * nT * sizeof(double), cudaMemcpyDeviceToHost, st);
        }
        cudaError_t e = cudaStreamSynchronize(st);
        if (!rc && e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    }
    cleanup();
    return rc;
}
