// oops_internal.h -- declarations shared between the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include "oops_common.cuh"

bool oops_ham_is_zero(const oops_ham *h);

// Krylov driver state kept on a Hamiltonian handle (expv.cu): workspace
// buffers, the norm estimate and the captured integration step.  A handle's
// expv calls must not overlap.
struct oops_expv_cache;
oops_expv_cache *&oops_ham_expv_cache(const oops_ham *h);
void oops_expv_cache_free(oops_expv_cache *c);

// y = alpha * H x on a block with pitch 2^pitch_log2 (nvec <= pitch live
// columns, optional per-column live mask).  Launches on st, no sync.
int oops_ham_apply_internal(const oops_ham *h, zd alpha, const zd *x, zd *y, size_t nvec,
                            int pitch_log2, const int *live, cudaStream_t st);

#include "oops_cce.h"
// sync: wait for the stream and report CUDA errors before returning
int oops_cce_reduce_device(int max_order, const size_t *counts, int nT,
                           const double *const *Lraw, double *const *til,
                           const unsigned long long *const *off, const unsigned *const *pairs,
                           double *each_dev, double *cum_dev, cudaStream_t st, bool sync);

// oops_cce_coherence with optional caller-owned counters (8 zeroed device
// ints): with them the call only enqueues work and the caller checks
// ext_ctr[3] (eigensolver failure) and ext_ctr[5] (tensor-core status) after
// synchronising the stream.
int oops_cce_coherence_enqueue(const double *coords_dev, size_t nbath,
                               const unsigned *clusters_dev, size_t ncl, int k,
                               const oops_cce_params *p, int precision, double *L_dev,
                               void *stream, int *ext_ctr);

// oops_cce_coherence_state with optional caller-owned counters (as above:
// with them the call only enqueues; the caller checks ext_ctr[3])
int oops_cce_coherence_state_enqueue(const double *coords_dev, size_t nbath,
                                     const unsigned char *state_dev, const unsigned *clusters_dev,
                                     size_t ncl, int k, const oops_cce_params *p, int precision,
                                     double *L_dev, void *stream, int *ext_ctr);

bool oops_tc64_supported(int pulse_num);
// phi: per cluster the phase advance per time step of every eigenvalue as a
// 64-bit fixed-point fraction of a turn, [cluster][branch][h, f][D]
// M32: the overlap matrices M = V0^H V1 in FP32, D x D per cluster (tc64:
// six-spin clusters, D = 64; tc32: five-spin clusters, D = 32)
int oops_coherence_tc64(const unsigned long long *phi, const float2 *M32, int ncl, int pulse_num,
                        int nT, double *L, int *queue, int *status, int tslice_mult, cudaStream_t st);
int oops_coherence_tc32(const unsigned long long *phi, const float2 *M32, int ncl, int pulse_num,
                        int nT, double *L, int *queue, int *status, int tslice_mult, cudaStream_t st);

// Coherence-kernel timing events (opt-in profiling).  Recorded around each
// coherence launch; resolved when the counters are read.  A thread-local sink
// collects them instead while a run is being captured into a CUDA graph (the
// graph's launches then resolve them after every replay).
#include <vector>
struct oops_prof_event {
    cudaEvent_t ev0, ev1;
    int k;
    double flop;
};
bool oops_prof_enabled();
void oops_prof_set_sink(std::vector<oops_prof_event> *sink);
void oops_prof_accumulate(const oops_prof_event &e, float ms);
// Liouville-path phase timers (cce_liouville.cu), cleared with the others
void oops_prof_reset_liouville();
