/*
 * oops_cce.h -- C-ABI of the batched cluster-correlation-expansion (CCE) path
 * of liboops_gb300.so: cluster coherence on the device, cluster enumeration and
 * the CCE reduction.  Plain C types; device buffers and streams are void* or
 * typed device pointers as documented per call.
 */
#ifndef OOPS_CCE_H
#define OOPS_CCE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical parameters of one CCE run (EnsembleCCE::set_parameters,
 * src/source/app/ensemble_cce.cpp:6-31; NV states from
 * NVCenter::make_espin_hamiltonian, src/source/app/DefectCenter.cpp:32-45). */
typedef struct {
    double B[3];           /* magnetic field (T)                                */
    double center[3];      /* NV electron position (Angstrom)                   */
    double gamma_center;   /* electron gamma (rad s^-1 T^-1), -1.760859708e11  */
    double gamma_bath;     /* bath gamma, 13C 6.728284e7                        */
    double sv0[3];         /* <S> of NV state 0 (conditions H_0)                */
    double sv1[3];         /* <S> of NV state 1 (conditions H_1)                */
    int pulse_num;         /* CPMG pulse count, 1 = Hahn echo (misc.cpp:59-84)  */
    size_t nT;             /* time points t_i = i*dt, i = 0..nT-1               */
    double dt;
    double fp64_below;     /* mixed modes: clusters whose L_C(t) drops below    */
                           /* this value at any t are recomputed in FP64 (the   */
                           /* CCE reduction divides by them); 0 = never          */
    int fp64_max_k;        /* mixed modes: clusters of at most this many spins  */
                           /* run entirely in FP64 (the reduction amplifies     */
                           /* low-order errors most; they are cheap); 0 = none   */
} oops_cce_params;

#define OOPS_PREC_FP64 0        /* every step in FP64                          */
#define OOPS_PREC_MIXED 1       /* FP64 eigenbasis; per-time-point products on   */
                                /* tensor cores (five- and six-spin clusters,    */
                                /* Hahn or even CPMG: FP16 hi/lo, FP32           */
                                /* accumulate) or FP32                           */
#define OOPS_PREC_MIXED_SIMT 2  /* as MIXED, FP32 products on CUDA cores only   */

/* Cluster coherence L_C(t_i) = Re Tr[B1^+ B0]/2^k for ncl clusters of k spin-1/2
 * bath spins (k = 1..6), the Hilbert-space equivalent of the reference's
 * EnsembleCCE::cluster_evolution (src/source/app/ensemble_cce.cpp:33-55,
 * PiecewiseFullMatrixVectorEvolution, QuantumEvolutionAlgorithm.cpp:60-83) at
 * zero bath polarisation and dephasing.  coords_dev: nbath x 3 doubles
 * (device); clusters_dev: ncl x k spin indices (device, uint32); L_dev:
 * ncl x nT doubles (device, cluster-major).  Asynchronous on stream except for
 * a final status read. */
int oops_cce_coherence(const double *coords_dev, size_t nbath,
                       const unsigned *clusters_dev, size_t ncl, int k,
                       const oops_cce_params *p, int precision, double *L_dev,
                       void *stream);

/* Cluster coherence like oops_cce_coherence, but it allocates no device
 * memory: no counterpart in the reference.  For callers that cannot allocate
 * during a run (a host code whose allocator reserved the device memory up
 * front, or a serving loop that must not let cudaMalloc/cudaFree synchronise
 * the device).  Scratch comes from one static 32 MiB device array inside the
 * library, held by every GPU that loads it until exit; batches needing more
 * are rejected with OOPS_ERR_SIZE (FP64 mode with k = 6 always needs more).
 * Mixed precision runs every cluster size on the FP32 CUDA-core kernels
 * (OOPS_PREC_MIXED and OOPS_PREC_MIXED_SIMT are the same here, and results
 * agree with oops_cce_coherence within the mixed-precision tolerance, not
 * bit for bit); fp64_max_k is honoured; fp64_below > 0 with a mixed precision
 * is OOPS_ERR_UNSUPPORTED.  Every call looks the array up on the current
 * device (cudaGetSymbolAddress), reads a failure counter back and
 * synchronises `stream`, so it cannot be captured into a CUDA graph; the
 * first call on a device loads the module and should come before any stream
 * capture on that device.  Calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int oops_cce_coherence_noalloc(const double *coords_dev, size_t nbath,
                               const unsigned *clusters_dev, size_t ncl, int k,
                               const oops_cce_params *p, int precision,
                               double *L_dev, void *stream);

/* Bath terms of the Liouville-space path (EnsembleCCE::set_parameters,
 * src/source/app/ensemble_cce.cpp:16-18): pure dephasing of every bath spin
 * along an axis (create_incoherent_operator, :73-84; SingleSpinDephasing,
 * src/source/spin/SpinInteraction/SpinInteractionComponent.cpp:285-304) and
 * the bath polarisation of the initial state (create_spin_density_state,
 * :94-102). */
typedef struct {
    double dephasing_rate;     /* Hz; multiplied by 2 pi, as the reference does */
    double dephasing_axis[3];  /* normalised here; unused at rate 0            */
    double polarization[3];    /* p: rho0 = I/2^k + sum_s p.S_s                */
} oops_cce_bath;

/* Cluster coherence in Liouville space, the reference's own formulation with
 * bath dephasing and polarisation (EnsembleCCE::cluster_evolution,
 * src/source/app/ensemble_cce.cpp:33-55, 104-113; PiecewiseFullMatrixVector
 * Evolution, QuantumEvolutionAlgorithm.cpp:60-83): L_C(t_i) =
 * Re <2^k rho0, E_n^i ... E_0^i rho0> with the 4^k x 4^k segment propagators
 * E_j of the Liouvillians SHARP(H_a) - FLAT(H_b) + dephasing.  FP64, clusters
 * of k = 1..6 spins (N = 1024 and 4096 at k = 5, 6: ~0.2 and ~10 s of FP64
 * GEMM per cluster, up to ~3.2 GB of scratch per six-spin cluster), pulse_num
 * 1..64; arguments and layouts as
 * oops_cce_coherence (precision is always FP64).  Synchronises `stream` once
 * per chunk of clusters (it reads the scaling exponents of the matrix
 * exponentials) and before returning. */
int oops_cce_coherence_liouville(const double *coords_dev, size_t nbath,
                                 const unsigned *clusters_dev, size_t ncl, int k,
                                 const oops_cce_params *p, const oops_cce_bath *bath,
                                 double *L_dev, void *stream);

/* Single-sample CCE (SingleSampleCCE, src/source/app/single_sample_cce.cpp):
 * the bath in a pure product state, state_dev[j] = 0 (bath spin j up along z)
 * or 1 (down), as prepare_bath_state draws it (:35-46); every cluster spin
 * feels the mean dipolar field of the bath spins outside the cluster
 * (create_spin_hamiltonian, :83-104); L_C(t_i) = Re <psi_1 | psi_2> with
 * psi_a the cluster's basis state propagated through riffle(H_a, H_{1-a})
 * (cluster_evolution and calc_observables, :48-127).  Arguments and layouts
 * as oops_cce_coherence; state_dev: nbath bytes (device).  FP64, or mixed
 * (FP64 eigenbasis, FP32 propagation).  Synchronises `stream` before
 * returning. */
int oops_cce_coherence_state(const double *coords_dev, size_t nbath,
                             const unsigned char *state_dev, const unsigned *clusters_dev,
                             size_t ncl, int k, const oops_cce_params *p, int precision,
                             double *L_dev, void *stream);

/* The bath state prepare_bath_state draws from a seed: srand(seed), then
 * rand() % 2 per bath spin, with glibc's rand() restated (so the states do not
 * depend on the host's C library).  state: nbath bytes (host). */
int oops_bath_state_from_seed(unsigned seed, size_t nbath, unsigned char *state);

/* ------------------------------------------------------------------------
 * Cluster enumeration (host)
 * ---------------------------------------------------------------------- */
typedef struct oops_clusters oops_clusters;

/* All connected clusters of 1..max_order spins of a bath (coords: nspin x 3,
 * Angstrom), as cSpinCollection::getConnectionMatrix + cDepthFirstPathTracing
 * build them (src/source/spin/SpinCollection/SpinCollection.cpp:51-57,
 * src/source/spin/SpinCluster/SpinClusterAlgorithm.cpp:75-148): connected iff
 * distance <= cutoff; clusters of one order in std::set<cClusterIndex> order
 * (SpinClusterIndex.cpp:55-64).  Order o holds clusters of o+1 spins. */
int oops_clusters_enumerate(size_t nspin, const double *coords, double cutoff,
                            int max_order, oops_clusters **out);
/* The same enumeration from a connection matrix instead of coordinates, as
 * cDepthFirstPathTracing(connection_matrix, max_order) takes it
 * (SpinClusterAlgorithm.cpp:75-111): row_off (nspin+1 entries) and cols hold
 * each spin's connected spins (CSR, any order); the diagonal is ignored and
 * the matrix must be symmetric (OOPS_ERR_ARG otherwise). */
int oops_clusters_enumerate_graph(size_t nspin, const size_t *row_off, const unsigned *cols,
                                  int max_order, oops_clusters **out);
int oops_clusters_destroy(oops_clusters *c);
size_t oops_clusters_count(const oops_clusters *c, int order);
/* sorted spin indices of every cluster of one order: count x (order+1) */
int oops_clusters_indices(const oops_clusters *c, int order, unsigned *out);
/* cSpinCluster::getSubClusters (src/source/spin/SpinCluster/SpinCluster.cpp:
 * 82-98) for every cluster of one order, as CSR: offsets (count+1 entries) and
 * (order, position) pairs in std::set<pair> order. */
size_t oops_clusters_subcluster_total(const oops_clusters *c, int order);
int oops_clusters_subclusters(const oops_clusters *c, int order, size_t *offsets,
                              unsigned *pairs);

/* NV electron: eigenvalues (ascending) and <S> of each eigenstate for field B
 * (NVCenter::make_espin_hamiltonian, src/source/app/DefectCenter.cpp:32-45;
 * cSPIN::get_spin_vector, src/source/spin/Spin/Spin.cpp:88-95).
 * svec[3*i + a]. */
int oops_nv_states(const double *B, double *evals, double *svec);

/* The CCE reduction on device data (CCE::cce_coherence_reduction and
 * compuate_final_coherence, src/source/app/cce.cpp:151-189).  Host arrays of
 * max_order device pointers: Lraw_dev[o] / til_dev[o] (counts[o] x nT,
 * cluster-major), off_dev[o] (counts[o]+1, uint64) and pairs_dev[o] (closure
 * (order, position) pairs, uint32) as oops_clusters_subclusters returns them.
 * each_dev / cum_dev: nT x max_order column-major (device).  The per-order
 * products are accumulated in FP64 as (mantissa, binary exponent) pairs, in a
 * fixed order. */
int oops_cce_reduce(int max_order, const size_t *counts, size_t nT,
                    const double *const *Lraw_dev, double *const *til_dev,
                    const unsigned long long *const *off_dev,
                    const unsigned *const *pairs_dev, double *each_dev,
                    double *cum_dev, void *stream);

/* ------------------------------------------------------------------------
 * Whole ensemble-CCE run (EnsembleCCE on one GPU)
 * ---------------------------------------------------------------------- */
/* Enumerate the bath's clusters up to max_order spins (max_order <= 6),
 * compute every cluster's coherence on the device, reduce them
 * (CCE::cce_coherence_reduction / compuate_final_coherence,
 * src/source/app/cce.cpp:151-189) and return, column-major nT x max_order,
 * final_cum (_final_result: product up to each order) and final_each
 * (_final_result_each_order; may be NULL).  counts_out (max_order entries,
 * may be NULL) receives the cluster count per order; cluster_L (may be NULL)
 * the raw L_C(t) of every cluster, order by order, cluster-major. */
int oops_ensemble_cce(size_t nbath, const double *coords, double cutoff,
                      int max_order, const oops_cce_params *p, int precision,
                      double *final_cum, double *final_each, size_t *counts_out,
                      double *cluster_L, size_t cluster_L_len, void *stream);

/* oops_ensemble_cce keeps, per calling thread, one run plan for its
 * Hilbert-space runs (FP64 or mixed without fp64_below): device buffers sized
 * for the run's shape and the run captured as a CUDA graph, keyed on the
 * cluster counts, closure sizes, parameters, precision and device.  A call
 * with a matching key uploads all its inputs into the plan and replays every
 * kernel; any other call rebuilds the plan.  This frees the calling thread's
 * plan (device memory ~ clusters x nT x 16 bytes). */
int oops_cce_release_plans(void);

/* The same run in Liouville space with bath dephasing and polarisation (the
 * reference's EnsembleCCE as its EnsNVeBath / EnsNVLattice applications run it
 * by default: 1e4 Hz along (1,1,1), src/application/EnsNVeBath.cpp:133-135),
 * every cluster through oops_cce_coherence_liouville; max_order 1..6, FP64. */
int oops_ensemble_cce_bath(size_t nbath, const double *coords, double cutoff,
                           int max_order, const oops_cce_params *p,
                           const oops_cce_bath *bath, double *final_cum,
                           double *final_each, size_t *counts_out, double *cluster_L,
                           size_t cluster_L_len, void *stream);

/* Whole single-sample CCE run with host buffers (SingleSampleCCE and the CCE
 * reduction it inherits): arguments as oops_ensemble_cce plus the bath state
 * (nbath bytes, host; oops_bath_state_from_seed draws the reference's). */
int oops_single_sample_cce(size_t nbath, const double *coords, const unsigned char *state,
                           double cutoff, int max_order, const oops_cce_params *p,
                           int precision, double *final_cum, double *final_each,
                           size_t *counts_out, double *cluster_L, size_t cluster_L_len,
                           void *stream);

/* The single-sample run on device-resident data: arguments as
 * oops_ensemble_cce_device plus the bath state (nbath bytes, device); the
 * size classes run concurrently on forked streams, one synchronisation. */
int oops_single_sample_cce_device(const double *coords_dev, size_t nbath,
                                  const unsigned char *state_dev, int max_order,
                                  const size_t *counts, const unsigned *const *clusters_dev,
                                  const oops_cce_params *p, int precision,
                                  double *const *Lraw_dev, double *const *til_dev,
                                  const unsigned long long *const *off_dev,
                                  const unsigned *const *pairs_dev, double *each_dev,
                                  double *cum_dev, void *stream);

/* The same run on device-resident data (the serving and benchmark form):
 * bath coordinates, per-order cluster index lists (clusters_dev[o]: counts[o]
 * x (o+1) uint32) and closures (off_dev / pairs_dev as oops_cce_reduce takes
 * them) already in device memory.  Every cluster size runs on its own stream
 * forked from `stream`, then the reduction on `stream`; Lraw_dev[o] /
 * til_dev[o] (counts[o] x nT) receive the raw and reduced cluster curves,
 * each_dev / cum_dev the final curves.  Returns after one synchronisation of
 * `stream`.  Replaces the same call chain as oops_ensemble_cce minus the
 * enumeration (EnsembleCCE::run_each_clusters + post_treatment,
 * src/source/app/cce.cpp:55-80). */
int oops_ensemble_cce_device(const double *coords_dev, size_t nbath, int max_order,
                             const size_t *counts, const unsigned *const *clusters_dev,
                             const oops_cce_params *p, int precision,
                             double *const *Lraw_dev, double *const *til_dev,
                             const unsigned long long *const *off_dev,
                             const unsigned *const *pairs_dev, double *each_dev,
                             double *cum_dev, void *stream);

/* The device-resident run captured once into a CUDA graph and replayed (no
 * counterpart in the reference, which launches nothing per cluster batch).
 * Create with the arguments of oops_ensemble_cce_device; the device buffers
 * must stay allocated and keep their addresses while the graph exists (their
 * contents may change between launches).  Each launch enqueues the whole run
 * (all size classes, the reduction) on `stream` as one graph launch, then
 * waits for it and checks the error flags.  Launches of one graph must not
 * overlap.  fp64_below > 0 in mixed precision is OOPS_ERR_UNSUPPORTED here
 * (its selection reads flags on the host between kernels). */
typedef struct oops_cce_graph oops_cce_graph;
int oops_cce_graph_create(const double *coords_dev, size_t nbath, int max_order,
                          const size_t *counts, const unsigned *const *clusters_dev,
                          const oops_cce_params *p, int precision,
                          double *const *Lraw_dev, double *const *til_dev,
                          const unsigned long long *const *off_dev,
                          const unsigned *const *pairs_dev, double *each_dev,
                          double *cum_dev, oops_cce_graph **out);
int oops_cce_graph_launch(oops_cce_graph *g, void *stream);
int oops_cce_graph_destroy(oops_cce_graph *g);

/* ------------------------------------------------------------------------
 * Result file
 * ---------------------------------------------------------------------- */
/* Write a run's results as a Level 5 MAT-file with the variables
 * CCE::export_mat_file stores (src/source/app/cce.cpp:191-234), without
 * MATLAB's libraries: CCE<o> and CCE<o>_tilder (nT x counts[o], the raw and
 * reduced cluster curves; host arrays, column = cluster, i.e. the
 * cluster-major layout of oops_ensemble_cce's cluster_L), final_result_each_order
 * and final_result (nT x max_order, column-major), time_list (nT x 1); all
 * flagged global as matPutVariableAsGlobal does.  cluster_L / cluster_til
 * may be NULL to leave those variables out. */
int oops_cce_export_mat(const char *path, int max_order, size_t nT, const size_t *counts,
                        const double *const *cluster_L, const double *const *cluster_til,
                        const double *final_each, const double *final_cum,
                        const double *time_list);

/* ------------------------------------------------------------------------
 * Launch tuning (the counterpart of the reference's launch geometry,
 * get_grid.cu:43-125, which derives grid sizes from the device limits)
 * ---------------------------------------------------------------------- */
/* Per device (the current one) and cluster size k = 1..6: value 0 restores
 * the built-in default, 1..64 overrides it.  The values change launch shapes
 * only, never results.  oops_gb300/tune.py measures candidates and keeps the
 * winners in an on-disk cache keyed by device and workload shape. */
#define OOPS_TUNE_EIG_PER_SM 0   /* eigensolver CTAs per SM                   */
#define OOPS_TUNE_COH_PER_SM 1   /* block coherence kernel CTAs per SM        */
#define OOPS_TUNE_TSLICE_MULT 2  /* time slices: about sms * value work items */
#define OOPS_TUNE_NPARAM 3
int oops_tune_set(int param, int k, int value);
/* the value in effect (the default when unset) */
int oops_tune_get(int param, int k, int *value);

/* ------------------------------------------------------------------------
 * Measurement hooks (no counterpart in the reference)
 * ---------------------------------------------------------------------- */
/* Turn on (1) or off (0) CUDA-event timing of the per-time-point coherence
 * kernel, per cluster size k, and reset the counters. */
int oops_profile_enable(int on);
/* Accumulated kernel time (ms), launch count and algorithmic flop count of
 * the coherence kernel for clusters of k spins since the last enable. */
int oops_profile_read(int k, double *ms_total, long *launches, double *flop);
/* Accumulated time (ms) and count of the eigensolver phase for clusters of
 * k spins since the last enable: Hamiltonian assembly and diagonalisation,
 * overlaps and phase steps, from the first to the last of those launches. */
int oops_profile_read_eig(int k, double *ms_total, long *launches);
/* Clusters of k spins recomputed in FP64 (fp64_below) since the last enable. */
int oops_profile_corrected(int k, long *count);
/* Liouville path (oops_cce_coherence_liouville), clusters of k spins, since the
 * last enable: accumulated time (ms, CUDA events; only while profiling is on),
 * kernel launches and FP64 flop of one phase -- 0 the matrix exponentials
 * and binary powers (batched FP64 GEMMs), 1 the outer-segment recurrences,
 * 2 the middle-segment passes. */
int oops_profile_liouville(int k, int phase, double *ms, long *launches, double *flop);
/* Kernels launched by the Liouville path since the last enable (counted
 * whether or not profiling is on). */
long oops_liouville_launches(void);

#ifdef __cplusplus
}
#endif
#endif
