/*
 * oracle.h -- CPU restatement of the nzhao/oops CCE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may load
 * it.  The product (oops_gb300/) never links, loads or calls it.
 *
 * Parity status: the reference ships no golden vectors or known-answer
 * tests, and its application does not build as shipped (Fortran Krylov and
 * Pade drivers, MKL, armadillo, boost, MPI, MATLAB).  oracle/build_ref.sh
 * compiles the reference's own C++ sources for this path with the
 * stand-ins of oracle/ref_shim (armadillo, boost's variables_map, MPI, the
 * XML reader, logging, a recording mat.h) into oracle/_ref, and the
 * fixtures their outputs give (tests/golden/, with the scripts that made
 * them) pin this restatement on the reference's own code: the Kronecker
 * matvec (hamvec_func3.cpp) bit for bit; the cluster enumeration and
 * closures, dipole tensors, Zeeman terms and CPMG intervals bit for bit;
 * the CCE reduction (cce.cpp) bit for bit; whole EnsembleCCE runs in
 * Liouville space with dephasing and polarisation (2e-13) and in the
 * Hilbert form (7.3e-11); whole SingleSampleCCE runs (2e-12); the term
 * lists MatExpVector hands main_mkl_ (bit for bit, coefficients to 4e-15).
 * UNPINNED on the reference's code: the Fortran Krylov driver (ZGEXPV) and
 * Pade exponential (ZGPADM), for which there is no compiler here; the
 * restatements of those are pinned against scipy.linalg.expm and
 * expm_multiply, and the generator against a big-integer restatement of
 * LAPACK's DLARAN.
 *
 * Every function cites the reference file:line it restates.  Complex numbers
 * are C99 double _Complex laid out as (re, im) pairs, identical to
 * std::complex<double> and Fortran COMPLEX*16.
 */
#ifndef OOPS_ORACLE_H
#define OOPS_ORACLE_H

#include <stddef.h>
#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex orc_z;

/* ---- random numbers ---------------------------------------------------- */
/* LAPACK DLARAN, src/expv/source/expokit/DLARAN.f:3-92: 48-bit multiplicative
 * congruential generator, multiplier 33952834046453, returns seed/2^48. */
double orc_dlaran(int iseed[4]);

/* ---- Kronecker matvec -------------------------------------------------- */
/* kron_func_v3, src/expv/source/hamvec_func3.cpp:73-100: in-place
 * x <- (I_m (x) A_s (x) I_n) x, A column-major s x s. */
void orc_kron_mode(size_t m, size_t s, size_t n, const orc_z *A, orc_z *x);

/* hamvec_func3, src/expv/source/hamvec_func3.cpp:307-389:
 * w = sum_t coeff[t] * (x)_b mat_{t,b} v, bodies applied last-to-first. */
void orc_hamvec(size_t nspin, size_t nterm, const orc_z *coeff,
                const size_t *nbody_lst, const size_t *pos_i_idx,
                const size_t *pos_i_lst, const size_t *dim_i_lst,
                const size_t *mat_i_idx, const orc_z *mat_i_lst, size_t vlen,
                const size_t *nspin_dim, const orc_z *v, orc_z *w, orc_z *w_med);

/* ---- Pade exponential --------------------------------------------------- */
/* ZGPADM, src/expv/source/expokit/expokit.f:762-933 (Sidje, ACM TOMS 24(1)
 * 1998): E = exp(t*H) by the irreducible (ideg,ideg) Pade form plus
 * scaling-and-squaring.  H is m x m column-major with leading dim ldh.
 * Returns 0, or -1 for a null H (the reference stops), -2 for a singular
 * denominator (the reference stops in ZGESV). */
int orc_padm(int ideg, int m, double t, const orc_z *H, int ldh, orc_z *E,
             int *ns);

/* ---- Krylov expv driver ------------------------------------------------- */
typedef struct {
    double anorm;      /* Lanczos + power-iteration norm estimate          */
    long   nmult;      /* matvecs in the integration (iwsp(1))             */
    long   nexph;      /* Hessenberg exponentials (iwsp(2))                */
    long   nscale;     /* squarings (iwsp(3))                              */
    long   nstep;      /* integration steps (iwsp(4))                      */
    long   nreject;    /* rejected steps (iwsp(5))                         */
    long   ibrkflag;   /* happy breakdown seen (iwsp(6))                   */
    long   mbrkdwn;    /* basis size at breakdown (iwsp(7))                */
    double step_min, step_max, x_error, s_error, hump, tbrkdwn, t_now;
    int    iflag;      /* 0 ok, <0 bad sizes, 3 reject/iteration cap hit   */
} orc_expv_stats;

/* MAIN_MKL + HAMVEC_ZGEXPV_W_MKL_PROFILE, src/expv/source/main_mkl.f:1-130
 * and src/expv/source/hamvec_zgexpv_w_mkl_profile.f:186-538.
 * w_seq(:, tt) = exp(-i H ta[tt]) v for every tt, H = sum coeff[t] (x) mats.
 * Arguments mirror main_mkl_ (src/expv/include/main_mkl.h:6) by value.
 * Deliberate, documented deviations from the Fortran:
 *   - sgn is +1 (the Fortran reads an uninitialised t, zgexpv:396);
 *   - the DLARAN seed restarts at (0,0,0,5) on every call (the Fortran SAVEs
 *     it across calls, zgexpv:210);
 *   - power iteration and step rejection carry iteration caps (iflag = 3). */
int orc_expv(size_t nspin, size_t nterm, const double *coeff_lst,
             const size_t *nbody_lst, const size_t *pos_i_idx,
             const size_t *pos_i_lst, const size_t *dim_i_lst,
             const size_t *mat_i_idx, const orc_z *mat_i_lst, size_t ham_dim,
             const size_t *nspin_dim, const orc_z *v, size_t klim, size_t tn,
             const double *ta, size_t m, double tol, orc_z *w_seq,
             orc_expv_stats *stats);

/* Same driver, but exp(-i H ta) applied to every column of V (ham_dim x nvec,
 * column-major) with a per-column time list ta (tn x nvec, column-major).
 * anorm is estimated once (as orc_expv does) and shared by all columns.
 * Used for cluster propagation: one column per basis state. */
int orc_expv_block(size_t nspin, size_t nterm, const double *coeff_lst,
                   const size_t *nbody_lst, const size_t *pos_i_idx,
                   const size_t *pos_i_lst, const size_t *dim_i_lst,
                   const size_t *mat_i_idx, const orc_z *mat_i_lst,
                   size_t ham_dim, const size_t *nspin_dim, const orc_z *V,
                   size_t nvec, size_t klim, size_t tn, const double *ta,
                   size_t m, double tol, orc_z *W_seq);

/* ---- spin physics ------------------------------------------------------- */
/* dipole(), src/source/misc/misc.cpp:11-36: 9 coefficients (row-major 3x3)
 * hbar mu0/4pi g1 g2 / r^3 (delta_ab - 3 n_a n_b), r in Angstrom. */
void orc_dipole(const double c1[3], const double c2[3], double g1, double g2,
                double out9[9]);

/* NVCenter::make_espin_hamiltonian, src/source/app/DefectCenter.cpp:32-45 +
 * cSPIN::get_spin_vector, src/source/spin/Spin/Spin.cpp:88-95: eigenvalues of
 * the spin-1 NV Hamiltonian in ascending order and <S> of each eigenstate
 * (svec[3*i + a], a = x,y,z). */
void orc_nv_states(const double B[3], double eval[3], double svec[9]);

/* EnsembleCCE::create_spin_hamiltonian, src/source/app/ensemble_cce.cpp:57-71,
 * flattened like MatExpVector::runInexplicit, src/source/math/MatExp.cpp:
 * 216-270.  Spin-1/2 bath of k spins at coords (k x 3, Angstrom), bath gamma
 * g, field B (T), centre spin at cc with gamma gc and spin vector sv.
 * Terms: dipolar pairs (i<j, xx..zz), Zeeman (x,y,z per spin), hyperfine
 * field (x,y,z per spin), zero coefficients skipped (SpinInteraction.cpp:58).
 * Arrays must hold 9k(k-1)/2 + 12k terms; returns nterm.  pos_i_idx has
 * nterm+1 entries; matC holds 4 complex entries per body. */
size_t orc_cluster_hamiltonian(size_t k, const double *coords, double g,
                               const double B[3], const double cc[3], double gc,
                               const double sv[3], double *coeff,
                               size_t *nbody, size_t *pos_i_idx,
                               size_t *pos_list, size_t *dim_list,
                               size_t *mat_offset, orc_z *matC);

/* Dense Hamiltonian matrix (D x D column-major) of a flattened term list,
 * i.e. SumKronProd::full(), src/source/kron/KronProd.cpp:60-66,150-156. */
void orc_dense_hamiltonian(size_t nspin, size_t nterm, const double *coeff,
                           const size_t *nbody, const size_t *pos_i_idx,
                           const size_t *pos_list, const size_t *dim_list,
                           const size_t *mat_offset, const orc_z *matC,
                           const size_t *spin_dim, orc_z *Hout);

/* Pulse_Interval for CPMG, src/source/misc/misc.cpp:59-84. Writes n+1
 * fractions. */
void orc_cpmg_intervals(int n, double *frac);

/* Coherence of one cluster, Hilbert-space form:
 * L(t_i) = Re Tr[B1(t_i)^+ B0(t_i)] / D with B0 = U0(s0 t) U1(s1 t) U0(s2 t)..
 * and B1 the same with 0 <-> 1, U_a(tau) = exp(-i H_a tau) (the segment order
 * of riffle(), src/include/misc/misc.h:25-40).  Equal to the reference's
 * Liouville-space observable (ensemble_cce.cpp:33-55,104-113) at zero bath
 * polarisation and zero dephasing.  Dense propagators U_j^i built as in
 * PiecewiseFullMatrixVectorEvolution::perform,
 * src/source/quantum/QuantumEvolution/QuantumEvolutionAlgorithm.cpp:60-83:
 * t_i = i*dt, dt = t[1]-t[0], Pade per segment, then one product per step. */
void orc_coherence_hilbert(size_t D, const orc_z *H0, const orc_z *H1,
                           int pulse_num, size_t nT, double dt, double *L);

/* Single-sample CCE observable (SingleSampleCCE, single_sample_cce.cpp:48-127):
 * the basis state e_b propagated through riffle(H0, H1) and riffle(H1, H0)
 * with PiecewiseFullMatrixVectorEvolution's powers; L_i = Re <state1, state2>. */
void orc_coherence_state(size_t D, const orc_z *H0, const orc_z *H1, int pulse_num,
                         size_t nT, double dt, size_t b, double *L);

/* Same observable, reference's own Liouville-space algorithm with per-spin
 * FLAT/SHARP expansion (KronProd.cpp:9-28,84-107), bath dephasing
 * (SpinInteractionComponent.cpp:285-304, rate in rad/s) and polarisation
 * rho0 = I/2^k + sum_i p.S_i (SpinState.cpp:5-60).  k <= 5. */
void orc_coherence_liouville(size_t k, const orc_z *H0, const orc_z *H1,
                             int pulse_num, size_t nT, double dt,
                             double dephase_rate, const double axis[3],
                             const double pol[3], double *L);

/* ---- cluster enumeration ------------------------------------------------ */
typedef struct orc_enum orc_enum;
/* getConnectionMatrix (SpinCollection.cpp:31-57), cDepthFirstPathTracing
 * (SpinClusterAlgorithm.cpp:75-148), cClusterIndex ordering
 * (SpinClusterIndex.cpp:55-64). */
orc_enum *orc_enumerate(size_t nspin, const double *coords, double cutoff,
                        int max_order);
size_t orc_enum_count(const orc_enum *e, int order);
void   orc_enum_cluster(const orc_enum *e, int order, size_t idx, size_t *out);
/* direct parent positions (order-1, set of positions), ascending */
size_t orc_enum_parents(const orc_enum *e, int order, size_t idx, size_t *out,
                        size_t cap);
/* getSubClusters (SpinCluster.cpp:82-98): transitive closure, as (order,pos)
 * pairs sorted like std::set<pair>. Returns count; writes 2*count entries. */
size_t orc_enum_subclusters(const orc_enum *e, int order, size_t idx,
                            size_t *out, size_t cap);
void   orc_enum_free(orc_enum *e);

/* ---- CCE reduction ------------------------------------------------------ */
/* cce_coherence_reduction + compuate_final_coherence, src/source/app/cce.cpp:
 * 151-189.  Lraw[o] is nT x count(o) column-major; outputs Ltilde[o] (same
 * shape), final_each (nT x max_order) and final_cum (nT x max_order). */
void orc_cce_reduce(const orc_enum *e, int max_order, size_t nT,
                    double *const *Lraw, double *const *Ltilde,
                    double *final_each, double *final_cum);

#ifdef __cplusplus
}
#endif
#endif
