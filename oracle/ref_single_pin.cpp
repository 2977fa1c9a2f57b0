// ref_single_pin.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own
// single-sample CCE application class end to end -- src/source/app/
// single_sample_cce.cpp (SingleSampleCCE: the bath's pure product state from
// srand(seed); rand() % 2, the NV-conditional Hamiltonians with the mean
// dipolar field of the bath spins outside the cluster, the cluster's basis
// state propagated through both pulse sequences, Re <psi_1 | psi_2>) and
// cce.cpp (job distribution on one rank, the reduction) over the same
// classes as ref_ensemble_pin -- compiled from the read-only reference tree
// by oracle/build_ref.sh with the stand-ins of oracle/ref_shim (the XML
// configuration is the reader's getters over entries set below); expokit's
// Fortran ZGPADM is the oracle's C restatement (orc_padm).
//
//   ref_single_pin <xyz file> <cutoff> <max_order> <nT> <t_max> <pulse_num>
//                  <Bx> <By> <Bz> <bath_state_seed> <out>
//
// The steps are those of the reference's SingleSampleCCE_NV_C13 main
// (application/SingleSampleCCE_NV_C13.cpp:11-57): NVCenter(N14) at the
// origin with the field, the bath from the xyz file, clusters from the
// connection matrix, prepare_bath_state, run_each_clusters, post_treatment;
// CPMG with pulse_num pulses, the time sequence (0, t_max, nT), NV states 0
// and 1.  <out> receives, in float64: order by order the raw cluster curves
// (cluster-major), then the reduced curves, then the per-order and the
// cumulative products (order-major, nT each).  The bath state drawn by the
// host C library's rand() is also printed, one digit per bath spin.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "include/app/single_sample_cce.h"

extern "C" {
#include "oracle.h"
}

// the application headers define these (include/app/app.h)
cSPINDATA SPIN_DATABASE = cSPINDATA();
string INPUT_PATH = "";
string OUTPUT_PATH = "";

// expokit's ZGPADM (Fortran) for MatExp::pade_exp_mat: exp(t H) of the
// m x m matrix H into wsp, at 1-based position iexph
extern "C" void zgpadm_(int *ideg, int *m, double *t, std::complex<double> *H, int *ldh,
                        std::complex<double> *wsp, int *lwsp, int *ipiv, int *iexph, int *ns, int *iflag)
{
    (void)lwsp;
    (void)ipiv;
    *iexph = 1;
    *iflag = orc_padm(*ideg, *m, *t, reinterpret_cast<const orc_z *>(H), *ldh, reinterpret_cast<orc_z *>(wsp), ns);
}

// the Krylov drivers MatExp.cpp names (MatExpVector); not on this path
#define OOPS_PIN_ABSENT(name)                                                          \
    {                                                                                  \
        std::fprintf(stderr, "ref_single_pin: %s is not part of the pin\n", name);     \
        std::abort();                                                                  \
    }
extern "C" {
void krylov_zgexpv_(const int *, const double _Complex *, const double _Complex *, const int *, const double *,
                    const int *, const double *, double *, double _Complex *, const int *, int *, const int *,
                    const int *, int *, double _Complex *, const int *) OOPS_PIN_ABSENT("krylov_zgexpv_")
void krylov_zcooexpv_(const int *, const int *, const int *, const int *, const double _Complex *,
                      const double _Complex *, const int *, const double *, const int *, const double *, double *,
                      double _Complex *, const int *, int *, const int *, const int *, int *, double _Complex *,
                      const int *) OOPS_PIN_ABSENT("krylov_zcooexpv_")
void main_cache_(size_t *, size_t *, double *, size_t *, size_t *, size_t *, size_t *, size_t *,
                 std::complex<double> *, size_t *, size_t *, std::complex<double> *, size_t *, size_t *, size_t *,
                 size_t *, size_t *, size_t *, double *, size_t *, double *, size_t *, std::complex<double> *,
                 size_t *) OOPS_PIN_ABSENT("main_cache_")
void main_mkl_(size_t *, size_t *, double *, size_t *, size_t *, size_t *, size_t *, size_t *,
               std::complex<double> *, size_t *, size_t *, std::complex<double> *, size_t *, size_t *, size_t *,
               size_t *, double *, size_t *, double *, size_t *, std::complex<double> *,
               size_t *) OOPS_PIN_ABSENT("main_mkl_")
}
// declared with C++ linkage by the reference's krylov_expv.h
int krylov_zgexpv(const int, const double _Complex *, const double _Complex *, const int, const double *,
                  double _Complex *, const int, const int, const double, const int) OOPS_PIN_ABSENT("krylov_zgexpv")
int krylov_zcooexpv(const int, const int, const int *, const int *, const double _Complex *, const double _Complex *,
                    const int, const double *, double _Complex *, const int, const int, const double,
                    const int) OOPS_PIN_ABSENT("krylov_zcooexpv")

namespace {

class PinSingle : public SingleSampleCCE {
public:
    explicit PinSingle(const ConfigXML &cfg) : SingleSampleCCE(0, 1, cfg) {}
    const vector<mat> &raw() const { return _cce_evovle_result; }
    const vector<mat> &tilde() const { return _cce_evovle_result_tilder; }
    const mat &each_order() const { return _final_result_each_order; }
    const mat &cumulative() const { return _final_result; }
};

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 12) {
        std::fprintf(stderr, "usage: ref_single_pin <xyz> <cutoff> <max_order> <nT> <t_max> <pulse_num> "
                             "<Bx> <By> <Bz> <bath_state_seed> <out>\n");
        return 1;
    }
    const std::string field = std::string(argv[7]) + " " + argv[8] + " " + argv[9];
    ConfigXML cfg;
    cfg.set("Data", "input_file", argv[1]);
    cfg.set("Data", "output_file", "pin");
    cfg.set("CenterSpin", "name", "NV");
    cfg.set("CenterSpin", "state_index0", "0");
    cfg.set("CenterSpin", "state_index1", "1");
    cfg.set("CenterSpin", "coordinate", "0.0 0.0 0.0");
    cfg.set("SpinBath", "cut_off_dist", argv[2]);
    cfg.set("SpinBath", "bath_state_seed", argv[10]);
    cfg.set("SpinBath", "max_order", argv[3]);
    cfg.set("Dynamics", "nTime", argv[4]);
    cfg.set("Dynamics", "t0", "0.0");
    cfg.set("Dynamics", "t1", argv[5]);
    cfg.set("Condition", "pulse_name", "CPMG");
    cfg.set("Condition", "pulse_number", argv[6]);
    cfg.set("Condition", "magnetic_field", field);

    PinSingle sol(cfg);

    // Step 1: the defect centre (SingleSampleCCE_NV_C13.cpp:create_defect_center)
    NVCenter nv(NVCenter::N14, cfg.getVectorParameter("CenterSpin", "coordinate"));
    nv.set_magB(cfg.getVectorParameter("Condition", "magnetic_field"));
    nv.make_espin_hamiltonian();
    sol.set_defect_center(&nv);

    // Step 2: the bath spins (create_spin_source)
    cSpinSourceFromFile src(cfg.getStringParameter("Data", "input_file"));
    sol.set_bath_spin(&src);

    // Step 3: the clusters (create_spin_cluster_algrithm)
    cSpinCollection bath_spins = sol.getSpinCollecion();
    sp_mat c = bath_spins.getConnectionMatrix(cfg.getDoubleParameter("SpinBath", "cut_off_dist"));
    cDepthFirstPathTracing dfpt(c, cfg.getIntParameter("SpinBath", "max_order"));
    sol.set_bath_cluster(&dfpt);

    // Steps 4 and 5
    sol.prepare_bath_state();
    sol.run_each_clusters();
    sol.post_treatment();

    // the bath state prepare_bath_state drew: the same srand/rand sequence
    srand(cfg.getIntParameter("SpinBath", "bath_state_seed"));
    std::printf("bath_state ");
    for (int i = 0; i < bath_spins.getSpinNum(); ++i) std::printf("%d", rand() % 2);
    std::printf("\n");

    FILE *out = std::fopen(argv[11], "wb");
    if (!out) { std::perror(argv[11]); return 1; }
    for (const mat &m : sol.raw()) std::fwrite(m.memptr(), sizeof(double), m.n_elem, out);
    for (const mat &m : sol.tilde()) std::fwrite(m.memptr(), sizeof(double), m.n_elem, out);
    std::fwrite(sol.each_order().memptr(), sizeof(double), sol.each_order().n_elem, out);
    std::fwrite(sol.cumulative().memptr(), sizeof(double), sol.cumulative().n_elem, out);
    std::fclose(out);
    return 0;
}
