// ref_ensemble_pin.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own
// ensemble-CCE application classes end to end -- src/source/app/
// ensemble_cce.cpp (EnsembleCCE::cluster_evolution: the NV-conditional
// Hamiltonians, their Liouvillians, bath dephasing, the polarised initial
// state, PiecewiseFullMatrixVectorEvolution, the observable), cce.cpp (job
// distribution on one rank, the reduction), DefectCenter.cpp (NVCenter),
// the quantum operator, state and evolution classes, KronProd/spkron,
// MatExp, and the spin, cluster and physics sources -- compiled from the
// read-only reference tree by oracle/build_ref.sh with the stand-ins of
// oracle/ref_shim (armadillo, boost's variables_map, MPI, logging, MATLAB's
// mat.h).  The reference's Pade exponential is Fortran (expokit ZGPADM), for
// which there is no compiler here: zgpadm_ below calls the oracle's C
// restatement of it (oracle/oracle.c, orc_padm, itself checked against
// scipy's expm); every other step is the reference's own code.
//
//   ref_ensemble_pin <xyz file> <cutoff> <max_order> <nT> <t_max> <pulse_num>
//                    <Bx> <By> <Bz> <dephasing_rate> <px> <py> <pz> <out>
//
// The steps are those of the reference's EnsNVeBath main (application/
// EnsNVeBath.cpp:40-62): NVCenter(N14) at the origin with the field, the
// bath from the xyz file (cSpinSourceFromFile), clusters from the
// connection matrix (cDepthFirstPathTracing), run_each_clusters,
// post_treatment; CPMG with pulse_num pulses, the time list
// linspace(0, t_max, nT), NV states 0 and 1, dephasing axis (1, 1, 1), bath
// polarisation (px, py, pz).  <out> receives, in float64: order by order the
// raw cluster curves L_C (cluster-major), then the reduced curves L~_C, then
// the per-order and the cumulative products (order-major, nT each).
// Linked with cce.cpp compiled with HAS_MATLAB (ref_export_pin), the
// reference's export_mat_file also runs, into the recording stand-in of
// oracle/ref_shim/mat.h.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "include/app/ensemble_cce.h"

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
#define OOPS_PIN_ABSENT(name)                                                            \
    {                                                                                    \
        std::fprintf(stderr, "ref_ensemble_pin: %s is not part of the pin\n", name);     \
        std::abort();                                                                    \
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

class PinEnsemble : public EnsembleCCE {
public:
    explicit PinEnsemble(const po::variables_map &para) : EnsembleCCE(0, 1, para) {}
    const vector<mat> &raw() const { return _cce_evovle_result; }
    const vector<mat> &tilde() const { return _cce_evovle_result_tilder; }
    const mat &each_order() const { return _final_result_each_order; }
    const mat &cumulative() const { return _final_result; }
};

std::string str3(const char *a, const char *b, const char *c)
{
    return std::string(a) + " " + b + " " + c;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 15) {
        std::fprintf(stderr, "usage: ref_ensemble_pin <xyz> <cutoff> <max_order> <nT> <t_max> <pulse_num> "
                             "<Bx> <By> <Bz> <dephasing_rate> <px> <py> <pz> <out>\n");
        return 1;
    }
    po::variables_map para;
    para.set("input", argv[1]);
    para.set("output", "pin");
    para.set("state0", "0");
    para.set("state1", "1");
    para.set("cce", argv[3]);
    para.set("cutoff", argv[2]);
    para.set("polarization", str3(argv[11], argv[12], argv[13]));
    para.set("dephasing_rate", argv[10]);
    para.set("dephasing_axis", "1.0 1.0 1.0");
    para.set("nTime", argv[4]);
    para.set("start", "0.0");
    para.set("finish", argv[5]);
    para.set("pulse", "CPMG");
    para.set("pulse_num", argv[6]);
    para.set("magnetic_field", str3(argv[7], argv[8], argv[9]));
    para.set("position", "0.0 0.0 0.0");

#ifdef OOPS_PIN_EXPORT
    // ref_export_pin: post_treatment's export_mat_file writes <dir>/pin.mat
    // (the recording mat.h stand-in's format) into OOPS_PIN_OUTPUT_DIR
    if (const char *dir = std::getenv("OOPS_PIN_OUTPUT_DIR")) OUTPUT_PATH = std::string(dir) + "/";
#endif
    PinEnsemble sol(para);

    // Step 1: the defect centre (EnsNVeBath.cpp:create_defect_center)
    vec coord(para["position"].as<string>());
    vec magB(para["magnetic_field"].as<string>());
    NVCenter nv(NVCenter::N14, coord);
    nv.set_magB(magB);
    nv.make_espin_hamiltonian();
    sol.set_defect_center(&nv);

    // Step 2: the bath spins
    cSpinSourceFromFile src(argv[1]);
    sol.set_bath_spin(&src);

    // Step 3: the clusters (EnsNVeBath.cpp:create_spin_cluster_algrithm)
    cSpinCollection bath_spins = sol.getSpinCollecion();
    sp_mat c = bath_spins.getConnectionMatrix(para["cutoff"].as<double>());
    cDepthFirstPathTracing dfpt(c, para["cce"].as<int>());
    sol.set_bath_cluster(&dfpt);

    // Steps 4 and 5
    sol.run_each_clusters();
    sol.post_treatment();

    FILE *out = std::fopen(argv[14], "wb");
    if (!out) { std::perror(argv[14]); return 1; }
    for (const mat &m : sol.raw()) std::fwrite(m.memptr(), sizeof(double), m.n_elem, out);
    for (const mat &m : sol.tilde()) std::fwrite(m.memptr(), sizeof(double), m.n_elem, out);
    std::fwrite(sol.each_order().memptr(), sizeof(double), sol.each_order().n_elem, out);
    std::fwrite(sol.cumulative().memptr(), sizeof(double), sol.cumulative().n_elem, out);
    std::fclose(out);
    return 0;
}
