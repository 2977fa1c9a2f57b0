// ref_expv_pin.cpp -- TEST INFRASTRUCTURE ONLY.  Records what the reference's
// own Krylov caller hands the drop-in: for a cluster read from an xyz file,
// the reference's NV-conditional Hamiltonian (the SpinDipolarInteraction,
// SpinZeemanInteraction and DipolarField terms of EnsembleCCE's
// create_spin_hamiltonian, src/source/app/ensemble_cce.cpp:57-71, with the
// NVCenter's state), its Kronecker form (QuantumOperator::getKronProdForm),
// and MatExpVector(skp, v, t, Inexplicit).run() (src/source/math/
// MatExp.cpp:86-103, 216-360), which flattens the form and calls main_mkl_.
// The main_mkl_ below takes the place of the Fortran driver: it writes the
// flattened arguments to a file and returns zeros.  Compiled from the
// read-only reference tree by oracle/build_ref.sh with the stand-ins of
// oracle/ref_shim, as ref_ensemble_pin.
//
//   ref_expv_pin <xyz file> <Bx> <By> <Bz> <state 0|1> <nT> <t_max> <out>
//
// The NVCenter (N14) sits at the origin with the field; the vector is basis
// state 0; the time list is linspace(t_max / nT, t_max, nT).  <out>
// receives, as consecutive records: the scalars nSpin, nTerm, nDim,
// total_nbody, total_dim, klim, nt, m (uint64), tol (float64), then
// coeff[nTerm] (float64), nbody[nTerm], pos_offset[nTerm+1],
// pos_list[total_nbody], dim_list[total_nbody], mat_offset[total_nbody+1],
// spin_dim[nSpin] (uint64), mats[total_dim] and v[nDim] (complex128),
// tlist[nt] (float64).
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "include/app/ensemble_cce.h"
#include "include/math/MatExp.h"

// the application headers define these (include/app/app.h)
cSPINDATA SPIN_DATABASE = cSPINDATA();
string INPUT_PATH = "";
string OUTPUT_PATH = "";

namespace {
const char *g_out = nullptr;

template <typename T>
void put(FILE *f, const T *p, size_t n)
{
    if (n) std::fwrite(p, sizeof(T), n, f);
}
}  // namespace

extern "C" void main_mkl_(size_t *nspin, size_t *nTerm, double *coeff_lst, size_t *nbody_lst, size_t *pos_i_idx,
                          size_t *pos_i_lst, size_t *dim_i_lst, size_t *mat_i_idx, std::complex<double> *mat_i_lst,
                          size_t *ham_dim, size_t *nspin_dim, std::complex<double> *v, size_t *pos_idx,
                          size_t *mat_idx, size_t *k, size_t *tn, double *ta, size_t *m, double *tol,
                          size_t *itrace, std::complex<double> *w_seq, size_t *w_seq_len)
{
    (void)itrace;
    FILE *f = std::fopen(g_out, "wb");
    if (!f) { std::perror(g_out); std::exit(1); }
    const unsigned long long sc[8] = {*nspin, *nTerm, *ham_dim, *pos_idx, *mat_idx, *k, *tn, *m};
    put(f, sc, 8);
    put(f, tol, 1);
    put(f, coeff_lst, *nTerm);
    put(f, nbody_lst, *nTerm);
    put(f, pos_i_idx, *nTerm + 1);
    put(f, pos_i_lst, *pos_idx);
    put(f, dim_i_lst, *pos_idx);
    put(f, mat_i_idx, *pos_idx + 1);
    put(f, nspin_dim, *nspin);
    put(f, mat_i_lst, *mat_idx);
    put(f, v, *ham_dim);
    put(f, ta, *tn);
    std::fclose(f);
    for (size_t i = 0; i < *w_seq_len; ++i) w_seq[i] = 0.0;
}

// the other Fortran entry points the reference's MatExp.cpp names; not on this path
#define OOPS_PIN_ABSENT(name)                                                        \
    {                                                                                \
        std::fprintf(stderr, "ref_expv_pin: %s is not part of the pin\n", name);     \
        std::abort();                                                                \
    }
extern "C" {
void zgpadm_(int *, int *, double *, std::complex<double> *, int *, std::complex<double> *, int *, int *, int *,
             int *, int *) OOPS_PIN_ABSENT("zgpadm_")
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
}
int krylov_zgexpv(const int, const double _Complex *, const double _Complex *, const int, const double *,
                  double _Complex *, const int, const int, const double, const int) OOPS_PIN_ABSENT("krylov_zgexpv")
int krylov_zcooexpv(const int, const int, const int *, const int *, const double _Complex *, const double _Complex *,
                    const int, const double *, double _Complex *, const int, const int, const double,
                    const int) OOPS_PIN_ABSENT("krylov_zcooexpv")

int main(int argc, char **argv)
{
    if (argc != 9) {
        std::fprintf(stderr, "usage: ref_expv_pin <xyz> <Bx> <By> <Bz> <state 0|1> <nT> <t_max> <out>\n");
        return 1;
    }
    g_out = argv[8];
    vec magB;
    magB << std::atof(argv[2]) << std::atof(argv[3]) << std::atof(argv[4]);
    vec coord;
    coord << 0.0 << 0.0 << 0.0;
    NVCenter nv(NVCenter::N14, coord);
    nv.set_magB(magB);
    nv.make_espin_hamiltonian();
    PureState state(nv.get_eigen_state(std::atoi(argv[5])));

    cSpinSourceFromFile src(argv[1]);
    cSpinCollection bath(&src);
    bath.make();
    vector<cSPIN> spin_list = bath.getSpinList();

    // the terms of EnsembleCCE::create_spin_hamiltonian (ensemble_cce.cpp:57-71)
    SpinDipolarInteraction dip(spin_list);
    SpinZeemanInteraction zee(spin_list, magB);
    DipolarField hf_field(spin_list, nv.get_espin(), state);
    Hamiltonian hami(spin_list);
    hami.addInteraction(dip);
    hami.addInteraction(zee);
    hami.addInteraction(hf_field);
    hami.make();

    const int nT = std::atoi(argv[6]);
    const double t_max = std::atof(argv[7]);
    SumKronProd skp = hami.getKronProdForm();
    cx_vec v(skp.getDim());
    v[0] = 1.0;
    vec tl = linspace<vec>(t_max / nT, t_max, nT);
    MatExpVector expv(skp, v, tl, MatExpVector::Inexplicit);
    expv.run();
    return 0;
}
