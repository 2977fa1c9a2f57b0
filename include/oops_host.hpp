// oops_host.hpp -- C++ host layer of liboops_gb300 above the C ABI.
//
// The reference's host side is C++ (armadillo types): MatExpVector drives the
// Krylov expv (src/include/math/MatExp.h, src/source/math/MatExp.cpp), and
// EnsembleCCE / CCE run the cluster expansion (src/include/app/cce.h,
// ensemble_cce.h; src/source/app/cce.cpp, ensemble_cce.cpp).  These classes
// keep those names, method names and argument meanings over plain std:: types
// (column-major matrices as in armadillo), so host code written against the
// reference's interface for this path ports line by line:
//
//   reference                                  here
//   KronProd(dim_list).fill(idx, coeff, mats)  same
//   SumKronProd(kp_list), append, scale        same
//   MatExpVector(skp, v, time_list, method)    same; run() -> N x nT cx_mat
//   EnsembleCCE: set_bath_spin, set_bath_cluster, run_each_clusters,
//                post_treatment, getResultMatrix same (parameters as a struct
//                instead of boost::program_options)
//
// Error behaviour: the reference has no error returns (Fortran `stop`,
// ignored CUDA errors).  Every method here throws oops::Error, carrying the
// library's status code and message, instead of stopping the process.
#pragma once

#include <array>
#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "oops_cce.h"
#include "oops_expv.h"

namespace oops {

typedef std::complex<double> cx_double;

// Dense column-major matrix (the role of armadillo's mat / cx_mat).
template <typename T>
struct Matrix {
    size_t n_rows = 0, n_cols = 0;
    std::vector<T> mem;
    Matrix() = default;
    Matrix(size_t r, size_t c, T fill = T()) : n_rows(r), n_cols(c), mem(r * c, fill) {}
    T &operator()(size_t i, size_t j) { return mem[i + n_rows * j]; }
    const T &operator()(size_t i, size_t j) const { return mem[i + n_rows * j]; }
    T *memptr() { return mem.data(); }
    const T *memptr() const { return mem.data(); }
};
typedef Matrix<cx_double> cx_mat;
typedef Matrix<double> mat;

class Error : public std::runtime_error {
public:
    Error(int status, const std::string &msg) : std::runtime_error(msg), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

// coeff * (mat_0 (x) mat_1 (x) ...) on the spins `indices` of a system whose
// spins have dimensions dim_list (src/include/kron/KronProd.h).  Coefficients
// are real, as SpinInteractionDefine.h defines MULTIPLIER.
class KronProd {
public:
    KronProd() = default;
    explicit KronProd(std::vector<size_t> dim_list);
    void fill(std::vector<size_t> idx, double coeff, std::vector<cx_mat> mats);
    KronProd &scale(double factor)
    {
        coeff_ *= factor;
        return *this;
    }
    const std::vector<size_t> &getDimList() const { return dim_list_; }
    size_t getDim() const;
    double getCoeff() const { return coeff_; }
    const std::vector<size_t> &getIndices() const { return idx_; }
    const std::vector<cx_mat> &getTermMat() const { return mats_; }
    size_t getKronNum() const { return dim_list_.size(); }
    size_t getMatNum() const { return mats_.size(); }

private:
    std::vector<size_t> dim_list_, idx_;
    double coeff_ = 0.0;
    std::vector<cx_mat> mats_;
};

class SumKronProd {
public:
    SumKronProd() = default;
    explicit SumKronProd(const std::vector<KronProd> &kp_lst);
    void append(const KronProd &kp);
    SumKronProd &scale(double factor);
    const std::vector<KronProd> &getKronProdList() const { return list_; }
    const std::vector<size_t> &getDimList() const { return dim_list_; }
    size_t getDim() const;
    size_t getKronProdSize() const { return list_.size(); }
    size_t getKronNum() const { return dim_list_.size(); }
    std::vector<double> getCoeffList() const;
    std::vector<std::vector<size_t>> getIndicesList() const;
    std::vector<std::vector<cx_mat>> getTermList() const;
    std::vector<size_t> getMatNumList() const;

private:
    std::vector<size_t> dim_list_;
    std::vector<KronProd> list_;
};

// w(t) = exp(-i H t) v for every t of time_list (increasing, from 0), H given
// as a SumKronProd; result N x nT, column j = w(time_list[j])
// (MatExpVector, MatExp.cpp:86-103, 139-160).  Inexplicit and InexplicitGPU
// both run the library's device Krylov path (main_mkl_ / main_cache_); the
// dense Explicit forms are not part of this path and throw
// OOPS_ERR_UNSUPPORTED.
class MatExpVector {
public:
    enum MatExpVectorMethod { Explicit, ExplicitSparse, Inexplicit, InexplicitGPU };
    MatExpVector(const SumKronProd &skp, const std::vector<cx_double> &v,
                 const std::vector<double> &time_list, MatExpVectorMethod method);
    cx_mat run();
    cx_mat runInexplicit();
    cx_mat runInexplicitGPU();
    cx_mat getResult() const { return res_; }
    void enable_step_print() { itrace_ = 1; }
    void disable_step_print() { itrace_ = 0; }
    // Krylov parameters as the reference's constructor sets them
    size_t klim = 10;         // Lanczos length of the norm estimate
    size_t krylov_m = 30;     // Krylov dimension
    double krylov_tol = 1e-12;

private:
    cx_mat run_krylov(bool gpu_symbol);
    MatExpVectorMethod method_;
    SumKronProd skp_;
    std::vector<cx_double> v_;
    std::vector<double> time_list_;
    size_t itrace_ = 0;
    cx_mat res_;
};

// The parameters EnsembleCCE::set_parameters / CCE's constructor read from the
// command line (src/source/app/ensemble_cce.cpp:6-31, cce.cpp:16-40).
struct CCEParameters {
    std::array<double, 3> magB = {0, 0, 0};    // T
    std::array<double, 3> center = {0, 0, 0};  // NV electron position (Angstrom)
    int state_idx0 = 0, state_idx1 = 1;         // NV eigenstates (ascending energy)
    double cut_off_dist = 0.0;                  // Angstrom
    int max_order = 2;                          // CCE order (clusters up to this size)
    int pulse_num = 1;                          // CPMG pulses, 1 = Hahn echo
    double t0 = 0.0, t1 = 0.0;                  // time grid [t0, t1] (s); t0 must be 0
    int nTime = 2;
    int precision = OOPS_PREC_FP64;             // OOPS_PREC_*
    double fp64_below = 0.0;                    // oops_cce_params.fp64_below
    int fp64_max_k = 0;                         // oops_cce_params.fp64_max_k
    // bath terms (ensemble_cce.cpp:16-18); zero = the Hilbert-space path
    double dephasing_rate = 0.0;                        // Hz
    std::array<double, 3> dephasing_axis = {1, 1, 1};   // normalised by the library
    std::array<double, 3> polarization = {0, 0, 0};
};

// Ensemble CCE of the NV coherence on one GPU (EnsembleCCE + CCE).  Clusters
// are enumerated on the host, every cluster's coherence runs on the device
// (oops_cce_coherence per order), the reduction on the device
// (oops_cce_reduce).  At zero bath polarisation and dephasing the clusters run
// in the Hilbert-space form of the reference's Liouville propagation; with a
// dephasing rate or a polarisation they run in Liouville space
// (oops_cce_coherence_liouville, FP64, max_order <= 4).
class EnsembleCCE {
public:
    explicit EnsembleCCE(const CCEParameters &para);
    ~EnsembleCCE();
    EnsembleCCE(const EnsembleCCE &) = delete;
    EnsembleCCE &operator=(const EnsembleCCE &) = delete;

    // bath spin coordinates in Angstrom (cSpinSource)
    void set_bath_spin(const std::vector<std::array<double, 3>> &coords);
    // connected clusters within cut_off_dist up to max_order (cSpinGrouping)
    void set_bath_cluster();
    void run_each_clusters();
    void post_treatment();
    // CCE::export_mat_file (cce.cpp:191-234): the results as a Level 5
    // MAT-file (oops_cce_export_mat), no MATLAB library needed
    void export_mat_file(const std::string &filename) const;

    size_t getClusterNum(int cce_order) const;
    std::vector<unsigned> getClusterIndices(int cce_order) const;  // count x (order+1)
    const std::vector<double> &getTimeList() const { return time_list_; }
    std::vector<mat> getResultMatrix() const { return result_; }       // per order: nT x count
    std::vector<mat> getResultMatrixTilder() const { return tilde_; }  // reduced ratios
    mat getFinalResult() const { return final_; }                       // nT x max_order
    mat getFinalResultEachOrder() const { return final_each_; }

private:
    void free_device();
    CCEParameters para_;
    oops_cce_params p_{};
    oops_cce_bath bath_{};
    bool liouville_ = false;
    std::vector<double> time_list_;
    std::vector<double> coords_;  // nbath x 3
    oops_clusters *clusters_ = nullptr;
    std::vector<size_t> counts_;
    double *d_coords_ = nullptr;
    std::vector<unsigned *> d_idx_;
    std::vector<double *> d_L_, d_til_;
    std::vector<unsigned long long *> d_off_;
    std::vector<unsigned *> d_pairs_;
    std::vector<mat> result_, tilde_;
    mat final_, final_each_;
};

}  // namespace oops
