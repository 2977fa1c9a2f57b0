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
//   EnsembleCCE(my_rank, worker_num, para)    same, para an oops::variables_map
//   set_defect_center(&nv), set_bath_spin(&src), set_bath_cluster(&dfpt),
//   getSpinCollecion, run_each_clusters, post_treatment, getResultMatrix  same
//   NVCenter, cSPIN, cSpinSourceFromFile, cSpinSourceUniformRandom,
//   cSpinCollection (getConnectionMatrix), cDepthFirstPathTracing      same
//   arma::vec / sp_mat, po::variables_map      oops::vec / sp_mat / variables_map
//
// so EnsNVeBath's main (src/application/EnsNVeBath.cpp:40-62) compiles
// against this header with only its type names' namespaces changed
// (tests/cpp/ensnvebath_demo.cpp does exactly that).
//
// Error behaviour: the reference has no error returns (Fortran `stop`,
// ignored CUDA errors).  Every method here throws oops::Error, carrying the
// library's status code and message, instead of stopping the process.
#pragma once

#include <array>
#include <complex>
#include <cstddef>
#include <initializer_list>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
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

// ---------------------------------------------------------------------------
// The reference application's classes (src/application/EnsNVeBath.cpp:40-62
// drives them): parameters, spins and spin sources, the spin collection and
// its connection matrix, the cluster-growth algorithm and the NV centre.
// Armadillo's vec and sp_mat and boost's variables_map are replaced by the
// small types below, with the members those call sites use.
// ---------------------------------------------------------------------------

// A column of doubles (armadillo's vec): vec("0.0 0.1 0.2") parses
// whitespace-separated numbers, as arma::vec(std::string) does.
class vec {
public:
    vec() = default;
    explicit vec(const std::string &text);
    vec(std::initializer_list<double> x) : v_(x) {}
    explicit vec(std::vector<double> x) : v_(std::move(x)) {}
    size_t n_elem() const { return v_.size(); }
    double &operator[](size_t i) { return v_.at(i); }
    double operator[](size_t i) const { return v_.at(i); }
    double &operator()(size_t i) { return v_.at(i); }
    double operator()(size_t i) const { return v_.at(i); }
    const std::vector<double> &std() const { return v_; }

private:
    std::vector<double> v_;
};

// One parsed option value: as<int>(), as<double>(), as<std::string>().
class variable_value {
public:
    variable_value() = default;
    explicit variable_value(std::string text) : text_(std::move(text)) {}
    template <typename T>
    T as() const;
    const std::string &text() const { return text_; }

private:
    std::string text_;
};

// The options map the reference's applications read with
// para["name"].as<T>() (boost::program_options::variables_map).
class variables_map {
public:
    const variable_value &operator[](const std::string &key) const;
    void set(const std::string &key, const std::string &value) { m_[key] = variable_value(value); }
    size_t count(const std::string &key) const { return m_.count(key); }
    std::vector<std::string> keys() const;

private:
    std::map<std::string, variable_value> m_;
};

// EnsNVeBath's options with their defaults (src/application/EnsNVeBath.cpp:
// 121-151), overridden by "--name value", "--name=value" or "-x value" from
// argv (argv[0] is the program name).  Also accepted, outside the
// reference's list: --precision fp64|mixed (the device path's arithmetic)
// and --output_dir DIR (where post_treatment writes <output>.mat).  The
// default "output" is "EnsNVeBath" followed by the command line, as the
// application builds it (EnsNVeBath.cpp:80-85).
variables_map ensnvebath_options(int argc, const char *const *argv);
// The same for EnsNVnBath, the nuclear-spin bath read from a file
// (src/application/EnsNVnBath.cpp:116-139: input C13Bath/RoyCoord.xyz,
// cutoff 6 A, CCE-3, no dephasing, 101 points of [0, 2 ms]).
variables_map ensnvnbath_options(int argc, const char *const *argv);

// A spin (src/include/spin/Spin.h): coordinate (Angstrom), isotope name and
// the properties of that isotope from the reference's table
// (src/source/spin/Spin/SpinData.cpp:4-18: "13C", "14C", "15C", "E", "NVe";
// "14N" and "15N" are accepted as names of the nitrogen entries).
class cSPIN {
public:
    cSPIN() = default;
    cSPIN(vec coord, const std::string &isotope);
    vec get_coordinate() const { return coordinate_; }
    std::string get_isotope() const { return isotope_; }
    int get_multiplicity() const { return multiplicity_; }
    int get_dimension() const { return multiplicity_; }
    double get_gamma() const { return gamma_; }
    double get_omegaQ() const { return omegaQ_; }

private:
    vec coordinate_{0.0, 0.0, 0.0};
    std::string isotope_ = "None";
    int multiplicity_ = 0;
    double gamma_ = 0.0, omegaQ_ = 0.0;
};

// Spin sources (src/include/spin/SpinSource.h,
// src/source/spin/SpinCollection/SpinSource.cpp).
class cSpinSource {
public:
    virtual ~cSpinSource() = default;
    virtual std::vector<cSPIN> &generate() = 0;
    std::vector<cSPIN> &get_spin_list() { return spin_list; }
    // "N" then "isotope<TAB>x<TAB>y<TAB>z" per spin, as the reference writes
    void export_coordinates(const std::string &filename);

protected:
    std::vector<cSPIN> spin_list;
};

// An .xyz file: the spin count, then "isotope x y z" per spin (:55-79).
class cSpinSourceFromFile : public cSpinSource {
public:
    explicit cSpinSourceFromFile(std::string filename) : filename_(std::move(filename)) {}
    std::vector<cSPIN> &generate() override;

private:
    std::string filename_;
};

// max_num points uniform in the cube [-range, range]^3 (armadillo's randu
// after arma_rng::set_seed(seed): here the C++11 generator armadillo uses,
// std::mt19937_64 with std::uniform_real_distribution, filled column by
// column), the num closest to the origin kept in order of distance (:112-129).
class cSpinSourceUniformRandom : public cSpinSource {
public:
    cSpinSourceUniformRandom(double range, int max_num, int num, const std::string &isotope, int seed)
        : range_(range), max_num_(max_num), num_(num), isotope_(isotope), seed_(seed) {}
    std::vector<cSPIN> &generate() override;

private:
    double range_;
    int max_num_, num_;
    std::string isotope_;
    int seed_;
};

// A sparse 0/1 matrix in compressed rows (the role of the sp_mat that
// getConnectionMatrix returns): row i's non-zero columns, ascending.
struct sp_mat {
    size_t n_rows = 0, n_cols = 0;
    std::vector<size_t> row_off;  // n_rows + 1
    std::vector<unsigned> cols;
    double operator()(size_t i, size_t j) const;
    size_t n_nonzero() const { return cols.size(); }
};

// The bath (src/include/spin/SpinCollection.h,
// src/source/spin/SpinCollection/SpinCollection.cpp:10-57).
class cSpinCollection {
public:
    cSpinCollection() = default;
    explicit cSpinCollection(cSpinSource *source) : source_(source) {}
    void make();
    size_t getSpinNum() const { return spin_list_.size(); }
    std::vector<cSPIN> getSpinList() const { return spin_list_; }
    mat getCoordinateMat() const;  // nspin x 3
    mat getDistanceMatrix() const;  // nspin x nspin
    // connected iff distance <= threshold, no self connection (:51-57)
    sp_mat getConnectionMatrix(double threshold) const;

private:
    cSpinSource *source_ = nullptr;
    std::vector<cSPIN> spin_list_;
};

// Cluster growth on a connection matrix (src/include/spin/
// SpinClusterAlgorithm.h; SpinClusterAlgorithm.cpp:75-148): order o holds the
// connected clusters of o+1 spins, each order in std::set<cClusterIndex>
// order.  The enumeration runs in liboops_gb300 (oops_clusters_enumerate_graph).
class cSpinGrouping {
public:
    explicit cSpinGrouping(const sp_mat &connection_matrix) : c_(connection_matrix) {}
    virtual ~cSpinGrouping();
    virtual void generate() = 0;
    size_t getMaxOrder() const { return max_order_; }
    const sp_mat &getConnectionMatrix() const { return c_; }
    // per order: count x (order+1) sorted spin indices, row-major
    std::vector<std::vector<unsigned>> get_cluster_index_mat() const { return index_; }

protected:
    sp_mat c_;
    size_t max_order_ = 0;
    std::vector<std::vector<unsigned>> index_;
};

class cDepthFirstPathTracing : public cSpinGrouping {
public:
    cDepthFirstPathTracing(const sp_mat &connection_matrix, size_t maxOrder)
        : cSpinGrouping(connection_matrix)
    {
        max_order_ = maxOrder;
    }
    void generate() override;
};

// The defect centre (src/include/app/DefectCenter.h,
// src/source/app/DefectCenter.cpp:3-45).
class DefectCenter {
public:
    virtual ~DefectCenter() = default;
    cSPIN get_espin() const { return electron_spin_; }
    cSPIN get_nspin() const { return nuclear_spin_; }
    virtual void make_espin_hamiltonian() = 0;
    void set_magB(vec b) { magB_ = std::move(b); }
    void set_magB(double bx, double by, double bz) { magB_ = vec{bx, by, bz}; }
    vec get_magB() const { return magB_; }
    // eigenvalues of the electron Hamiltonian (ascending, rad/s) and the spin
    // vector <S> of eigenstate i (the conditioning field of the bath)
    double get_eigen_value(int i) const { return evals_.at(i); }
    vec get_spin_vector(int i) const;

protected:
    cSPIN electron_spin_, nuclear_spin_;
    vec magB_{0.0, 0.0, 0.0};
    std::vector<double> evals_, svec_;
};

// NV centre: nitrogen at coord, electron at coord + (3.57/4)(1,1,1);
// H = D S_111^2 + gamma B.S with D = 2.87 GHz (make_espin_hamiltonian,
// computed by oops_nv_states).
class NVCenter : public DefectCenter {
public:
    enum NVNuclearSpin { N14, N15 };
    explicit NVCenter(NVNuclearSpin nuc);
    NVCenter(NVNuclearSpin nuc, vec coord);
    void make_espin_hamiltonian() override;
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
// (oops_cce_coherence_liouville, FP64, max_order <= 6).
class EnsembleCCE {
public:
    explicit EnsembleCCE(const CCEParameters &para);
    // The reference's constructor (ensemble_cce.h:13; set_parameters,
    // ensemble_cce.cpp:6-31): the run's parameters from the options map.
    // my_rank and worker_num are accepted as the reference takes them; every
    // rank computes the whole run on its GPU (one bath's clusters fit one
    // GPU), and rank 0 alone writes the result file.
    EnsembleCCE(int my_rank, int worker_num, const variables_map &para);
    // Step 1 of EnsNVeBath: the NV states condition the bath Hamiltonians
    // (CCE::set_defect_center, cce.cpp:22-29)
    void set_defect_center(DefectCenter *defect);
    // Step 2: cSpinCollection(source).make() (CCE::set_bath_spin, :31-38)
    void set_bath_spin(cSpinSource *source);
    cSpinCollection getSpinCollecion() const { return bath_spins_; }
    // Step 3: the clusters of the grouping's connection matrix up to its
    // order (CCE::set_bath_cluster, :40-50)
    void set_bath_cluster(cSpinGrouping *grouping);
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
    int my_rank_ = 0;
    std::string output_dir_, output_name_;
    cSpinCollection bath_spins_;
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
