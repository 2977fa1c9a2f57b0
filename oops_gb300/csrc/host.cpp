// host.cpp -- the C++ host layer (include/oops_host.hpp) over the library's
// C ABI: KronProd / SumKronProd / MatExpVector drive main_cache_ exactly as
// the reference's MatExpVector::runInexplicitGPU packs its arguments
// (src/source/math/MatExp.cpp:216-270, 367-521), and EnsembleCCE runs the
// cluster expansion through oops_clusters_*, oops_cce_coherence and
// oops_cce_reduce (src/source/app/cce.cpp:42-80, 151-189).
#include <cuda_runtime.h>

#include <cmath>
#include <numeric>
#include <string>

#include "oops_host.hpp"

namespace oops {

namespace {

void check(int rc, const char *what)
{
    if (rc != OOPS_OK) throw Error(rc, std::string(what) + ": " + oops_last_error());
}

void check_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw Error(OOPS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T *dev_upload(const T *h, size_t n, const char *what)
{
    T *d = nullptr;
    check_cuda(cudaMalloc((void **)&d, (n ? n : 1) * sizeof(T)), what);
    if (n) {
        cudaError_t e = cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d);
            check_cuda(e, what);
        }
    }
    return d;
}

}  // namespace

// ---------------------------------------------------------------------------
// KronProd / SumKronProd
// ---------------------------------------------------------------------------
KronProd::KronProd(std::vector<size_t> dim_list) : dim_list_(std::move(dim_list)) {}

void KronProd::fill(std::vector<size_t> idx, double coeff, std::vector<cx_mat> mats)
{
    if (idx.size() != mats.size()) throw Error(OOPS_ERR_ARG, "KronProd::fill: one matrix per index");
    for (size_t q = 0; q < idx.size(); ++q) {
        if (idx[q] >= dim_list_.size()) throw Error(OOPS_ERR_ARG, "KronProd::fill: spin index out of range");
        if (mats[q].n_rows != dim_list_[idx[q]] || mats[q].n_cols != dim_list_[idx[q]])
            throw Error(OOPS_ERR_ARG, "KronProd::fill: matrix size differs from the spin dimension");
    }
    idx_ = std::move(idx);
    coeff_ = coeff;
    mats_ = std::move(mats);
}

size_t KronProd::getDim() const
{
    size_t d = 1;
    for (size_t x : dim_list_) d *= x;
    return d;
}

SumKronProd::SumKronProd(const std::vector<KronProd> &kp_lst)
{
    for (const KronProd &kp : kp_lst) append(kp);
}

void SumKronProd::append(const KronProd &kp)
{
    if (list_.empty() && dim_list_.empty()) dim_list_ = kp.getDimList();
    else if (kp.getDimList() != dim_list_)
        throw Error(OOPS_ERR_ARG, "SumKronProd::append: terms act on different spin systems");
    list_.push_back(kp);
}

SumKronProd &SumKronProd::scale(double factor)
{
    for (KronProd &kp : list_) kp.scale(factor);
    return *this;
}

size_t SumKronProd::getDim() const
{
    size_t d = 1;
    for (size_t x : dim_list_) d *= x;
    return d;
}

std::vector<double> SumKronProd::getCoeffList() const
{
    std::vector<double> c;
    for (const KronProd &kp : list_) c.push_back(kp.getCoeff());
    return c;
}

std::vector<std::vector<size_t>> SumKronProd::getIndicesList() const
{
    std::vector<std::vector<size_t>> r;
    for (const KronProd &kp : list_) r.push_back(kp.getIndices());
    return r;
}

std::vector<std::vector<cx_mat>> SumKronProd::getTermList() const
{
    std::vector<std::vector<cx_mat>> r;
    for (const KronProd &kp : list_) r.push_back(kp.getTermMat());
    return r;
}

std::vector<size_t> SumKronProd::getMatNumList() const
{
    std::vector<size_t> r;
    for (const KronProd &kp : list_) r.push_back(kp.getMatNum());
    return r;
}

// ---------------------------------------------------------------------------
// MatExpVector
// ---------------------------------------------------------------------------
MatExpVector::MatExpVector(const SumKronProd &skp, const std::vector<cx_double> &v,
                           const std::vector<double> &time_list, MatExpVectorMethod method)
    : method_(method), skp_(skp), v_(v), time_list_(time_list)
{
}

cx_mat MatExpVector::run()
{
    switch (method_) {
        case Inexplicit: return runInexplicit();
        case InexplicitGPU: return runInexplicitGPU();
        default:
            throw Error(OOPS_ERR_UNSUPPORTED,
                        "MatExpVector: dense Explicit forms are not part of this library's path");
    }
}

cx_mat MatExpVector::runInexplicit() { return run_krylov(false); }
cx_mat MatExpVector::runInexplicitGPU() { return run_krylov(true); }

// The flattening of MatExp.cpp:216-270: per term its body count, a prefix sum
// of positions, every body's dimension and column-major matrix, a prefix sum
// of matrix sizes.
cx_mat MatExpVector::run_krylov(bool gpu_symbol)
{
    const size_t nDim = skp_.getDim();
    if (v_.size() != nDim) throw Error(OOPS_ERR_ARG, "MatExpVector: vector length differs from the Hamiltonian's dimension");
    std::vector<double> coeff = skp_.getCoeffList();
    std::vector<size_t> nBody = skp_.getMatNumList();
    std::vector<size_t> spin_dim = skp_.getDimList();
    size_t nSpin = skp_.getKronNum(), nTerm = skp_.getKronProdSize();
    std::vector<size_t> pos_offset(nTerm + 1, 0);
    std::partial_sum(nBody.begin(), nBody.end(), pos_offset.begin() + 1);
    std::vector<size_t> pos_list, dim_list, mat_offset(1, 0);
    std::vector<cx_double> matC;
    for (const KronProd &kp : skp_.getKronProdList())
        for (size_t q = 0; q < kp.getMatNum(); ++q) {
            const cx_mat &m = kp.getTermMat()[q];
            pos_list.push_back(kp.getIndices()[q]);
            dim_list.push_back(m.n_cols);
            matC.insert(matC.end(), m.mem.begin(), m.mem.end());
            mat_offset.push_back(matC.size());
        }
    size_t total_nbody = pos_offset[nTerm], total_dim = matC.size();
    size_t nt = time_list_.size();
    res_ = cx_mat(nDim, nt);
    size_t w_seq_len = nDim * nt;
    std::vector<cx_double> v = v_;
    std::vector<double> tlist = time_list_;
    size_t klim_v = klim, m = krylov_m, itrace = itrace_;
    double tol = krylov_tol;
    if (pos_list.empty()) {
        pos_list.push_back(0);
        dim_list.push_back(1);
    }
    if (matC.empty()) matC.push_back(cx_double(0, 0));
    if (gpu_symbol) {
        size_t mtpb = 256, mgs[3] = {2147483647u, 65535u, 65535u};
        main_cache_(&nSpin, &nTerm, coeff.data(), nBody.data(), pos_offset.data(), pos_list.data(),
                    dim_list.data(), mat_offset.data(), matC.data(), const_cast<size_t *>(&nDim),
                    spin_dim.data(), v.data(), &total_nbody, &total_dim, &klim_v, &mtpb, mgs, &nt,
                    tlist.data(), &m, &tol, &itrace, res_.memptr(), &w_seq_len);
    } else {
        main_mkl_(&nSpin, &nTerm, coeff.data(), nBody.data(), pos_offset.data(), pos_list.data(),
                  dim_list.data(), mat_offset.data(), matC.data(), const_cast<size_t *>(&nDim),
                  spin_dim.data(), v.data(), &total_nbody, &total_dim, &klim_v, &nt, tlist.data(), &m,
                  &tol, &itrace, res_.memptr(), &w_seq_len);
    }
    const int rc = oops_expv_status();
    if (rc != OOPS_OK) throw Error(rc, std::string("MatExpVector: ") + oops_expv_error());
    return res_;
}

// ---------------------------------------------------------------------------
// EnsembleCCE
// ---------------------------------------------------------------------------
EnsembleCCE::EnsembleCCE(const CCEParameters &para) : para_(para)
{
    if (para.max_order < 1 || para.max_order > 6) throw Error(OOPS_ERR_ARG, "EnsembleCCE: max_order must be 1..6");
    if (para.nTime < 1) throw Error(OOPS_ERR_ARG, "EnsembleCCE: nTime must be >= 1");
    if (para.t0 != 0.0) throw Error(OOPS_ERR_ARG, "EnsembleCCE: the time grid must start at t0 = 0");
    time_list_.resize(para.nTime);
    const double dt = para.nTime > 1 ? (para.t1 - para.t0) / (para.nTime - 1) : 0.0;
    for (int i = 0; i < para.nTime; ++i) time_list_[i] = para.t0 + dt * i;
    double evals[3], svec[9];
    check(oops_nv_states(para.magB.data(), evals, svec), "EnsembleCCE: NV states");
    if (para.state_idx0 < 0 || para.state_idx0 > 2 || para.state_idx1 < 0 || para.state_idx1 > 2)
        throw Error(OOPS_ERR_ARG, "EnsembleCCE: NV state index must be 0..2");
    for (int a = 0; a < 3; ++a) {
        p_.B[a] = para.magB[a];
        p_.center[a] = para.center[a];
        p_.sv0[a] = svec[3 * para.state_idx0 + a];
        p_.sv1[a] = svec[3 * para.state_idx1 + a];
    }
    p_.gamma_center = -1.760859708e11;
    p_.gamma_bath = 6.728284e7;
    p_.pulse_num = para.pulse_num;
    p_.nT = (size_t)para.nTime;
    p_.dt = dt;
    p_.fp64_below = para.fp64_below;
    p_.fp64_max_k = para.fp64_max_k;
    bath_.dephasing_rate = para.dephasing_rate;
    for (int a = 0; a < 3; ++a) {
        bath_.dephasing_axis[a] = para.dephasing_axis[a];
        bath_.polarization[a] = para.polarization[a];
    }
    liouville_ = para.dephasing_rate != 0.0 || para.polarization[0] != 0.0 ||
                 para.polarization[1] != 0.0 || para.polarization[2] != 0.0;
}

EnsembleCCE::~EnsembleCCE()
{
    free_device();
    if (clusters_) oops_clusters_destroy(clusters_);
}

void EnsembleCCE::free_device()
{
    if (d_coords_) cudaFree(d_coords_);
    d_coords_ = nullptr;
    for (auto p : d_idx_) cudaFree(p);
    for (auto p : d_L_) cudaFree(p);
    for (auto p : d_til_) cudaFree(p);
    for (auto p : d_off_) cudaFree(p);
    for (auto p : d_pairs_) cudaFree(p);
    d_idx_.clear();
    d_L_.clear();
    d_til_.clear();
    d_off_.clear();
    d_pairs_.clear();
}

void EnsembleCCE::set_bath_spin(const std::vector<std::array<double, 3>> &coords)
{
    coords_.clear();
    for (const auto &c : coords) coords_.insert(coords_.end(), c.begin(), c.end());
}

void EnsembleCCE::set_bath_cluster()
{
    if (clusters_) oops_clusters_destroy(clusters_);
    clusters_ = nullptr;
    check(oops_clusters_enumerate(coords_.size() / 3, coords_.data(), para_.cut_off_dist,
                                  para_.max_order, &clusters_),
          "EnsembleCCE::set_bath_cluster");
    counts_.assign(para_.max_order, 0);
    for (int o = 0; o < para_.max_order; ++o) counts_[o] = oops_clusters_count(clusters_, o);
}

size_t EnsembleCCE::getClusterNum(int cce_order) const
{
    return (cce_order >= 0 && cce_order < (int)counts_.size()) ? counts_[cce_order] : 0;
}

std::vector<unsigned> EnsembleCCE::getClusterIndices(int cce_order) const
{
    std::vector<unsigned> r(getClusterNum(cce_order) * (cce_order + 1));
    if (!r.empty()) check(oops_clusters_indices(clusters_, cce_order, r.data()), "getClusterIndices");
    return r;
}

// CCE::run_each_clusters (cce.cpp:54-70): every order's clusters in one
// batched device call instead of one cluster_evolution per cluster.
void EnsembleCCE::run_each_clusters()
{
    if (!clusters_) throw Error(OOPS_ERR_ARG, "EnsembleCCE: set_bath_cluster() first");
    free_device();
    const size_t nbath = coords_.size() / 3, nT = (size_t)para_.nTime;
    d_coords_ = dev_upload(coords_.data(), coords_.size(), "EnsembleCCE: coordinates");
    result_.assign(para_.max_order, mat());
    for (int o = 0; o < para_.max_order; ++o) {
        const size_t n = counts_[o];
        std::vector<unsigned> idx = getClusterIndices(o);
        d_idx_.push_back(dev_upload(idx.data(), idx.size(), "EnsembleCCE: cluster indices"));
        double *L = nullptr, *T = nullptr;
        check_cuda(cudaMalloc((void **)&L, (n ? n : 1) * nT * sizeof(double)), "EnsembleCCE: curves");
        d_L_.push_back(L);
        check_cuda(cudaMalloc((void **)&T, (n ? n : 1) * nT * sizeof(double)), "EnsembleCCE: curves");
        d_til_.push_back(T);
        if (n && liouville_)
            check(oops_cce_coherence_liouville(d_coords_, nbath, d_idx_.back(), n, o + 1, &p_, &bath_, L, nullptr),
                  "EnsembleCCE::run_each_clusters");
        else if (n)
            check(oops_cce_coherence(d_coords_, nbath, d_idx_.back(), n, o + 1, &p_, para_.precision, L, nullptr),
                  "EnsembleCCE::run_each_clusters");
        // _cce_evovle_result[o]: nTime x clst_num, column i = cluster i
        result_[o] = mat(nT, n);
        if (n) check_cuda(cudaMemcpy(result_[o].memptr(), L, n * nT * sizeof(double), cudaMemcpyDeviceToHost),
                          "EnsembleCCE: curves to host");
    }
}

// CCE::post_treatment (cce.cpp:72-80): cce_coherence_reduction and
// compuate_final_coherence (cce.cpp:151-189) on the device.
void EnsembleCCE::post_treatment()
{
    if (d_L_.size() != (size_t)para_.max_order) throw Error(OOPS_ERR_ARG, "EnsembleCCE: run_each_clusters() first");
    const int K = para_.max_order;
    const size_t nT = (size_t)para_.nTime;
    for (int o = 0; o < K; ++o) {
        std::vector<size_t> offs(counts_[o] + 1);
        const size_t tot = oops_clusters_subcluster_total(clusters_, o);
        std::vector<unsigned> pairs(2 * tot + 2);  // never empty: single spins have no sub-clusters
        check(oops_clusters_subclusters(clusters_, o, offs.data(), pairs.data()), "post_treatment: closures");
        std::vector<unsigned long long> off64(offs.begin(), offs.end());
        d_off_.push_back(dev_upload(off64.data(), off64.size(), "post_treatment: closures"));
        d_pairs_.push_back(dev_upload(pairs.data(), 2 * tot, "post_treatment: closures"));
    }
    double *each = nullptr, *cum = nullptr;
    check_cuda(cudaMalloc((void **)&each, K * nT * sizeof(double)), "post_treatment");
    cudaError_t e = cudaMalloc((void **)&cum, K * nT * sizeof(double));
    if (e != cudaSuccess) {
        cudaFree(each);
        check_cuda(e, "post_treatment");
    }
    std::vector<const double *> Lp(d_L_.begin(), d_L_.end());
    std::vector<const unsigned long long *> offp(d_off_.begin(), d_off_.end());
    std::vector<const unsigned *> pairp(d_pairs_.begin(), d_pairs_.end());
    int rc = oops_cce_reduce(K, counts_.data(), nT, Lp.data(), d_til_.data(), offp.data(), pairp.data(),
                             each, cum, nullptr);
    final_ = mat(nT, K);
    final_each_ = mat(nT, K);
    tilde_.assign(K, mat());
    if (rc == OOPS_OK) {
        e = cudaMemcpy(final_.memptr(), cum, K * nT * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(final_each_.memptr(), each, K * nT * sizeof(double), cudaMemcpyDeviceToHost);
        for (int o = 0; o < K && e == cudaSuccess; ++o) {
            tilde_[o] = mat(nT, counts_[o]);
            if (counts_[o])
                e = cudaMemcpy(tilde_[o].memptr(), d_til_[o], counts_[o] * nT * sizeof(double), cudaMemcpyDeviceToHost);
        }
    }
    cudaFree(each);
    cudaFree(cum);
    check(rc, "EnsembleCCE::post_treatment");
    check_cuda(e, "EnsembleCCE::post_treatment");
    // the reference's post_treatment ends with export_mat_file on rank 0
    // (cce.cpp:72-80); here when an output directory was given
    if (!output_dir_.empty() && my_rank_ == 0) export_mat_file(output_dir_ + "/" + output_name_ + ".mat");
}

void EnsembleCCE::export_mat_file(const std::string &filename) const
{
    if (final_.mem.empty()) throw Error(OOPS_ERR_ARG, "EnsembleCCE::export_mat_file: post_treatment() first");
    std::vector<const double *> L(para_.max_order), T(para_.max_order);
    for (int o = 0; o < para_.max_order; ++o) {
        L[o] = result_[o].mem.data();
        T[o] = tilde_[o].mem.data();
    }
    check(oops_cce_export_mat(filename.c_str(), para_.max_order, time_list_.size(), counts_.data(), L.data(),
                              T.data(), final_each_.mem.data(), final_.mem.data(), time_list_.data()),
          "EnsembleCCE::export_mat_file");
}

}  // namespace oops
