// TEST INFRASTRUCTURE ONLY.  Stand-in for the reference's application header
// src/include/app/cce.h, found ahead of it on oracle/build_ref.sh's include
// path so that the reference's own src/source/app/cce.cpp compiles without
// the application's class tree, boost, MPI or the XML configuration.  It
// declares the CCE base class with the members and methods cce.cpp defines
// and uses (names and types as the reference declares them), and minimal
// stand-ins for the types those methods touch outside the reduction:
// ConfigXML, boost's variables_map, DefectCenter, PureState and the four MPI
// calls of job_distribution / DataGathering, which abort if ever called.  The
// pin (oracle/ref_cce_pin.cpp) derives from CCE, fills the per-order cluster
// curves and the cluster set, and calls post_treatment(), which runs the
// reference's cce_coherence_reduction and compuate_final_coherence
// (cce.cpp:151-189); export_mat_file is compiled without HAS_MATLAB.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include <armadillo>

#include "include/spin/Spin.h"
#include "include/spin/SpinCluster.h"
#include "include/spin/SpinClusterAlgorithm.h"
#include "include/spin/SpinCollection.h"
#include "include/spin/SpinSource.h"

using namespace std;
using namespace arma;

// ---- configuration objects (constructed, never read by the reduction)
class ConfigXML {
public:
    void printParameters() const {}
};
namespace po {
struct variables_map {};
}

// ---- defect centre and pure state (set_defect_center only)
class DefectCenter {
public:
    cSPIN get_espin() const { return cSPIN(); }
    cx_vec get_eigen_state(int) const { return cx_vec(); }
};
class PureState {
public:
    PureState() = default;
    explicit PureState(const cx_vec &v) : _v(v) {}

private:
    cx_vec _v;
};

// ---- MPI (job_distribution and DataGathering only; the pin runs one rank)
typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Status;
static const MPI_Datatype MPI_UNSIGNED = 1, MPI_DOUBLE = 2;
static const MPI_Comm MPI_COMM_WORLD = 0;
static MPI_Status *const MPI_STATUS_IGNORE = nullptr;
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm)
{
    std::fprintf(stderr, "ref_cce_pin: MPI_Send called in a one-rank pin\n");
    std::abort();
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *)
{
    std::fprintf(stderr, "ref_cce_pin: MPI_Recv called in a one-rank pin\n");
    std::abort();
}

class CCE {
public:
    CCE(int my_rank, int worker_num, const ConfigXML &cfg);
    CCE(int my_rank, int worker_num, const po::variables_map &para);
    virtual ~CCE() = default;

    void set_defect_center(DefectCenter *defect);
    void set_bath_spin(cSpinSource *source);
    void set_bath_cluster(cSpinGrouping *spin_grouping);
    void run_each_clusters();
    void post_treatment();

    vector<mat> getResultMatrix() const { return _cce_evovle_result; }

protected:
    po::variables_map _para;
    ConfigXML _cfg;
    string _result_filename;

    DefectCenter *_defect_center = nullptr;
    cSPIN _center_spin;
    int _state_idx0 = 0;
    int _state_idx1 = 1;
    pair<PureState, PureState> _state_pair;

    int _max_order = 0;
    cSpinSource *_spin_source = nullptr;
    cSpinGrouping *_spin_grouping = nullptr;
    cSpinCollection _bath_spins;
    cSpinCluster _spin_clusters;

    int _nTime = 0;
    vec _time_list;

    int _my_rank = 0;
    int _worker_num = 1;
    cSpinCluster _my_clusters;

    vector<mat> _cce_evovle_result;
    vector<mat> _cce_evovle_result_tilder;
    mat _final_result;
    mat _final_result_each_order;

private:
    virtual void set_parameters() = 0;
    virtual vec cluster_evolution(int cce_order, int index) = 0;

    void job_distribution();
    void DataGathering(mat &resMat, int cce_order, int clst_num);
    void cce_coherence_reduction();
    void compuate_final_coherence();
    void export_mat_file();
};
