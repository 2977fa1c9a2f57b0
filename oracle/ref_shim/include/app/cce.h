// TEST INFRASTRUCTURE ONLY.  Stand-in for the reference's application header
// src/include/app/cce.h, found ahead of it on oracle/build_ref.sh's include
// path so that the reference's own src/source/app/cce.cpp, ensemble_cce.cpp
// and single_sample_cce.cpp compile without boost, MPI or the XML reader (the
// stand-in include/oops.h replaces those).  It declares the CCE base class
// with the members and methods those files define and use, with the
// reference's names and types, over the reference's own DefectCenter,
// PureState and spin classes.  The pins (oracle/ref_cce_pin.cpp,
// oracle/ref_ensemble_pin.cpp, oracle/ref_single_pin.cpp) derive from CCE,
// EnsembleCCE or SingleSampleCCE, run one rank (job_distribution and
// DataGathering then make no MPI call) and read the protected results;
// export_mat_file is compiled without HAS_MATLAB.
#pragma once

#include "include/oops.h"
#include "include/app/DefectCenter.h"

extern string INPUT_PATH;
extern string OUTPUT_PATH;

namespace po = boost::program_options;

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

    cSPIN getCenterSpin() const { return _center_spin; }
    cSpinCollection getSpinCollecion() const { return _bath_spins; }
    cSpinCluster getSpinClusters() const { return _my_clusters; }
    vector<mat> getResultMatrix() const { return _cce_evovle_result; }

protected:
    // I/O
    po::variables_map _para;
    ConfigXML _cfg;
    string _bath_spin_filename;
    string _result_filename;

    // defect centre
    DefectCenter *_defect_center = nullptr;
    string _center_spin_name;
    cSPIN _center_spin;
    int _state_idx0 = 0;
    int _state_idx1 = 1;
    pair<PureState, PureState> _state_pair;

    // spin bath
    double _cut_off_dist = 0.0;
    int _max_order = 0;
    cSpinSource *_spin_source = nullptr;
    cSpinGrouping *_spin_grouping = nullptr;
    cSpinCollection _bath_spins;
    cSpinCluster _spin_clusters;

    // conditions
    vec _magB;
    string _pulse_name;
    int _pulse_num = 1;
    double _t0 = 0.0;
    double _t1 = 0.0;
    int _nTime = 0;
    vec _time_list;

    // MPI
    int _my_rank = 0;
    int _worker_num = 1;
    cSpinCluster _my_clusters;

    // results
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
