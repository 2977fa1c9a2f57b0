// ensnvnbath_demo.cpp -- the reference application EnsNVnBath's main
// (src/application/EnsNVnBath.cpp:13-60, its path set-up :84-104 and its
// helpers :164-194: an NV centre in a nuclear-spin bath read from a file)
// written against liboops_gb300's C++ layer (include/oops_host.hpp): the
// same five steps, classes and calls, with arma/boost type names in
// namespace oops and without MPI (one process per GPU) or the logging
// library.  The bath file is INPUT_PATH + --input, INPUT_PATH being
// $CCE_PROJ_PATH/dat/input/ (else the working directory's dat/input/), as
// the application sets it.
//
//   ensnvnbath_demo [--bath-only] <EnsNVnBath options>
//
// Prints one JSON object for the tests: the bath read (full precision), the
// connection-matrix size, the clusters per order and the "output" option,
// and (without --bath-only, which stops after step 3 and needs no device)
// the time list and the final coherence per order.  Exit status 2 on an
// oops::Error.
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "oops_host.hpp"

using namespace oops;
using std::string;

static string PROJECT_PATH, INPUT_PATH, OUTPUT_PATH;

NVCenter create_defect_center(const variables_map &para);
cSpinSourceFromFile create_spin_bath_from_file(const variables_map &para);
cDepthFirstPathTracing create_spin_cluster_algrithm(const variables_map &para, const cSpinCollection &bath_spins);

static void set_paths()
{
    const char *env_path = std::getenv("CCE_PROJ_PATH");
    if (env_path != NULL) {
        PROJECT_PATH = env_path;
    } else {
        char pwd[500];
        if (!getcwd(pwd, sizeof(pwd))) pwd[0] = '\0';
        PROJECT_PATH = pwd;
    }
    INPUT_PATH = PROJECT_PATH + "/dat/input/";
    OUTPUT_PATH = PROJECT_PATH + "/dat/output/";
}

static void print_json(EnsembleCCE &sol, const cSpinCollection &bath, const sp_mat &c,
                       const cDepthFirstPathTracing &dfpt, const string &output, bool with_results);

int main(int argc, char *argv[])
{
    bool bath_only = argc > 1 && std::strcmp(argv[1], "--bath-only") == 0;
    if (bath_only) {
        argv[1] = argv[0];
        ++argv;
        --argc;
    }
    try {
        variables_map para = ensnvnbath_options(argc, argv);
        set_paths();
        int worker_num(1), my_rank(0);

        EnsembleCCE sol(my_rank, worker_num, para);

        NVCenter nv = create_defect_center(para);
        sol.set_defect_center(&nv);

        cSpinSourceFromFile src = create_spin_bath_from_file(para);
        sol.set_bath_spin(&src);

        cSpinCollection bath_spins = sol.getSpinCollecion();
        cDepthFirstPathTracing dfpt = create_spin_cluster_algrithm(para, bath_spins);
        sol.set_bath_cluster(&dfpt);

        if (!bath_only) {
            sol.run_each_clusters();

            sol.post_treatment();
        }
        dfpt.generate();
        print_json(sol, bath_spins, bath_spins.getConnectionMatrix(para["cutoff"].as<double>()), dfpt,
                   para["output"].as<string>(), !bath_only);
    } catch (const Error &e) {
        std::cerr << "oops::Error " << e.status() << ": " << e.what() << std::endl;
        return 2;
    }
    return 0;
}

NVCenter create_defect_center(const variables_map &para)
{
    vec coord(para["position"].as<string>());
    vec magB(para["magnetic_field"].as<string>());

    NVCenter nv(NVCenter::N14, coord);
    nv.set_magB(magB);
    nv.make_espin_hamiltonian();

    return nv;
}

cSpinSourceFromFile create_spin_bath_from_file(const variables_map &para)
{
    string input_filename = INPUT_PATH + para["input"].as<string>();
    cSpinSourceFromFile spin_file(input_filename);
    return spin_file;
}

cDepthFirstPathTracing create_spin_cluster_algrithm(const variables_map &para, const cSpinCollection &bath_spins)
{
    double cut_off_dist = para["cutoff"].as<double>();
    int max_order = para["cce"].as<int>();
    sp_mat c = bath_spins.getConnectionMatrix(cut_off_dist);
    cDepthFirstPathTracing dfpt(c, max_order);
    return dfpt;
}

static void print_json(EnsembleCCE &sol, const cSpinCollection &bath, const sp_mat &c,
                       const cDepthFirstPathTracing &dfpt, const string &output, bool with_results)
{
    char buf[64];
    auto num = [&](double x) {
        std::snprintf(buf, sizeof buf, "%.17g", x);
        return string(buf);
    };
    std::cout << "{\"coords\": [";
    const mat xyz = bath.getCoordinateMat();
    for (size_t i = 0; i < xyz.n_rows; ++i)
        std::cout << (i ? ", " : "") << "[" << num(xyz(i, 0)) << ", " << num(xyz(i, 1)) << ", "
                  << num(xyz(i, 2)) << "]";
    std::cout << "], \"isotope\": \"" << (bath.getSpinNum() ? bath.getSpinList()[0].get_isotope() : "")
              << "\", \"output\": \"" << output << "\", \"connections\": " << c.n_nonzero()
              << ", \"clusters\": [";
    const auto idx = dfpt.get_cluster_index_mat();
    for (size_t o = 0; o < idx.size(); ++o) {
        std::cout << (o ? ", " : "") << "[";
        for (size_t q = 0; q < idx[o].size(); ++q) std::cout << (q ? ", " : "") << idx[o][q];
        std::cout << "]";
    }
    std::cout << "]";
    if (with_results) {
        const std::vector<double> &t = sol.getTimeList();
        std::cout << ", \"time\": [";
        for (size_t i = 0; i < t.size(); ++i) std::cout << (i ? ", " : "") << num(t[i]);
        const mat f = sol.getFinalResult();
        std::cout << "], \"final\": [";
        for (size_t o = 0; o < f.n_cols; ++o) {
            std::cout << (o ? ", " : "") << "[";
            for (size_t i = 0; i < f.n_rows; ++i) std::cout << (i ? ", " : "") << num(f(i, o));
            std::cout << "]";
        }
        std::cout << "]";
    }
    std::cout << "}" << std::endl;
}
