// ensnvebath_demo.cpp -- the reference application EnsNVeBath's main
// (src/application/EnsNVeBath.cpp:40-62 and its helpers :184-216) written
// against liboops_gb300's C++ layer (include/oops_host.hpp): the same five
// steps, classes and calls, with arma/boost type names in namespace oops and
// without MPI (one process per GPU) or the logging library.
//
//   ensnvebath_demo [--bath-only] <EnsNVeBath options>
//
// Prints one JSON object for the tests: the generated bath (full precision),
// the connection-matrix size and the clusters per order, and (without
// --bath-only, which stops after step 3 and needs no device) the time list and
// the final coherence per order.  Exit status 2 on an oops::Error.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "oops_host.hpp"

using namespace oops;
using std::string;

NVCenter create_defect_center(const variables_map &para);
cSpinSourceUniformRandom create_spin_source(const variables_map &para);
cDepthFirstPathTracing create_spin_cluster_algrithm(const variables_map &para, const cSpinCollection &bath_spins);

static void print_json(EnsembleCCE &sol, const cSpinCollection &bath, const sp_mat &c,
                       const cDepthFirstPathTracing &dfpt, bool with_results);

int main(int argc, char *argv[])
{
    bool bath_only = argc > 1 && std::strcmp(argv[1], "--bath-only") == 0;
    if (bath_only) {
        argv[1] = argv[0];
        ++argv;
        --argc;
    }
    try {
        variables_map para = ensnvebath_options(argc, argv);
        int worker_num(1), my_rank(0);

        EnsembleCCE sol(my_rank, worker_num, para);

        // Step 1: make a defect center
        NVCenter nv = create_defect_center(para);
        sol.set_defect_center(&nv);

        // Step 2: make bath spins
        cSpinSourceUniformRandom spinUR = create_spin_source(para);
        sol.set_bath_spin(&spinUR);
        if (!para["output_dir"].as<string>().empty())
            spinUR.export_coordinates(para["output_dir"].as<string>() + "/" + para["coord_file"].as<string>());

        // Step 3: make clusters
        cSpinCollection bath_spins = sol.getSpinCollecion();
        cDepthFirstPathTracing dfpt = create_spin_cluster_algrithm(para, bath_spins);
        sol.set_bath_cluster(&dfpt);

        if (!bath_only) {
            // Step 4: run_each_cluster
            sol.run_each_clusters();

            // Step 5: post_treatment
            sol.post_treatment();
        }
        dfpt.generate();
        print_json(sol, bath_spins, bath_spins.getConnectionMatrix(para["cutoff"].as<double>()), dfpt,
                   !bath_only);
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

cSpinSourceUniformRandom create_spin_source(const variables_map &para)
{
    double l0 = para["length"].as<double>();
    int num_in_cell = para["num_cell"].as<int>();
    double concentration = para["concentration"].as<double>();
    int max_num = para["max_number"].as<int>();
    int num = para["number"].as<int>();
    int seed = para["seed"].as<int>();
    string isotope = para["isotope"].as<string>();

    double range = 0.5e2 * l0 * std::pow(max_num / concentration / num_in_cell, 1.0 / 3.0);
    cSpinSourceUniformRandom spinUR(range, max_num, num, isotope, seed);
    return spinUR;
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
                       const cDepthFirstPathTracing &dfpt, bool with_results)
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
              << "\", \"connections\": " << c.n_nonzero() << ", \"clusters\": [";
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
