// ref_cce_pin.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own CCE
// reduction, src/source/app/cce.cpp (compiled from the read-only reference
// tree by oracle/build_ref.sh against oracle/ref_shim/include/app/cce.h and
// oracle/ref_shim/armadillo), on cluster curves given in a file, so that
// tests/golden/make_reference_reduction.py can record its results as
// fixtures:
//
//   ref_cce_pin <xyz file> <cutoff> <max_order> <nT> <curves in> <results out>
//
// The clusters come from the reference's own enumeration (cSpinSourceFromFile
// -> cSpinCollection -> cDepthFirstPathTracing -> cSpinCluster, as in
// ref_pin.cpp).  <curves in> holds, order by order, every cluster's nT
// values of L_C(t) (cluster-major, float64, the enumeration's order).
// A class derived from the reference's CCE takes them as its per-order
// result matrices and calls post_treatment(), i.e. cce_coherence_reduction
// and compuate_final_coherence (cce.cpp:151-189).  <results out> receives,
// in float64: order by order the reduced curves L~_C (cluster-major), then
// the per-order products and the cumulative products (order-major, nT each).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "include/app/cce.h"

// the application headers define the spin database (include/app/app.h:13)
cSPINDATA SPIN_DATABASE = cSPINDATA();

namespace {

class PinCCE : public CCE {
public:
    PinCCE() : CCE(0, 1, po::variables_map()) {}
    void load(const cSpinCluster &clusters, int max_order, int nT, const std::vector<mat> &curves)
    {
        _spin_clusters = clusters;
        _max_order = max_order;
        _nTime = nT;
        _cce_evovle_result = curves;
    }
    const std::vector<mat> &tilde() const { return _cce_evovle_result_tilder; }
    const mat &each_order() const { return _final_result_each_order; }
    const mat &cumulative() const { return _final_result; }

private:
    void set_parameters() override {}
    vec cluster_evolution(int, int) override { return vec(); }
};

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: ref_cce_pin <xyz> <cutoff> <max_order> <nT> <curves in> <results out>\n");
        return 1;
    }
    const double cutoff = std::atof(argv[2]);
    const int max_order = std::atoi(argv[3]);
    const int nT = std::atoi(argv[4]);
    cSpinSourceFromFile src(argv[1]);
    cSpinCollection bath(&src);
    bath.make();
    sp_mat c = bath.getConnectionMatrix(cutoff);
    cDepthFirstPathTracing dfpt(c, max_order);
    cSpinCluster clusters(bath, &dfpt);
    clusters.make();

    FILE *in = std::fopen(argv[5], "rb");
    if (!in) { std::perror(argv[5]); return 1; }
    std::vector<mat> curves;
    for (int o = 0; o < max_order; ++o) {
        const size_t n = clusters.getClusterNum(o);
        mat L(nT, n);
        if (std::fread(L.memptr(), sizeof(double), (size_t)nT * n, in) != (size_t)nT * n) {
            std::fprintf(stderr, "ref_cce_pin: %s is too short at order %d\n", argv[5], o);
            return 1;
        }
        curves.push_back(L);
    }
    std::fclose(in);

    PinCCE pin;
    pin.load(clusters, max_order, nT, curves);
    pin.post_treatment();

    FILE *out = std::fopen(argv[6], "wb");
    if (!out) { std::perror(argv[6]); return 1; }
    for (int o = 0; o < max_order; ++o)
        std::fwrite(pin.tilde()[o].memptr(), sizeof(double), pin.tilde()[o].n_elem, out);
    std::fwrite(pin.each_order().memptr(), sizeof(double), pin.each_order().n_elem, out);
    std::fwrite(pin.cumulative().memptr(), sizeof(double), pin.cumulative().n_elem, out);
    std::fclose(out);
    std::printf("counts");
    for (int o = 0; o < max_order; ++o) std::printf(" %zu", clusters.getClusterNum(o));
    std::printf("\n");
    return 0;
}
