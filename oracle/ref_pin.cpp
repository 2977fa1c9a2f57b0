// ref_pin.cpp -- TEST INFRASTRUCTURE ONLY.  A driver that links the
// reference's own spin, cluster and physics sources (compiled from the
// read-only reference tree by oracle/build_ref.sh, with oracle/ref_shim/
// armadillo standing in for armadillo) and prints their results as plain
// text, so that tests/golden/make_golden.py can record them as fixtures:
//
//   ref_pin enum <xyz file> <cutoff> <max_order>
//       cSpinSourceFromFile -> cSpinCollection::make / getConnectionMatrix ->
//       cDepthFirstPathTracing -> cSpinCluster::make; per order the count,
//       then per cluster its sorted spin indices and getSubClusters' set of
//       (order, position) pairs (SpinCollection.cpp:31-57,
//       SpinClusterAlgorithm.cpp:75-148, SpinCluster.cpp:9-98)
//   ref_pin phys <xyz file> <npairs> <Bx> <By> <Bz>
//       dipole() of the first npairs spin pairs (i < j in order),
//       zeeman() of every spin and Pulse_Interval("CPMG", n), n = 1..8
//       (misc.cpp:11-84), all in %.17g
//   ref_pin random <range> <max_num> <num> <isotope> <seed>
//       cSpinSourceUniformRandom::generate (SpinSource.cpp:112-129) over the
//       stand-in's armadillo C++11 generator: every spin's isotope and
//       coordinates in %.17g
#include <cstdio>
#include <cstdlib>
#include <set>
#include <string>
#include <vector>

#include "include/misc/misc.h"
#include "include/spin/SpinCluster.h"
#include "include/spin/SpinClusterAlgorithm.h"
#include "include/spin/SpinCollection.h"
#include "include/spin/SpinSource.h"

// the application headers define the spin database (include/app/app.h:13)
cSPINDATA SPIN_DATABASE = cSPINDATA();

static int run_enum(const char *file, double cutoff, int max_order)
{
    cSpinSourceFromFile src(file);
    cSpinCollection bath(&src);
    bath.make();
    sp_mat c = bath.getConnectionMatrix(cutoff);
    cDepthFirstPathTracing dfpt(c, max_order);
    cSpinCluster clusters(bath, &dfpt);
    clusters.make();
    std::printf("nspin %zu\n", bath.getSpinNum());
    for (int o = 0; o < max_order; ++o) {
        const size_t n = clusters.getClusterNum(o);
        std::printf("order %d %zu\n", o, n);
        for (size_t i = 0; i < n; ++i) {
            uvec idx = clusters.getClusterIndex(o, i).getIndex();
            std::printf("c");
            for (size_t a = 0; a < idx.n_elem; ++a) std::printf(" %llu", (unsigned long long)idx[a]);
            std::set<ClusterPostion> sub = clusters.getSubClusters(o, i);
            std::printf(" | %zu", sub.size());
            for (const ClusterPostion &p : sub) std::printf(" %zu %zu", p.first, p.second);
            std::printf("\n");
        }
    }
    return 0;
}

static int run_phys(const char *file, int npairs, double bx, double by, double bz)
{
    cSpinSourceFromFile src(file);
    std::vector<cSPIN> spins = src.generate();
    vec B;
    B << bx << by << bz;
    int done = 0;
    for (size_t i = 0; i < spins.size() && done < npairs; ++i)
        for (size_t j = i + 1; j < spins.size() && done < npairs; ++j, ++done) {
            vec d = dipole(spins[i], spins[j]);
            std::printf("dip %zu %zu", i, j);
            for (size_t a = 0; a < d.n_elem; ++a) std::printf(" %.17g", d[a]);
            std::printf("\n");
        }
    for (size_t i = 0; i < spins.size(); ++i) {
        vec z = zeeman(spins[i], B);
        std::printf("zee %zu", i);
        for (size_t a = 0; a < z.n_elem; ++a) std::printf(" %.17g", z[a]);
        std::printf("\n");
    }
    for (int n = 1; n <= 8; ++n) {
        std::vector<double> iv = Pulse_Interval("CPMG", n);
        std::printf("cpmg %d", n);
        for (double x : iv) std::printf(" %.17g", x);
        std::printf("\n");
    }
    return 0;
}

static int run_random(double range, int max_num, int num, const char *isotope, int seed)
{
    cSpinSourceUniformRandom src(range, max_num, num, isotope, seed);
    std::vector<cSPIN> spins = src.generate();
    for (const cSPIN &s : spins) {
        vec c = s.get_coordinate();
        std::printf("spin %s %.17g %.17g %.17g\n", s.get_isotope().c_str(), c[0], c[1], c[2]);
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 5 && std::string(argv[1]) == "enum")
        return run_enum(argv[2], std::atof(argv[3]), std::atoi(argv[4]));
    if (argc == 7 && std::string(argv[1]) == "phys")
        return run_phys(argv[2], std::atoi(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atof(argv[6]));
    if (argc == 7 && std::string(argv[1]) == "random")
        return run_random(std::atof(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), argv[5], std::atoi(argv[6]));
    std::fprintf(stderr, "usage: ref_pin enum <xyz> <cutoff> <max_order> | phys <xyz> <npairs> <Bx> <By> <Bz> | "
                         "random <range> <max_num> <num> <isotope> <seed>\n");
    return 1;
}
