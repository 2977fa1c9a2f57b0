// host_demo.cpp -- drives the C++ host layer (include/oops_host.hpp) the way
// the reference's own C++ drives its classes, for the parity tests:
//
//   host_demo expv <in> <out>   KronProd / SumKronProd / MatExpVector
//   host_demo cce  <in> <out> [mat]
//                               EnsembleCCE: set_bath_spin, set_bath_cluster,
//                               run_each_clusters, post_treatment, and with a
//                               fourth argument export_mat_file(mat)
//   host_demo --help            usage only (no device call)
//
// Inputs and outputs are whitespace-separated text written and read by
// tests/test_cpp_host.py.  Exit status 0 on success, 2 on an oops::Error (its
// status and message on stderr), 1 on bad usage or input.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>

#include "oops_host.hpp"

using oops::cx_double;

static int usage()
{
    std::cout << "usage: host_demo expv|cce <input> <output> [cce: <matfile>]\n";
    return 1;
}

// expv input: nspin; spin_dim[nspin]; nterm; per term: coeff nbody, then per
// body: pos dim and dim*dim (re im) column-major; v: N (re im); nt; t[nt];
// m tol.  Output: N x nt (re im), column-major.
static int run_expv(std::istream &in, std::ostream &out)
{
    size_t nspin, nterm;
    in >> nspin;
    std::vector<size_t> dims(nspin);
    for (auto &d : dims) in >> d;
    in >> nterm;
    oops::SumKronProd skp;
    for (size_t t = 0; t < nterm; ++t) {
        double coeff;
        size_t nbody;
        in >> coeff >> nbody;
        std::vector<size_t> idx(nbody);
        std::vector<oops::cx_mat> mats;
        for (size_t b = 0; b < nbody; ++b) {
            size_t pos, dim;
            in >> pos >> dim;
            idx[b] = pos;
            oops::cx_mat m(dim, dim);
            for (size_t e = 0; e < dim * dim; ++e) {
                double re, im;
                in >> re >> im;
                m.mem[e] = cx_double(re, im);
            }
            mats.push_back(m);
        }
        oops::KronProd kp(dims);
        kp.fill(idx, coeff, mats);
        skp.append(kp);
    }
    const size_t N = skp.getDim();
    std::vector<cx_double> v(N);
    for (auto &x : v) {
        double re, im;
        in >> re >> im;
        x = cx_double(re, im);
    }
    size_t nt;
    in >> nt;
    std::vector<double> tl(nt);
    for (auto &t : tl) in >> t;
    size_t m;
    double tol;
    in >> m >> tol;
    if (!in) return 1;
    oops::MatExpVector expv(skp, v, tl, oops::MatExpVector::InexplicitGPU);
    expv.krylov_m = m;
    expv.krylov_tol = tol;
    oops::cx_mat w = expv.run();
    out << std::setprecision(17);
    for (const cx_double &z : w.mem) out << z.real() << " " << z.imag() << "\n";
    return 0;
}

// cce input: B[3] cutoff max_order pulse_num t1 nTime precision nbath, then
// nbath x 3 coordinates, then optionally dephasing_rate axis[3] pol[3].
// Output: counts[max_order], then final_result and final_result_each_order
// (nTime x max_order, column-major).
static int run_cce(std::istream &in, std::ostream &out, const char *matfile)
{
    oops::CCEParameters p;
    size_t nbath;
    in >> p.magB[0] >> p.magB[1] >> p.magB[2] >> p.cut_off_dist >> p.max_order >> p.pulse_num >> p.t1 >>
        p.nTime >> p.precision >> nbath;
    std::vector<std::array<double, 3>> coords(nbath);
    for (auto &c : coords) in >> c[0] >> c[1] >> c[2];
    if (!in) return 1;
    double rate;
    if (in >> rate) {
        p.dephasing_rate = rate;
        in >> p.dephasing_axis[0] >> p.dephasing_axis[1] >> p.dephasing_axis[2] >> p.polarization[0] >>
            p.polarization[1] >> p.polarization[2];
        if (!in) return 1;
    }
    oops::EnsembleCCE cce(p);
    cce.set_bath_spin(coords);
    cce.set_bath_cluster();
    cce.run_each_clusters();
    cce.post_treatment();
    if (matfile) cce.export_mat_file(matfile);
    out << std::setprecision(17);
    for (int o = 0; o < p.max_order; ++o) out << cce.getClusterNum(o) << "\n";
    for (double x : cce.getFinalResult().mem) out << x << "\n";
    for (double x : cce.getFinalResultEachOrder().mem) out << x << "\n";
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 2 && std::strcmp(argv[1], "--help") == 0) return usage() - 1;
    if (argc != 4 && !(argc == 5 && std::strcmp(argv[1], "cce") == 0)) return usage();
    std::ifstream in(argv[2]);
    std::ofstream out(argv[3]);
    if (!in || !out) return usage();
    try {
        if (std::strcmp(argv[1], "expv") == 0) return run_expv(in, out);
        if (std::strcmp(argv[1], "cce") == 0) return run_cce(in, out, argc == 5 ? argv[4] : nullptr);
    } catch (const oops::Error &e) {
        std::cerr << "oops::Error " << e.status() << ": " << e.what() << "\n";
        return 2;
    }
    return usage();
}
