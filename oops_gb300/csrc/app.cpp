// app.cpp -- the reference application's classes over liboops_gb300 (host C++):
// options map, spins and spin sources, the spin collection and its connection
// matrix, cluster growth, the NV centre, and the EnsembleCCE constructor and
// set-up steps that src/application/EnsNVeBath.cpp:40-62 calls.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>

#include "oops_host.hpp"

namespace oops {

namespace {

void check(int rc, const char *what)
{
    if (rc != OOPS_OK) throw Error(rc, std::string(what) + ": " + oops_last_error());
}

struct IsotopeData {
    const char *name;
    int multiplicity;
    double gamma, omegaQ;
};

// src/source/spin/Spin/SpinData.cpp:4-18 (the table's "14C"/"15C" keys hold
// the nitrogen data; "14N"/"15N" name the same entries here)
const IsotopeData kIsotopes[] = {
    {"13C", 2, 6.728284e7, 0.0},       {"14C", 3, 1.9337792e7, 2.96},
    {"15C", 2, -2.71261804e7, 0.0},    {"E", 2, -1.760859708e11, 0.0},
    {"NVe", 3, -1.760859708e11, 2.87e3}, {"14N", 3, 1.9337792e7, 2.96},
    {"15N", 2, -2.71261804e7, 0.0},
};

// The applications' option tables: long name, short name, default; the
// "output" default is the application's name followed by its command line,
// as both build it (EnsNVeBath.cpp:80-85, EnsNVnBath.cpp:74-79).
struct OptionDef {
    const char *name, *shortname, *def;
};
// EnsNVeBath (src/application/EnsNVeBath.cpp:121-151), then this library's two
const OptionDef kOptions[] = {
    {"input", "i", "None"},           {"output", "o", ""},
    {"logfile", "l", "EnsembleCCE.conf"},
    {"position", "P", "0.0 0.0 0.0"}, {"state0", "a", "0"},
    {"state1", "b", "1"},             {"cce", "c", "3"},
    {"cutoff", "d", "300.0"},         {"polarization", "z", "0.0 0.0 0.0"},
    {"dephasing_rate", "r", "10000.0"}, {"dephasing_axis", "x", "1.0 1.0 1.0"},
    {"length", "L", "3.57"},          {"num_cell", "u", "8"},
    {"concentration", "C", "1.0"},    {"max_number", "M", "2000"},
    {"number", "N", "100"},           {"seed", "D", "1"},
    {"isotope", "", "E"},             {"coord_file", "F", "coord.xyz"},
    {"nTime", "n", "101"},            {"start", "s", "0.0"},
    {"finish", "f", "0.0002"},        {"magnetic_field", "B", "0.1 0.1 0.1"},
    {"pulse", "p", "CPMG"},           {"pulse_num", "m", "1"},
    {"precision", "", "fp64"},        {"output_dir", "", ""},
};
// EnsNVnBath (src/application/EnsNVnBath.cpp:116-139), then this library's two
const OptionDef kNBathOptions[] = {
    {"input", "i", "C13Bath/RoyCoord.xyz"}, {"output", "o", ""},
    {"logfile", "l", "EnsembleCCE.conf"},
    {"position", "P", "0.0 0.0 0.0"}, {"state0", "a", "0"},
    {"state1", "b", "1"},             {"cce", "c", "3"},
    {"cutoff", "d", "6.0"},           {"polarization", "z", "0.0 0.0 0.0"},
    {"dephasing_rate", "r", "0.0"},   {"dephasing_axis", "x", "1.0 1.0 1.0"},
    {"range", "g", "1000.0"},         {"number", "N", "100"},
    {"seed", "D", "1"},               {"isotope", "", "E"},
    {"nTime", "n", "101"},            {"start", "s", "0.0"},
    {"finish", "f", "0.002"},         {"magnetic_field", "B", "0.1 0.1 0.1"},
    {"pulse", "p", "CPMG"},           {"pulse_num", "m", "1"},
    {"precision", "", "fp64"},        {"output_dir", "", ""},
};

double dist(const vec &a, const vec &b)
{
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

// ---------------------------------------------------------------- vec, options
vec::vec(const std::string &text)
{
    std::istringstream in(text);
    double x;
    while (in >> x) v_.push_back(x);
    if (!in.eof()) throw Error(OOPS_ERR_ARG, "vec: cannot parse \"" + text + "\"");
}

template <>
int variable_value::as<int>() const
{
    size_t pos = 0;
    int v = std::stoi(text_, &pos);
    if (pos != text_.size()) throw Error(OOPS_ERR_ARG, "option value is not an integer: " + text_);
    return v;
}
template <>
double variable_value::as<double>() const
{
    size_t pos = 0;
    double v = std::stod(text_, &pos);
    if (pos != text_.size()) throw Error(OOPS_ERR_ARG, "option value is not a number: " + text_);
    return v;
}
template <>
std::string variable_value::as<std::string>() const
{
    return text_;
}

const variable_value &variables_map::operator[](const std::string &key) const
{
    auto it = m_.find(key);
    if (it == m_.end()) throw Error(OOPS_ERR_ARG, "unknown option: " + key);
    return it->second;
}

std::vector<std::string> variables_map::keys() const
{
    std::vector<std::string> k;
    for (const auto &kv : m_) k.push_back(kv.first);
    return k;
}

namespace {
template <size_t N>
variables_map parse_options(const OptionDef (&table)[N], const char *app, int argc, const char *const *argv)
{
    variables_map vm;
    for (const OptionDef &o : table) vm.set(o.name, o.def);
    std::string output = app;
    for (int i = 1; i < argc; ++i) output += argv[i];
    vm.set("output", output);
    auto lookup = [&table](const std::string &name, bool is_short) -> const OptionDef * {
        for (const OptionDef &o : table)
            if ((is_short ? std::string(o.shortname) : std::string(o.name)) == name && !name.empty()) return &o;
        return nullptr;
    };
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i], value;
        const OptionDef *o = nullptr;
        if (a.rfind("--", 0) == 0) {
            std::string name = a.substr(2);
            const size_t eq = name.find('=');
            if (eq != std::string::npos) {
                value = name.substr(eq + 1);
                name = name.substr(0, eq);
                o = lookup(name, false);
                if (!o) throw Error(OOPS_ERR_ARG, "unknown option --" + name);
                vm.set(o->name, value);
                continue;
            }
            o = lookup(name, false);
        } else if (a.size() == 2 && a[0] == '-') {
            o = lookup(a.substr(1), true);
        }
        if (!o) throw Error(OOPS_ERR_ARG, "unknown option " + a);
        if (i + 1 >= argc) throw Error(OOPS_ERR_ARG, "option " + a + " needs a value");
        vm.set(o->name, argv[++i]);
    }
    return vm;
}
}  // namespace

variables_map ensnvebath_options(int argc, const char *const *argv)
{
    return parse_options(kOptions, "EnsNVeBath", argc, argv);
}

variables_map ensnvnbath_options(int argc, const char *const *argv)
{
    return parse_options(kNBathOptions, "EnsNVnBath", argc, argv);
}

// ---------------------------------------------------------------- spins
cSPIN::cSPIN(vec coord, const std::string &isotope) : coordinate_(std::move(coord)), isotope_(isotope)
{
    for (const IsotopeData &d : kIsotopes)
        if (isotope == d.name) {
            multiplicity_ = d.multiplicity;
            gamma_ = d.gamma;
            omegaQ_ = d.omegaQ;
            return;
        }
    throw Error(OOPS_ERR_ARG, "cSPIN: unknown isotope \"" + isotope + "\"");
}

void cSpinSource::export_coordinates(const std::string &filename)
{
    std::ofstream f(filename);
    if (!f) throw Error(OOPS_ERR_ARG, "export_coordinates: cannot open " + filename);
    f << spin_list.size() << std::endl;
    for (const cSPIN &s : spin_list) {
        const vec c = s.get_coordinate();
        f << s.get_isotope() << "\t" << c[0] << "\t" << c[1] << "\t" << c[2] << std::endl;
    }
}

std::vector<cSPIN> &cSpinSourceFromFile::generate()
{
    std::ifstream f(filename_);
    if (!f) throw Error(OOPS_ERR_ARG, "cSpinSourceFromFile: cannot open " + filename_);
    int n = 0;
    if (!(f >> n) || n < 0) throw Error(OOPS_ERR_ARG, "cSpinSourceFromFile: bad spin count in " + filename_);
    spin_list.clear();
    for (int i = 0; i < n; ++i) {
        std::string iso;
        double x, y, z;
        if (!(f >> iso >> x >> y >> z)) throw Error(OOPS_ERR_ARG, "cSpinSourceFromFile: short file " + filename_);
        spin_list.push_back(cSPIN(vec{x, y, z}, iso));
    }
    return spin_list;
}

std::vector<cSPIN> &cSpinSourceUniformRandom::generate()
{
    if (num_ > max_num_ || num_ < 0) throw Error(OOPS_ERR_ARG, "cSpinSourceUniformRandom: num must be 0..max_num");
    std::mt19937_64 eng((std::mt19937_64::result_type)seed_);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::vector<double> m(3 * (size_t)max_num_);  // 3 x max_num, column-major
    for (double &x : m) x = u(eng);
    std::vector<double> d(max_num_);
    for (int i = 0; i < max_num_; ++i) {
        const double x = 2.0 * range_ * m[3 * i] - range_, y = 2.0 * range_ * m[3 * i + 1] - range_,
                     z = 2.0 * range_ * m[3 * i + 2] - range_;
        d[i] = std::sqrt(x * x + y * y + z * z);
    }
    std::vector<size_t> idx(max_num_);
    for (int i = 0; i < max_num_; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return d[a] < d[b]; });
    spin_list.clear();
    for (int i = 0; i < num_; ++i) {
        const size_t c = idx[i];
        spin_list.push_back(cSPIN(vec{2.0 * range_ * m[3 * c] - range_, 2.0 * range_ * m[3 * c + 1] - range_,
                                      2.0 * range_ * m[3 * c + 2] - range_},
                                  isotope_));
    }
    return spin_list;
}

// ---------------------------------------------------------------- collection
double sp_mat::operator()(size_t i, size_t j) const
{
    if (i >= n_rows || j >= n_cols) throw Error(OOPS_ERR_ARG, "sp_mat: index out of range");
    return std::binary_search(cols.begin() + row_off[i], cols.begin() + row_off[i + 1], (unsigned)j) ? 1.0 : 0.0;
}

void cSpinCollection::make()
{
    if (!source_) throw Error(OOPS_ERR_ARG, "cSpinCollection: no spin source");
    spin_list_ = source_->generate();
}

mat cSpinCollection::getCoordinateMat() const
{
    mat r(spin_list_.size(), 3);
    for (size_t i = 0; i < spin_list_.size(); ++i)
        for (int a = 0; a < 3; ++a) r(i, a) = spin_list_[i].get_coordinate()[a];
    return r;
}

mat cSpinCollection::getDistanceMatrix() const
{
    const size_t n = spin_list_.size();
    mat d(n, n);
    for (size_t i = 0; i < n; ++i)
        for (size_t j = i; j < n; ++j)
            d(i, j) = d(j, i) = dist(spin_list_[i].get_coordinate(), spin_list_[j].get_coordinate());
    return d;
}

sp_mat cSpinCollection::getConnectionMatrix(double threshold) const
{
    const size_t n = spin_list_.size();
    sp_mat c;
    c.n_rows = c.n_cols = n;
    c.row_off.assign(n + 1, 0);
    for (size_t i = 0; i < n; ++i) {
        const vec ci = spin_list_[i].get_coordinate();
        for (size_t j = 0; j < n; ++j)
            if (j != i && dist(ci, spin_list_[j].get_coordinate()) <= threshold) c.cols.push_back((unsigned)j);
        c.row_off[i + 1] = c.cols.size();
    }
    return c;
}

// ---------------------------------------------------------------- grouping
cSpinGrouping::~cSpinGrouping() = default;

void cDepthFirstPathTracing::generate()
{
    if (max_order_ < 1) throw Error(OOPS_ERR_ARG, "cDepthFirstPathTracing: max order must be >= 1");
    oops_clusters *h = nullptr;
    check(oops_clusters_enumerate_graph(c_.n_rows, c_.row_off.data(), c_.cols.data(), (int)max_order_, &h),
          "cDepthFirstPathTracing::generate");
    index_.assign(max_order_, {});
    for (size_t o = 0; o < max_order_; ++o) {
        index_[o].resize(oops_clusters_count(h, (int)o) * (o + 1));
        if (!index_[o].empty()) oops_clusters_indices(h, (int)o, index_[o].data());
    }
    oops_clusters_destroy(h);
}

// ---------------------------------------------------------------- NV centre
vec DefectCenter::get_spin_vector(int i) const
{
    if (i < 0 || 3 * (size_t)i + 2 >= svec_.size()) throw Error(OOPS_ERR_ARG, "DefectCenter: make_espin_hamiltonian() first");
    return vec{svec_[3 * i], svec_[3 * i + 1], svec_[3 * i + 2]};
}

NVCenter::NVCenter(NVNuclearSpin nuc) : NVCenter(nuc, vec{0.0, 0.0, 0.0}) {}

NVCenter::NVCenter(NVNuclearSpin nuc, vec coord)
{
    if (coord.n_elem() != 3) throw Error(OOPS_ERR_ARG, "NVCenter: the position needs three coordinates");
    const double dia4 = 3.57 / 4.0;  // DefectCenter.cpp:16
    nuclear_spin_ = cSPIN(coord, nuc == N14 ? "14N" : "15N");
    electron_spin_ = cSPIN(vec{coord[0] + dia4, coord[1] + dia4, coord[2] + dia4}, "NVe");
}

void NVCenter::make_espin_hamiltonian()
{
    if (magB_.n_elem() != 3) throw Error(OOPS_ERR_ARG, "NVCenter: the field needs three components");
    double B[3] = {magB_[0], magB_[1], magB_[2]}, ev[3], sv[9];
    check(oops_nv_states(B, ev, sv), "NVCenter::make_espin_hamiltonian");
    evals_.assign(ev, ev + 3);
    svec_.assign(sv, sv + 9);
}

// ---------------------------------------------------------------- EnsembleCCE
namespace {
CCEParameters parameters_from(const variables_map &para)
{
    CCEParameters p;
    p.state_idx0 = para["state0"].as<int>();
    p.state_idx1 = para["state1"].as<int>();
    p.max_order = para["cce"].as<int>();
    p.cut_off_dist = para["cutoff"].as<double>();
    const vec pol(para["polarization"].as<std::string>());
    const vec ax(para["dephasing_axis"].as<std::string>());
    const vec B(para["magnetic_field"].as<std::string>());
    if (pol.n_elem() != 3 || ax.n_elem() != 3 || B.n_elem() != 3)
        throw Error(OOPS_ERR_ARG, "EnsembleCCE: polarization, dephasing_axis and magnetic_field need 3 values");
    for (int a = 0; a < 3; ++a) {
        p.polarization[a] = pol[a];
        p.dephasing_axis[a] = ax[a];
        p.magB[a] = B[a];
    }
    p.dephasing_rate = para["dephasing_rate"].as<double>();
    p.nTime = para["nTime"].as<int>();
    p.t0 = para["start"].as<double>();
    p.t1 = para["finish"].as<double>();
    const std::string pulse = para["pulse"].as<std::string>();
    if (pulse != "CPMG") throw Error(OOPS_ERR_UNSUPPORTED, "EnsembleCCE: pulse sequences other than CPMG");
    p.pulse_num = para["pulse_num"].as<int>();
    const std::string prec = para.count("precision") ? para["precision"].as<std::string>() : "fp64";
    if (prec == "fp64") p.precision = OOPS_PREC_FP64;
    else if (prec == "mixed") p.precision = OOPS_PREC_MIXED;
    else throw Error(OOPS_ERR_ARG, "EnsembleCCE: precision must be fp64 or mixed");
    return p;
}
}  // namespace

EnsembleCCE::EnsembleCCE(int my_rank, int worker_num, const variables_map &para)
    : EnsembleCCE(parameters_from(para))
{
    if (my_rank < 0 || worker_num < 1 || my_rank >= worker_num)
        throw Error(OOPS_ERR_ARG, "EnsembleCCE: rank must be 0..worker_num-1");
    my_rank_ = my_rank;
    output_name_ = para["output"].as<std::string>();
    output_dir_ = para.count("output_dir") ? para["output_dir"].as<std::string>() : "";
}

void EnsembleCCE::set_defect_center(DefectCenter *defect)
{
    if (!defect) throw Error(OOPS_ERR_ARG, "set_defect_center: null defect");
    const vec c = defect->get_espin().get_coordinate();
    const vec s0 = defect->get_spin_vector(para_.state_idx0), s1 = defect->get_spin_vector(para_.state_idx1);
    for (int a = 0; a < 3; ++a) {
        para_.center[a] = c[a];
        p_.center[a] = c[a];
        p_.sv0[a] = s0[a];
        p_.sv1[a] = s1[a];
    }
    p_.gamma_center = defect->get_espin().get_gamma();
}

void EnsembleCCE::set_bath_spin(cSpinSource *source)
{
    bath_spins_ = cSpinCollection(source);
    bath_spins_.make();
    const std::vector<cSPIN> spins = bath_spins_.getSpinList();
    std::vector<std::array<double, 3>> coords;
    for (const cSPIN &s : spins) {
        if (s.get_multiplicity() != 2)
            throw Error(OOPS_ERR_UNSUPPORTED, "EnsembleCCE: bath spins must be spin-1/2 (isotope " + s.get_isotope() + ")");
        if (s.get_gamma() != spins[0].get_gamma())
            throw Error(OOPS_ERR_UNSUPPORTED, "EnsembleCCE: one bath isotope per run");
        const vec c = s.get_coordinate();
        coords.push_back({c[0], c[1], c[2]});
    }
    if (!spins.empty()) p_.gamma_bath = spins[0].get_gamma();
    set_bath_spin(coords);
    if (my_rank_ == 0) std::cout << spins.size() << " spins are generated." << std::endl;
}

void EnsembleCCE::set_bath_cluster(cSpinGrouping *grouping)
{
    if (!grouping) throw Error(OOPS_ERR_ARG, "set_bath_cluster: null grouping");
    const sp_mat &c = grouping->getConnectionMatrix();
    if (c.n_rows != coords_.size() / 3)
        throw Error(OOPS_ERR_ARG, "set_bath_cluster: the connection matrix does not match the bath");
    if (grouping->getMaxOrder() < 1 || grouping->getMaxOrder() > 6)
        throw Error(OOPS_ERR_ARG, "set_bath_cluster: cluster order must be 1..6");
    para_.max_order = (int)grouping->getMaxOrder();
    if (clusters_) oops_clusters_destroy(clusters_);
    clusters_ = nullptr;
    check(oops_clusters_enumerate_graph(c.n_rows, c.row_off.data(), c.cols.data(), para_.max_order, &clusters_),
          "EnsembleCCE::set_bath_cluster");
    counts_.assign(para_.max_order, 0);
    for (int o = 0; o < para_.max_order; ++o) counts_[o] = oops_clusters_count(clusters_, o);
}

}  // namespace oops
