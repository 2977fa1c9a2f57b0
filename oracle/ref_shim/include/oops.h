// TEST INFRASTRUCTURE ONLY.  Stand-in for the reference's umbrella header
// src/include/oops.h, found ahead of it on oracle/build_ref.sh's include path.
// It includes the reference's own spin, Kronecker, misc and quantum headers
// as that header does, and replaces what the pins cannot link: MPI (the four
// calls CCE's job distribution names, which abort if called, since the pins
// run one rank), boost::program_options (a variables_map of strings whose
// values convert with as<T>(), as the application reads its options), the
// XML configuration reader (its getters over entries a pin sets) and the
// logging library (include/el stand-in).
#ifndef OOPS_H
#define OOPS_H

#include <algorithm>
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <armadillo>

#ifdef HAS_MATLAB
#include <mat.h>
#endif

#include "include/el/easylogging++.h"

// ---- MPI (one rank)
typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Status;
static const MPI_Datatype MPI_UNSIGNED = 1, MPI_DOUBLE = 2;
static const MPI_Comm MPI_COMM_WORLD = 0;
static MPI_Status *const MPI_STATUS_IGNORE = nullptr;
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm)
{
    std::fprintf(stderr, "reference pin: MPI_Send called in a one-rank pin\n");
    std::abort();
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *)
{
    std::fprintf(stderr, "reference pin: MPI_Recv called in a one-rank pin\n");
    std::abort();
}

// ---- boost::program_options: values kept as strings, converted on as<T>()
namespace boost {
namespace program_options {
struct variable_value {
    std::string text;
    template <typename T>
    T as() const
    {
        std::istringstream in(text);
        T v{};
        in >> v;
        return v;
    }
};
template <>
inline std::string variable_value::as<std::string>() const { return text; }
struct variables_map : std::map<std::string, variable_value> {
    const variable_value &operator[](const std::string &k) const
    {
        auto it = find(k);
        if (it == end()) {
            std::fprintf(stderr, "reference pin: option '%s' not set\n", k.c_str());
            std::abort();
        }
        return it->second;
    }
    void set(const std::string &k, const std::string &v) { std::map<std::string, variable_value>::operator[](k).text = v; }
};
}  // namespace program_options
}  // namespace boost

// ---- XML configuration: the reader's interface (src/include/misc/
// xmlreader.h) over (section, name) -> text entries that a pin sets instead
// of parsing a file; absent entries read as the reader's defaults (0, 0.0,
// "None"), vectors as whitespace-separated numbers
class ConfigXML {
public:
    void printParameters() const {}
    void set(const std::string &section, const std::string &name, const std::string &value)
    {
        _entries[section + "\n" + name] = value;
    }
    std::string getStringParameter(std::string section, std::string name) const
    {
        auto it = _entries.find(section + "\n" + name);
        return it == _entries.end() ? std::string("None") : it->second;
    }
    int getIntParameter(std::string section, std::string name) const
    {
        auto it = _entries.find(section + "\n" + name);
        return it == _entries.end() ? 0 : std::atoi(it->second.c_str());
    }
    double getDoubleParameter(std::string section, std::string name) const
    {
        auto it = _entries.find(section + "\n" + name);
        return it == _entries.end() ? 0.0 : std::strtod(it->second.c_str(), nullptr);
    }
    arma::vec getVectorParameter(std::string section, std::string name) const
    {
        std::istringstream in(getStringParameter(section, name));
        std::vector<double> v;
        for (double x; in >> x;) v.push_back(x);
        arma::vec out(v.size());
        for (size_t i = 0; i < v.size(); ++i) out(i) = v[i];
        return out;
    }

private:
    std::map<std::string, std::string> _entries;
};

#include "include/spin/Spin.h"
#include "include/spin/SpinCluster.h"
#include "include/spin/SpinClusterAlgorithm.h"
#include "include/spin/SpinCollection.h"
#include "include/spin/SpinData.h"
#include "include/spin/SpinInteraction.h"
#include "include/spin/SpinInteractionComponent.h"
#include "include/spin/SpinInteractionDefine.h"
#include "include/spin/SpinSource.h"
#include "include/spin/SpinState.h"

#include "include/kron/KronProd.h"
#include "include/misc/misc.h"

#include "include/quantum/HilbertSpaceOperator.h"
#include "include/quantum/LiouvilleSpaceOperator.h"
#include "include/quantum/MixedState.h"
#include "include/quantum/PureState.h"
#include "include/quantum/QuantumEvolution.h"
#include "include/quantum/QuantumEvolutionAlgorithm.h"
#include "include/quantum/QuantumOperator.h"
#include "include/quantum/QuantumState.h"

using namespace std;
using namespace arma;

#endif
