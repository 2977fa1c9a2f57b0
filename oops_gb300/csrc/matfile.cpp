// matfile.cpp -- the CCE result file, without MATLAB's libraries.
//
// The reference stores its results only when built against MATLAB's external
// interface (CCE::export_mat_file, src/source/app/cce.cpp:191-234: matOpen /
// mxCreateDoubleMatrix / matPutVariableAsGlobal), so a build without MATLAB
// loses them.  This writer produces the same variables as a Level 5 MAT-file
// (the published MAT-file format: a 128-byte header, then one miMATRIX data
// element per variable holding array flags, dimensions, name and the real
// part as miDOUBLE, each sub-element padded to 8 bytes), readable by MATLAB,
// Octave and scipy.io.loadmat:
//   CCE<i>, CCE<i>_tilder   nTime x nClst(i)   raw and reduced cluster curves
//   final_result_each_order nTime x max_order
//   final_result            nTime x max_order
//   time_list               nTime x 1
// every one flagged global, as matPutVariableAsGlobal does.  Host code only,
// little- or big-endian (the header's endian indicator records which).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "oops_cce.h"
#include "oops_expv.h"

int oops_set_status(int code, const char *msg);

namespace {

enum : uint32_t { miINT8 = 1, miINT32 = 5, miUINT32 = 6, miDOUBLE = 9, miMATRIX = 14 };
constexpr uint32_t mxDOUBLE_CLASS = 6;
constexpr uint32_t FLAG_GLOBAL = 0x04;

struct Buf {
    std::vector<unsigned char> b;
    void raw(const void *p, size_t n)
    {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        b.insert(b.end(), c, c + n);
    }
    void u32(uint32_t v) { raw(&v, 4); }
    void pad8()
    {
        while (b.size() % 8) b.push_back(0);
    }
    // one data element: tag (type, byte count) then the data, padded to 8
    void element(uint32_t type, const void *p, size_t n)
    {
        u32(type);
        u32((uint32_t)n);
        raw(p, n);
        pad8();
    }
};

bool put_matrix(FILE *f, const std::string &name, size_t rows, size_t cols, const double *data)
{
    if (rows > 0x7fffffffu || cols > 0x7fffffffu || rows * cols > ((size_t)1 << 28)) return false;
    Buf body;
    const uint32_t flags[2] = {(FLAG_GLOBAL << 8) | mxDOUBLE_CLASS, 0};
    body.element(miUINT32, flags, sizeof flags);
    const int32_t dims[2] = {(int32_t)rows, (int32_t)cols};
    body.element(miINT32, dims, sizeof dims);
    body.element(miINT8, name.data(), name.size());
    const size_t n = rows * cols;
    body.u32(miDOUBLE);
    body.u32((uint32_t)(n * sizeof(double)));
    Buf head;
    head.u32(miMATRIX);
    head.u32((uint32_t)(body.b.size() + n * sizeof(double)));  // n * 8: no padding needed
    if (std::fwrite(head.b.data(), 1, head.b.size(), f) != head.b.size()) return false;
    if (std::fwrite(body.b.data(), 1, body.b.size(), f) != body.b.size()) return false;
    return !n || std::fwrite(data, sizeof(double), n, f) == n;
}

}  // namespace

extern "C" int oops_cce_export_mat(const char *path, int max_order, size_t nT, const size_t *counts,
                                   const double *const *cluster_L, const double *const *cluster_til,
                                   const double *final_each, const double *final_cum,
                                   const double *time_list)
{
    if (!path || max_order < 1 || nT < 1 || !counts || !final_each || !final_cum || !time_list)
        return oops_set_status(OOPS_ERR_ARG, "oops_cce_export_mat: bad arguments");
    for (int o = 0; o < max_order; ++o)
        if (counts[o] && ((cluster_L && !cluster_L[o]) || (cluster_til && !cluster_til[o])))
            return oops_set_status(OOPS_ERR_ARG, "oops_cce_export_mat: missing cluster curves");
    FILE *f = std::fopen(path, "wb");
    if (!f) return oops_set_status(OOPS_ERR_ARG, "oops_cce_export_mat: cannot open the file");
    // header: 116 bytes of text, 8 bytes of subsystem offset, version, endian indicator
    char text[116];
    std::memset(text, ' ', sizeof text);
    const char *desc = "MATLAB 5.0 MAT-file, written by liboops_gb300 (ensemble CCE results)";
    std::memcpy(text, desc, std::strlen(desc));
    Buf h;
    h.raw(text, sizeof text);
    const unsigned char zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    h.raw(zero8, 8);
    const uint16_t version = 0x0100, endian = ('M' << 8) | 'I';
    h.raw(&version, 2);
    h.raw(&endian, 2);
    bool ok = std::fwrite(h.b.data(), 1, h.b.size(), f) == h.b.size();
    for (int o = 0; o < max_order && ok; ++o) {
        const std::string label = "CCE" + std::to_string(o);
        static const double none = 0.0;
        if (cluster_L) ok = put_matrix(f, label, nT, counts[o], counts[o] ? cluster_L[o] : &none);
        if (ok && cluster_til)
            ok = put_matrix(f, label + "_tilder", nT, counts[o], counts[o] ? cluster_til[o] : &none);
    }
    ok = ok && put_matrix(f, "final_result_each_order", nT, (size_t)max_order, final_each);
    ok = ok && put_matrix(f, "final_result", nT, (size_t)max_order, final_cum);
    ok = ok && put_matrix(f, "time_list", nT, 1, time_list);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? OOPS_OK : oops_set_status(OOPS_ERR_ARG, "oops_cce_export_mat: write failed or matrix too large");
}
