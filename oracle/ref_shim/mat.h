// TEST INFRASTRUCTURE ONLY.  Stand-in for MATLAB's mat.h, which the
// reference's include/oops.h and include/quantum/QuantumOperator.h include
// when HAS_MATLAB is defined.  Without HAS_MATLAB (every pin but
// ref_export_pin) it is empty and the reference's export code is compiled
// out.  With HAS_MATLAB it records the calls the reference's
// CCE::export_mat_file makes (cce.cpp:191-234): matOpen names a file, and
// every matPutVariableAsGlobal appends one record to it -- the name's length
// (uint32) and bytes, the rows and columns (uint64), a complex flag (uint32)
// and the real (then imaginary) parts, column-major float64 -- so a test can
// read back exactly which variables, shapes and values the reference wrote.
#pragma once

#ifdef HAS_MATLAB
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

struct MATFile {
    std::FILE *f;
};
enum mxComplexity { mxREAL = 0, mxCOMPLEX = 1 };
struct mxArray {
    size_t m, n;
    double *pr, *pi;
};

inline mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c)
{
    mxArray *a = new mxArray{m, n, nullptr, nullptr};
    a->pr = static_cast<double *>(std::calloc(m * n ? m * n : 1, sizeof(double)));
    if (c == mxCOMPLEX) a->pi = static_cast<double *>(std::calloc(m * n ? m * n : 1, sizeof(double)));
    return a;
}
inline double *mxGetPr(const mxArray *a) { return a->pr; }
inline double *mxGetPi(const mxArray *a) { return a->pi; }
inline void mxDestroyArray(mxArray *a)
{
    std::free(a->pr);
    std::free(a->pi);
    delete a;
}
inline MATFile *matOpen(const char *path, const char *)
{
    std::FILE *f = std::fopen(path, "wb");
    if (!f) {
        std::perror(path);
        std::abort();
    }
    return new MATFile{f};
}
inline int matPutVariableAsGlobal(MATFile *mf, const char *name, const mxArray *a)
{
    const uint32_t len = (uint32_t)std::strlen(name), cplx = a->pi ? 1u : 0u;
    const uint64_t dims[2] = {a->m, a->n};
    std::fwrite(&len, sizeof len, 1, mf->f);
    std::fwrite(name, 1, len, mf->f);
    std::fwrite(dims, sizeof dims[0], 2, mf->f);
    std::fwrite(&cplx, sizeof cplx, 1, mf->f);
    std::fwrite(a->pr, sizeof(double), a->m * a->n, mf->f);
    if (a->pi) std::fwrite(a->pi, sizeof(double), a->m * a->n, mf->f);
    return 0;
}
inline int matClose(MATFile *mf)
{
    std::fclose(mf->f);
    delete mf;
    return 0;
}
#endif
