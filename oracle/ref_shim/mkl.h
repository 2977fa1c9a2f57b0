/*
 * mkl.h -- minimal stand-in for the three MKL CBLAS routines that the
 * reference's src/expv/source/hamvec_func3.cpp names (cblas_zcopy and
 * cblas_zaxpy on its live path, cblas_zgemm in a dead variant), so that file
 * can be compiled from its own source as a test pin.  TEST INFRASTRUCTURE
 * ONLY: used by oracle/build_ref.sh, never by the product.
 */
#ifndef OOPS_REF_SHIM_MKL_H
#define OOPS_REF_SHIM_MKL_H
#include <complex>
#include <cstddef>

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

static inline void cblas_zcopy(long long n, const void *x, long long incx,
                               void *y, long long incy)
{
    const std::complex<double> *a = (const std::complex<double> *)x;
    std::complex<double> *b = (std::complex<double> *)y;
    for (long long i = 0; i < n; ++i) b[i * incy] = a[i * incx];
}

static inline void cblas_zaxpy(long long n, const void *alpha, const void *x,
                               long long incx, void *y, long long incy)
{
    const std::complex<double> al = *(const std::complex<double> *)alpha;
    const std::complex<double> *a = (const std::complex<double> *)x;
    std::complex<double> *b = (std::complex<double> *)y;
    for (long long i = 0; i < n; ++i) b[i * incy] += al * a[i * incx];
}

/* column-major, only the (NoTrans, Trans) form the dead variant names */
static inline void cblas_zgemm(int layout, int ta, int tb, long long m,
                               long long n, long long k, const void *alpha,
                               const void *A, long long lda, const void *B,
                               long long ldb, const void *beta, void *C,
                               long long ldc)
{
    const std::complex<double> al = *(const std::complex<double> *)alpha;
    const std::complex<double> be = *(const std::complex<double> *)beta;
    const std::complex<double> *a = (const std::complex<double> *)A;
    const std::complex<double> *b = (const std::complex<double> *)B;
    std::complex<double> *c = (std::complex<double> *)C;
    for (long long j = 0; j < n; ++j)
        for (long long i = 0; i < m; ++i) {
            std::complex<double> s = 0;
            for (long long l = 0; l < k; ++l) {
                std::complex<double> av = ta == CblasNoTrans ? a[i + l * lda] : a[l + i * lda];
                std::complex<double> bv = tb == CblasNoTrans ? b[l + j * ldb] : b[j + l * ldb];
                s += av * bv;
            }
            c[i + j * ldc] = al * s + be * c[i + j * ldc];
        }
    (void)layout;
}
#endif
