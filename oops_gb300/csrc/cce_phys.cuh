// cce_phys.cuh -- the cluster Hamiltonian of one NV-conditional branch, shared
// by the Hilbert-space (cce_dense.cu) and Liouville-space (cce_liouville.cu)
// coherence paths.
//
// H = sum_{i<j} S_i . J_ij . S_j            dipolar pairs  (misc.cpp:11-36)
//   + sum_i (-gamma_b B + D_i,e <S_e>) . S_i Zeeman + hyperfine mean field
//                                            (misc.cpp:38-57,
//                                             SpinInteraction.cpp:29-65)
// for k spin-1/2 bath nuclei, spin 0 the most significant bit of the basis
// index (KronProd order).  Units: rad/s; coordinates in Angstrom.
#pragma once

#include "oops_cce.h"
#include "oops_common.cuh"

namespace {

constexpr double PI_D = 3.14159265358979323846;
constexpr double HBAR = 1.054571800e-34;
constexpr double MU0 = 1.2566370614e-06;
constexpr int MAX_K = 6;

struct PhysParams {
    double B[3];
    double center[3];
    double gc, gb;
    double sv[2][3];
};

// dipolar tensor (row-major 3x3), misc.cpp:11-36
__device__ void dipole_tensor(const double *c1, const double *c2, double g1, double g2,
                              double out[9])
{
    double r[3] = {c1[0] - c2[0], c1[1] - c2[1], c1[2] - c2[2]};
    double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (d <= 1e-10) {
        for (int q = 0; q < 9; ++q) out[q] = 0.0;
        return;
    }
    double n[3] = {r[0] / d, r[1] / d, r[2] / d};
    double d0 = d * 1e-10;
    double pre = HBAR * MU0 / (4.0 * PI_D) * (g1 * g2) / (d0 * d0 * d0);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            out[3 * a + b] = pre * ((a == b ? 1.0 : 0.0) - 3.0 * n[a] * n[b]);
}

// matrix element of S_a (spin-1/2) between basis bits r (row) and c (col)
__device__ inline zd s_elem(int a, int r, int c)
{
    if (a == 2) return zmake(r == c ? (r == 0 ? 0.5 : -0.5) : 0.0, 0.0);
    if (r == c) return zmake(0, 0);
    if (a == 0) return zmake(0.5, 0.0);
    return zmake(0.0, r == 0 ? -0.5 : 0.5);  // S_y: (0,1) = -i/2, (1,0) = +i/2
}

// Coupling coefficients of cluster idx[0..K-1] in branch br, computed by the
// first K*K threads of the block: J[(i*K+j)*9 + 3a+b] for pairs i<j and
// h[3i+a] for single spins.  The caller synchronises before reading them.
template <int K>
__device__ void cluster_couplings(const double *__restrict__ coords, const unsigned *idx,
                                  const PhysParams &pp, int br, double *J, double *h)
{
    if (threadIdx.x < K * K) {
        int i = threadIdx.x / K, j = threadIdx.x % K;
        if (i < j) {
            double t9[9];
            dipole_tensor(coords + 3 * idx[i], coords + 3 * idx[j], pp.gb, pp.gb, t9);
            for (int q = 0; q < 9; ++q) J[(i * K + j) * 9 + q] = t9[q];
        }
    }
    if (threadIdx.x < K) {
        int i = threadIdx.x;
        double t9[9];
        dipole_tensor(coords + 3 * idx[i], pp.center, pp.gb, pp.gc, t9);
        for (int a = 0; a < 3; ++a) {
            double f = t9[a] * pp.sv[br][0] + t9[3 + a] * pp.sv[br][1] + t9[6 + a] * pp.sv[br][2];
            h[3 * i + a] = -pp.gb * pp.B[a] + f;
        }
    }
}

// Nonzero components of S_a (spin-1/2) between basis bits r (row) and c:
// r == c: S_z = +-1/2; r != c: S_x = 1/2 and S_y = -i/2 (r = 0) or +i/2.
// Each factor is real or imaginary with magnitude 1/2, so a product of two is
// +-1/4 or +-i/4 and every term of H costs one FP64 FMA (no complex
// products of constants, no FP64 compares).
struct SpinFactors {
    int n;       // 1 or 2 nonzero components
    int a[2];    // component index (0 x, 1 y, 2 z)
    int im[2];   // 1: the factor is imaginary
    int neg[2];  // 1: the factor is negative
};

__device__ __forceinline__ SpinFactors spin_factors(int r, int c)
{
    SpinFactors f;
    if (r == c) {
        f.n = 1;
        f.a[0] = 2; f.im[0] = 0; f.neg[0] = r;          // S_z: +1/2 (r = 0), -1/2
        f.a[1] = 0; f.im[1] = 0; f.neg[1] = 0;
    } else {
        f.n = 2;
        f.a[0] = 0; f.im[0] = 0; f.neg[0] = 0;          // S_x: 1/2
        f.a[1] = 1; f.im[1] = 1; f.neg[1] = r == 0;     // S_y: -i/2 (r = 0), +i/2
    }
    return f;
}

// H[r][c] from the couplings (zero unless r and c differ in at most two spins)
template <int K>
__device__ zd hamiltonian_elem(int r, int c, const double *J, const double *h)
{
    const int diff = r ^ c;
    double re = 0.0, im = 0.0;
    if (__popc(diff) > 2) return zmake(0.0, 0.0);
    for (int i = 0; i < K; ++i) {
        const int bi = K - 1 - i;
        const SpinFactors fi = spin_factors((r >> bi) & 1, (c >> bi) & 1);
        if ((diff & ~(1 << bi)) == 0) {  // single-spin terms, the other spins equal
            for (int u = 0; u < fi.n; ++u) {
                const double v = fi.neg[u] ? -0.5 : 0.5;
                if (fi.im[u]) im = fma(v, h[3 * i + fi.a[u]], im);
                else re = fma(v, h[3 * i + fi.a[u]], re);
            }
        }
        for (int j = i + 1; j < K; ++j) {
            const int bj = K - 1 - j;
            if ((diff & ~((1 << bi) | (1 << bj))) != 0) continue;
            const SpinFactors fj = spin_factors((r >> bj) & 1, (c >> bj) & 1);
            const double *Jij = J + (i * K + j) * 9;
            for (int u = 0; u < fi.n; ++u)
                for (int v = 0; v < fj.n; ++v) {
                    // (+-1/2 [i]) (+-1/2 [i]) = +-1/4, +-i/4, or -+1/4 for i*i
                    const int both = fi.im[u] & fj.im[v];
                    const int neg = fi.neg[u] ^ fj.neg[v] ^ both;
                    const double w = neg ? -0.25 : 0.25;
                    const double jab = Jij[3 * fi.a[u] + fj.a[v]];
                    if (fi.im[u] ^ fj.im[v]) im = fma(w, jab, im);
                    else re = fma(w, jab, re);
                }
        }
    }
    return zmake(re, im);
}

inline PhysParams phys_params(const oops_cce_params *p)
{
    PhysParams pp;
    for (int a = 0; a < 3; ++a) {
        pp.B[a] = p->B[a];
        pp.center[a] = p->center[a];
        pp.sv[0][a] = p->sv0[a];
        pp.sv[1][a] = p->sv1[a];
    }
    pp.gc = p->gamma_center;
    pp.gb = p->gamma_bath;
    return pp;
}

}  // namespace
