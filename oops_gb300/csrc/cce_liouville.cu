// cce_liouville.cu -- Liouville-space cluster coherence with bath dephasing and
// bath polarisation: EnsembleCCE::cluster_evolution as the reference runs it
// by default (src/source/app/ensemble_cce.cpp:33-113; the EnsNVeBath and
// EnsNVLattice applications default to a 1e4 Hz dephasing rate along (1,1,1),
// src/application/EnsNVeBath.cpp:133-135).
//
// Per cluster of k spin-1/2 nuclei (D = 2^k, N = D^2 = 4^k, k <= 6), with rho
// vectorised column-major (entry r + D c):
//   L_A rho = rho H_0 - H_1 rho + i g sum_s (sigma_s rho sigma_s - rho)
//   L_B rho = rho H_1 - H_0 rho + (the same dephasing term)
// (create_spin_liouvillian = SHARP(H_0) - FLAT(H_1), ensemble_cce.cpp:86-92;
// SingleSpinDephasing = i (sigma^T (x) sigma - 1) per spin,
// SpinInteractionComponent.cpp:285-304, g = 2 pi rate, sigma = n.sigma);
// segments j = 0..n alternate A, B (riffle, misc.h:25-40) over the CPMG
// interval fractions 1/(2n), 1/n, ..., 1/n, 1/(2n) of t (Pulse_Interval,
// misc.cpp:59-84); rho0 = I/D + sum_s p.S_s (SpinPolarization and
// cSpinState::make, SpinState.cpp:9-60); and
//   L(t_i) = Re < D rho0, E_n^i ... E_1^i E_0^i rho0 >,  E_j = exp(-i L_j s_j dt)
// (PiecewiseFullMatrixVectorEvolution, QuantumEvolutionAlgorithm.cpp:60-83;
// calc_observables, ensemble_cce.cpp:104-113).
//
// The reference advances each segment's power E_j^i by one N x N product per
// time step, nT (n+1) products of N^3 per cluster.  Here:
//   * one exponential per cluster, G_A = exp(-i L_A tau) at the shortest
//     interval tau = dt / (2n) (the 1/n segments use G^2): the Taylor polynomial of
//     degree 19, evaluated by Paterson-Stockmeyer (X^2, X^3, X^4, then four
//     Horner steps in X^4: 7 products) after the argument has been scaled by
//     2^-s to 1-norm <= 1 (truncation error < 1e-18), then squared s times
//     (scaling and squaring, Moler & Van Loan).  Branch B needs no
//     exponential of its own: with J rho = rho^+, J L_A J = L_B (the
//     Hamiltonian part changes sign under J and swaps H_0, H_1; the dephasing
//     part commutes with J), so G_B rho = (G_A rho^+)^+, i.e.
//     G_B[r + D c, r1 + D c1] = conj(G_A[c + D r, c1 + D r1]), and the same
//     for every power: branch B's matrices are a permuted conjugate copy;
//   * the first and the last segment become vector recurrences: u_i =
//     G_A u_{i-1} from rho0, and y_i = G_last^H y_{i-1} from D rho0 (the
//     observable is an inner product, so the last factor moves to the left
//     as its adjoint);
//   * the n - 1 middle segments (CPMG n >= 2) apply G^{2i} to column i of the
//     state block through the binary digits of i: the squarings G^{2^(b+1)}
//     multiply the columns whose bit b is set, ceil(log2 nT) batched GEMM
//     passes per segment instead of nT products of N^3;
//   * L_i = Re y_i^H (middle) u_i.
// A Hahn echo (n = 1) needs no matrix power beyond G.  Everything is FP64: the
// recurrences raise G to powers up to nT, which multiplies G's relative error
// by up to nT, so FP32 products would cost ~1e-5 in L.  FP64 GEMM is the
// bound (GB300 issues FP64 at 1/64 of the FP32 rate); the tiles are sized so
// that shared-memory traffic stays far below the FP64 pipe's rate.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "cce_phys.cuh"
#include "oops_cce.h"
#include "oops_common.cuh"
#include "oops_internal.h"

namespace {

constexpr int LV_MAX_K = 6;
constexpr int NTHR = 256;

// slots of the per-item (cluster, branch) matrix slab; after the exponential,
// slot b holds G^{2^b}
enum { SX = 0, SX2 = 1, SX3 = 2, SX4 = 3, SP = 4, SQ = 5, NSCRATCH = 6 };

struct LvParams {
    PhysParams pp;
    double gamma;  // 2 pi * dephasing rate (rad/s)
    zd sg[4];      // sigma_n, column-major 2 x 2
    double pol[3];
    double tau;    // shortest interval dt / (2n)
};

// epilogue of a product: + c0 I + c1 M[e0] + c2 M[e1] + c3 M[e2] (slots, -1 = none)
struct LinComb {
    int e[3];
    double c[4];
};

// element (out, in) of the Liouvillian L (not yet multiplied by -i tau)
template <int K>
__device__ zd lv_elem(int out, int in, const zd *Hs, const zd *Hf, const LvParams &lp)
{
    constexpr int D = 1 << K;
    const int r = out % D, c = out / D, r1 = in % D, c1 = in / D;
    zd v = zmake(0, 0);
    if (r == r1) v = Hs[c1 + D * c];             // (rho H_s)_{r c}
    if (c == c1) v = zsub(v, Hf[r + D * r1]);    // -(H_f rho)_{r c}
    if (lp.gamma != 0.0) {
        const int dr = r ^ r1, dc = c ^ c1;
        for (int s = 0; s < K; ++s) {
            const int bit = 1 << (K - 1 - s);
            if ((dr & ~bit) != 0 || (dc & ~bit) != 0) continue;
            // (sigma rho sigma)_{r c} = sigma_{r r1} rho_{r1 c1} sigma_{c1 c}
            const int ar = (r & bit) != 0, br = (r1 & bit) != 0;
            const int bc = (c1 & bit) != 0, ac = (c & bit) != 0;
            const zd val = zmul(lp.sg[ar + 2 * br], lp.sg[bc + 2 * ac]);
            v = zadd(v, zmake(-lp.gamma * val.y, lp.gamma * val.x));  // + i g val
        }
        if (out == in) v = zadd(v, zmake(0.0, -lp.gamma * K));       // - i g k
    }
    return v;
}

// ---------------------------------------------------------------------------
// Kernel 1: X = -i tau L_A 2^-s for cluster blockIdx.x (item 2 cl of the
// slab; item 2 cl + 1, branch B, is mirrored from it later); s = the smallest
// power with ||X||_1 <= 1.  One CTA per cluster.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(NTHR)
k_lv_generator(const double *__restrict__ coords, const unsigned *__restrict__ clusters,
               LvParams lp, zd *__restrict__ slab, size_t slab_elems, int *__restrict__ sexp)
{
    constexpr int D = 1 << K, N = D * D;
    extern __shared__ zd lv_dyn[];  // the two conditional Hamiltonians, D x D each
    zd *H[2] = {lv_dyn, lv_dyn + D * D};
    __shared__ double J[MAX_K * MAX_K * 9];
    __shared__ double h[MAX_K * 3];
    __shared__ double red[NTHR / 32];
    __shared__ int s_s;
    const int cl = blockIdx.x, item = 2 * cl, which = 0;
    const unsigned *idx = clusters + (size_t)cl * K;
    for (int br = 0; br < 2; ++br) {
        cluster_couplings<K>(coords, idx, lp.pp, br, J, h);
        __syncthreads();
        for (int e = threadIdx.x; e < D * D; e += NTHR) H[br][e] = hamiltonian_elem<K>(e % D, e / D, J, h);
        __syncthreads();
    }
    // branch A (which = 0): rho H_0 - H_1 rho; branch B: rho H_1 - H_0 rho
    const zd *Hs = H[which], *Hf = H[which ^ 1];
    double mx = 0.0;
    for (int in = threadIdx.x; in < N; in += NTHR) {
        double cs = 0.0;
        for (int out = 0; out < N; ++out) cs += zabs(lv_elem<K>(out, in, Hs, Hf, lp));
        mx = fmax(mx, cs);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double nrm = 0.0;
        for (int w = 0; w < NTHR / 32; ++w) nrm = fmax(nrm, red[w]);
        nrm *= lp.tau;
        int s = 0;
        if (!(nrm <= 1e300)) s = -1;         // NaN or overflow: reported by the host
        else if (nrm > 1.0) frexp(nrm, &s);  // nrm < 2^s
        s_s = s;
        sexp[item] = s;
    }
    __syncthreads();
    const double sc = ldexp(lp.tau, -max(s_s, 0));
    zd *X = slab + (size_t)item * slab_elems + (size_t)SX * N * N;
    for (int e = threadIdx.x; e < N * N; e += NTHR) {
        const zd l = lv_elem<K>(e % N, e / N, Hs, Hf, lp);
        X[e] = zmake(l.y * sc, -l.x * sc);  // -i tau 2^-s l
    }
}

__device__ __forceinline__ zd lincomb_at(const zd *base, size_t NN, size_t e, bool diag,
                                         const LinComb &lc)
{
    zd v = zmake(diag ? lc.c[0] : 0.0, 0.0);
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if (lc.e[q] >= 0) {
            const zd m = base[(size_t)lc.e[q] * NN + e];
            v.x = fma(lc.c[q + 1], m.x, v.x);
            v.y = fma(lc.c[q + 1], m.y, v.y);
        }
    return v;
}

// ---------------------------------------------------------------------------
// Kernel 2: batched C = A B (+ LinComb) on N x N slab slots, N >= 64.
// 64 x 64 output tile per CTA, 16-deep k chunks staged in shared memory; each
// thread owns a 4 x 4 complex tile (rows tx + 16 a, columns ty + 16 b, so the
// stores are coalesced down the columns).  sq_pass >= 0 restricts the
// product to the items that still square (sexp[item] > sq_pass).
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(NTHR)
k_lv_gemm(zd *__restrict__ slab, size_t slab_elems, int istride, int a, int b, int c, LinComb lc,
          const int *__restrict__ sexp, int sq_pass)
{
    constexpr int T = N / 64;
    constexpr size_t NN = (size_t)N * N;
    const int item = blockIdx.y * istride;
    if (sq_pass >= 0 && sexp[item] <= sq_pass) return;
    const int tr = blockIdx.x % T, tc = blockIdx.x / T;
    zd *base = slab + (size_t)item * slab_elems;
    const zd *A = base + (size_t)a * NN, *B = base + (size_t)b * NN;
    zd *C = base + (size_t)c * NN;
    __shared__ zd As[16][64], Bs[16][64];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    zd acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = zmake(0, 0);
    for (int k0 = 0; k0 < N; k0 += 16) {
        for (int q = threadIdx.x; q < 1024; q += NTHR) {
            const int row = q & 63, kk = q >> 6;
            As[kk][row] = A[(size_t)(tr * 64 + row) + (size_t)N * (k0 + kk)];
        }
        for (int q = threadIdx.x; q < 1024; q += NTHR) {
            const int kk = q & 15, col = q >> 4;
            Bs[kk][col] = B[(size_t)(k0 + kk) + (size_t)N * (tc * 64 + col)];
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; ++kk) {
            zd av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) zfma(acc[i][j], av[i], bv[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int row = tr * 64 + tx + 16 * i, col = tc * 64 + ty + 16 * j;
            const size_t e = (size_t)row + (size_t)N * col;
            const zd add = lincomb_at(base, NN, e, row == col, lc);
            C[e] = zadd(acc[i][j], add);
        }
}

// the same for N = 4, 16: one CTA per item, one thread per output element
template <int N>
__global__ void __launch_bounds__(NTHR)
k_lv_gemm_small(zd *__restrict__ slab, size_t slab_elems, int istride, int a, int b, int c, LinComb lc,
                const int *__restrict__ sexp, int sq_pass)
{
    constexpr size_t NN = (size_t)N * N;
    const int item = blockIdx.y * istride;
    if (sq_pass >= 0 && sexp[item] <= sq_pass) return;
    zd *base = slab + (size_t)item * slab_elems;
    const zd *A = base + (size_t)a * NN, *B = base + (size_t)b * NN;
    zd *C = base + (size_t)c * NN;
    __shared__ zd As[NN], Bs[NN];
    for (int e = threadIdx.x; e < (int)NN; e += NTHR) {
        As[e] = A[e];
        Bs[e] = B[e];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < (int)NN; e += NTHR) {
        const int row = e % N, col = e / N;
        zd acc = zmake(0, 0);
        for (int l = 0; l < N; ++l) zfma(acc, As[row + N * l], Bs[l + N * col]);
        C[e] = zadd(acc, lincomb_at(base, NN, e, row == col, lc));
    }
}

// C = LinComb only (the leading Horner coefficient)
template <int N>
__global__ void k_lv_lincomb(zd *__restrict__ slab, size_t slab_elems, int istride, int c, LinComb lc)
{
    constexpr size_t NN = (size_t)N * N;
    zd *base = slab + (size_t)blockIdx.y * istride * slab_elems;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < NN;
         e += (size_t)gridDim.x * blockDim.x)
        base[(size_t)c * NN + e] = lincomb_at(base, NN, e, (e % N) == (e / N), lc);
}

// slot 0 <- the squaring result (slot P after an even number of squarings,
// Q after an odd one)
template <int N>
__global__ void k_lv_finalize(zd *__restrict__ slab, size_t slab_elems, int istride,
                              const int *__restrict__ sexp)
{
    constexpr size_t NN = (size_t)N * N;
    const int item = blockIdx.y * istride;
    zd *base = slab + (size_t)item * slab_elems;
    const int src = (sexp[item] & 1) ? SQ : SP;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < NN;
         e += (size_t)gridDim.x * blockDim.x)
        base[e] = base[(size_t)src * NN + e];
}

// branch B's slots from branch A's: B[P o + N P i] = conj(A[o + N i]) with
// P(r + D c) = c + D r (the rho -> rho^+ symmetry); grid.y = cluster x slot
template <int K>
__global__ void k_lv_mirror(zd *__restrict__ slab, size_t slab_elems, int nused)
{
    constexpr int D = 1 << K, N = D * D;
    constexpr size_t NN = (size_t)N * N;
    const int cl = blockIdx.y / nused, slot = blockIdx.y % nused;
    const zd *A = slab + (size_t)(2 * cl) * slab_elems + (size_t)slot * NN;
    zd *B = slab + (size_t)(2 * cl + 1) * slab_elems + (size_t)slot * NN;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < NN;
         e += (size_t)gridDim.x * blockDim.x) {
        const int o = (int)(e % N), i = (int)(e / N);
        const int po = o / D + D * (o % D), pi = i / D + D * (i % D);
        const zd a = A[e];
        B[(size_t)po + (size_t)N * pi] = zmake(a.x, -a.y);
    }
}

// ---------------------------------------------------------------------------
// Kernel 3: the outer segments as vector recurrences, one CTA per (cluster,
// side): side 0 writes u_i = G_A^i rho0 to S, side 1 writes
// y_i = (G_last^H)^i D rho0 to Y (N x nT per cluster, column i = time i).
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(NTHR)
k_lv_recur(const zd *__restrict__ slab, size_t slab_elems, int last_branch, LvParams lp, int nT,
           zd *__restrict__ S, zd *__restrict__ Y)
{
    constexpr int D = 1 << K, N = D * D;
    extern __shared__ zd lv_dyn[];  // x and y, N each
    zd *x = lv_dyn, *y = lv_dyn + N;
    const int cl = blockIdx.x >> 1, side = blockIdx.x & 1;
    const zd *G = slab + (size_t)(2 * cl + (side ? last_branch : 0)) * slab_elems;  // slot 0
    zd *out = (side ? Y : S) + (size_t)cl * N * nT;
    for (int e = threadIdx.x; e < N; e += NTHR) {
        const int r = e % D, c = e / D;
        zd v = zmake(r == c ? 1.0 / D : 0.0, 0.0);
        for (int s = 0; s < K; ++s) {
            const int bit = 1 << (K - 1 - s);
            if (((r ^ c) & ~bit) != 0) continue;
            const int ar = (r & bit) != 0, ac = (c & bit) != 0;
            for (int a = 0; a < 3; ++a) v = zadd(v, zscale(s_elem(a, ar, ac), lp.pol[a]));
        }
        if (side) v = zscale(v, (double)D);
        x[e] = v;
        out[e] = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = 1; i < nT; ++i) {
        if (side == 0) {  // y = G x: thread per row, coalesced down G's columns
            for (int r = threadIdx.x; r < N; r += NTHR) {
                zd acc = zmake(0, 0);
#pragma unroll 4
                for (int l = 0; l < N; ++l) zfma(acc, G[r + (size_t)N * l], x[l]);
                y[r] = acc;
            }
        } else {  // y = G^H x: warp per row r, lanes down column r of G
            for (int r = warp; r < N; r += NTHR / 32) {
                zd acc = zmake(0, 0);
                for (int l = lane; l < N; l += 32) {
                    const zd g = G[l + (size_t)N * r];
                    const zd xv = x[l];
                    acc.x = fma(g.x, xv.x, acc.x);
                    acc.x = fma(g.y, xv.y, acc.x);
                    acc.y = fma(g.x, xv.y, acc.y);
                    acc.y = fma(-g.y, xv.x, acc.y);
                }
                for (int o = 16; o > 0; o >>= 1) {
                    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
                    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
                }
                if (lane == 0) y[r] = acc;
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < N; e += NTHR) {
            x[e] = y[e];
            out[e + (size_t)N * i] = y[e];
        }
        __syncthreads();
    }
}

// column index of the j-th time point whose bit b is set
__device__ __forceinline__ int set_bit_col(int j, int b)
{
    return ((j >> b) << (b + 1)) | (1 << b) | (j & ((1 << b) - 1));
}

// ---------------------------------------------------------------------------
// Kernel 4: one binary digit of one middle segment, N >= 64:
// Sout[:, i] = G^{2^(b+1)} Sin[:, i] for the columns i with bit b set
// (compressed to nact columns); k_lv_pass_copy copies the others.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(NTHR)
k_lv_pass(const zd *__restrict__ slab, size_t slab_elems, int branch, int gslot, int b, int nact,
          int nT, const zd *__restrict__ Sin, zd *__restrict__ Sout)
{
    constexpr int T = N / 64;
    const int ctiles = (nact + 63) / 64;
    const int cl = blockIdx.y;
    const int tr = blockIdx.x % T, tcol = blockIdx.x / T;
    if (tcol >= ctiles) return;
    const zd *A = slab + (size_t)(2 * cl + branch) * slab_elems + (size_t)gslot * N * N;
    const zd *Bm = Sin + (size_t)cl * N * nT;
    zd *Cm = Sout + (size_t)cl * N * nT;
    __shared__ zd As[16][64], Bs[16][64];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    zd acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = zmake(0, 0);
    for (int k0 = 0; k0 < N; k0 += 16) {
        for (int q = threadIdx.x; q < 1024; q += NTHR) {
            const int row = q & 63, kk = q >> 6;
            As[kk][row] = A[(size_t)(tr * 64 + row) + (size_t)N * (k0 + kk)];
        }
        for (int q = threadIdx.x; q < 1024; q += NTHR) {
            const int kk = q & 15, col = q >> 4;
            const int j = tcol * 64 + col;
            Bs[kk][col] = j < nact ? Bm[(size_t)(k0 + kk) + (size_t)N * set_bit_col(j, b)] : zmake(0, 0);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; ++kk) {
            zd av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) zfma(acc[i][j], av[i], bv[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int jj = tcol * 64 + ty + 16 * j;
        if (jj >= nact) continue;
        const size_t col = (size_t)set_bit_col(jj, b);
#pragma unroll
        for (int i = 0; i < 4; ++i) Cm[(size_t)(tr * 64 + tx + 16 * i) + (size_t)N * col] = acc[i][j];
    }
}

// N = 4, 16: thread per (row, active column)
template <int N>
__global__ void __launch_bounds__(NTHR)
k_lv_pass_small(const zd *__restrict__ slab, size_t slab_elems, int branch, int gslot, int b,
                int nact, int nT, const zd *__restrict__ Sin, zd *__restrict__ Sout)
{
    const int cl = blockIdx.y;
    const zd *A = slab + (size_t)(2 * cl + branch) * slab_elems + (size_t)gslot * N * N;
    const zd *Bm = Sin + (size_t)cl * N * nT;
    zd *Cm = Sout + (size_t)cl * N * nT;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)N * nact;
         e += (long)gridDim.x * blockDim.x) {
        const int row = (int)(e % N);
        const size_t col = (size_t)set_bit_col((int)(e / N), b);
        zd acc = zmake(0, 0);
        for (int l = 0; l < N; ++l) zfma(acc, A[row + N * l], Bm[l + N * col]);
        Cm[row + N * col] = acc;
    }
}

// columns i whose bit b is clear: copied unchanged
__global__ void k_lv_pass_copy(int N, int b, int nT, const zd *__restrict__ Sin, zd *__restrict__ Sout)
{
    const size_t per = (size_t)N * nT;
    const zd *src = Sin + (size_t)blockIdx.y * per;
    zd *dst = Sout + (size_t)blockIdx.y * per;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < per;
         e += (size_t)gridDim.x * blockDim.x)
        if (!(((e / N) >> b) & 1)) dst[e] = src[e];
}

// ---------------------------------------------------------------------------
// Kernel 5: L_i = Re y_i^H s_i, one warp per (cluster, time point)
// ---------------------------------------------------------------------------
__global__ void k_lv_dot(int N, int nT, int ncl, const zd *__restrict__ S, const zd *__restrict__ Y,
                         double *__restrict__ L)
{
    const int lane = threadIdx.x & 31;
    const long nw = (long)gridDim.x * (blockDim.x >> 5);
    for (long w = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < (long)ncl * nT; w += nw) {
        const zd *s = S + (size_t)w * N, *y = Y + (size_t)w * N;
        double acc = 0.0;
        for (int q = lane; q < N; q += 32) acc += y[q].x * s[q].x + y[q].y * s[q].y;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) L[w] = acc;
    }
}

// 1/j! for the Taylor coefficients
double inv_fact(int j)
{
    double f = 1.0;
    for (int q = 2; q <= j; ++q) f *= q;
    return 1.0 / f;
}

LinComb taylor_block(int j, bool with_identity)
{
    LinComb lc;
    lc.c[0] = with_identity ? inv_fact(4 * j) : 0.0;
    lc.e[0] = SX;
    lc.c[1] = inv_fact(4 * j + 1);
    lc.e[1] = SX2;
    lc.c[2] = inv_fact(4 * j + 2);
    lc.e[2] = SX3;
    lc.c[3] = inv_fact(4 * j + 3);
    return lc;
}

LinComb no_comb()
{
    LinComb lc;
    lc.e[0] = lc.e[1] = lc.e[2] = -1;
    lc.c[0] = lc.c[1] = lc.c[2] = lc.c[3] = 0.0;
    return lc;
}

// products on the branch-A items 0, 2, 4, ... of the slab (nc of them)
template <int N>
void launch_gemm(zd *slab, size_t slab_elems, int nc, int a, int b, int c, const LinComb &lc,
                 const int *sexp, int sq_pass, cudaStream_t st)
{
    if constexpr (N >= 64) {
        dim3 grid((N / 64) * (N / 64), nc);
        k_lv_gemm<N><<<grid, NTHR, 0, st>>>(slab, slab_elems, 2, a, b, c, lc, sexp, sq_pass);
    } else {
        dim3 grid(1, nc);
        k_lv_gemm_small<N><<<grid, NTHR, 0, st>>>(slab, slab_elems, 2, a, b, c, lc, sexp, sq_pass);
    }
}

int bit_length(int v)
{
    int b = 0;
    while (v > 0) {
        ++b;
        v >>= 1;
    }
    return b;
}

// count of i in [0, nT) with bit b set
int count_bit(int nT, int b)
{
    const long period = 2L << b, full = nT / period, rem = nT % period;
    return (int)(full * (period / 2) + std::max(0L, rem - (period / 2)));
}

// Per-cluster device memory of one chunk: the two items' slabs, S (two
// buffers for the middle passes) and Y.
size_t chunk_bytes(int N, int nslots, int nT, bool middle)
{
    return (2 * (size_t)nslots * N * N + (size_t)(middle ? 3 : 2) * N * nT) * sizeof(zd);
}

// Phase timers (profiling on): per cluster size k and phase -- 0 the
// exponentials (Taylor products, squarings, binary powers), 1 the outer
// recurrences, 2 the middle-segment passes -- accumulated time, kernel
// launches and FP64 flop; g_lv_launches counts every kernel this path
// launches, profiling or not.
std::mutex g_lv_mu;
double g_lv_ms[LV_MAX_K + 1][3], g_lv_flop[LV_MAX_K + 1][3];
long g_lv_n[LV_MAX_K + 1][3], g_lv_launches = 0;

void lv_account(int k, const long *n, const double *flop, const float *ms, long launches)
{
    std::lock_guard<std::mutex> lk(g_lv_mu);
    for (int q = 0; q < 3; ++q) {
        g_lv_n[k][q] += n[q];
        g_lv_flop[k][q] += flop[q];
        if (ms) g_lv_ms[k][q] += ms[q];
    }
    g_lv_launches += launches;
}

template <int K>
int run_liouville(const double *coords, const unsigned *clusters, int ncl, const LvParams &lp,
                  int pulse_num, int nT, double *L, cudaStream_t st)
{
    constexpr int D = 1 << K, N = D * D;
    const bool middle = pulse_num >= 2;
    const int nbits = bit_length(nT - 1);
    const int nslots = std::max<int>(NSCRATCH, middle ? nbits + 1 : 1);
    const size_t slab_elems = (size_t)nslots * N * N;
    const int last_branch = pulse_num & 1;  // segment n: A for even n, B for odd n
    // chunk: at most ~6 GiB of scratch at a time (a CCE-4 four-spin class,
    // ~150 clusters of ~16 MB, runs as one chunk)
    const size_t per = chunk_bytes(N, nslots, nT, middle);
    // and grid.y (clusters x mirrored slots) within the 65535 launch limit
    const int chunk = (int)std::max<size_t>(
        1, std::min<size_t>({(size_t)ncl, ((size_t)6 << 30) / per, (size_t)(65535 / nslots)}));
    zd *slab = nullptr, *S = nullptr, *S2 = nullptr, *Y = nullptr;
    int *sexp = nullptr;
    auto cleanup = [&]() {
        if (slab) cudaFreeAsync(slab, st);
        if (S) cudaFreeAsync(S, st);
        if (S2) cudaFreeAsync(S2, st);
        if (Y) cudaFreeAsync(Y, st);
        if (sexp) cudaFreeAsync(sexp, st);
    };
    if (cudaMallocAsync((void **)&slab, (size_t)2 * chunk * slab_elems * sizeof(zd), st) != cudaSuccess ||
        cudaMallocAsync((void **)&S, (size_t)chunk * N * nT * sizeof(zd), st) != cudaSuccess ||
        cudaMallocAsync((void **)&Y, (size_t)chunk * N * nT * sizeof(zd), st) != cudaSuccess ||
        (middle && cudaMallocAsync((void **)&S2, (size_t)chunk * N * nT * sizeof(zd), st) != cudaSuccess) ||
        cudaMallocAsync((void **)&sexp, (size_t)2 * chunk * sizeof(int), st) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return oops_set_status(OOPS_ERR_NOMEM, "device allocation failed (Liouville path)");
    }
    std::vector<int> hs((size_t)2 * chunk);
    int rc = OOPS_OK;
    // dynamic shared memory: the generator's two Hamiltonians (128 KB at
    // k = 6), the recurrence's two vectors (128 KB at k = 6)
    const size_t gen_smem = (size_t)2 * D * D * sizeof(zd), rec_smem = (size_t)2 * N * sizeof(zd);
    cudaFuncSetAttribute(k_lv_generator<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gen_smem);
    cudaFuncSetAttribute(k_lv_recur<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rec_smem);
    const bool prof = oops_prof_enabled();
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    if (prof)
        for (auto &e : ev) cudaEventCreate(&e);
    const double f3 = 8.0 * N * N * N, f2 = 8.0 * N * N;  // FP64 flop of one product, one matvec
    for (int c0 = 0; c0 < ncl && rc == OOPS_OK; c0 += chunk) {
        const int nc = std::min(chunk, ncl - c0), items = 2 * nc;
        long nl[3] = {0, 0, 0}, launches = 2;  // generator and dot
        double fl[3] = {0, 0, 0};
        k_lv_generator<K><<<nc, NTHR, gen_smem, st>>>(coords, clusters + (size_t)c0 * K, lp, slab,
                                                      slab_elems, sexp);
        if (cudaMemcpyAsync(hs.data(), sexp, (size_t)items * sizeof(int), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        int smax = 0;
        for (int q = 0; q < items; q += 2) {
            if (hs[q] < 0) rc = oops_set_status(OOPS_ERR_NUMERIC, "non-finite Liouvillian norm");
            smax = std::max(smax, hs[q]);
        }
        if (rc != OOPS_OK) break;
        if (prof) cudaEventRecord(ev[0], st);
        // exp(X) by the degree-19 Taylor polynomial (Paterson-Stockmeyer)
        const LinComb none = no_comb();
        const int nused = middle ? nbits + 1 : 1;  // slots branch B needs
        nl[0] += 10 + smax + (middle ? nbits : 0);
        fl[0] += f3 * nc * (7 + (middle ? nbits : 0));
        for (int q = 0; q < items; q += 2) fl[0] += f3 * hs[q];
        launch_gemm<N>(slab, slab_elems, nc, SX, SX, SX2, none, sexp, -1, st);
        launch_gemm<N>(slab, slab_elems, nc, SX2, SX, SX3, none, sexp, -1, st);
        launch_gemm<N>(slab, slab_elems, nc, SX2, SX2, SX4, none, sexp, -1, st);
        const unsigned eblocks = (unsigned)std::max<size_t>(1, std::min<size_t>(64, ((size_t)N * N + NTHR - 1) / NTHR));
        k_lv_lincomb<N><<<dim3(eblocks, nc), NTHR, 0, st>>>(slab, slab_elems, 2, SP, taylor_block(4, true));
        int cur = SP;
        for (int j = 3; j >= 0; --j) {
            const int nxt = cur == SP ? SQ : SP;
            launch_gemm<N>(slab, slab_elems, nc, cur, SX4, nxt, taylor_block(j, true), sexp, -1, st);
            cur = nxt;
        }
        // cur == SP after four steps; square back: pass p maps P->Q (even p), Q->P (odd p)
        for (int p = 0; p < smax; ++p) {
            const int src = (p & 1) ? SQ : SP, dst = (p & 1) ? SP : SQ;
            launch_gemm<N>(slab, slab_elems, nc, src, src, dst, none, sexp, p, st);
        }
        k_lv_finalize<N><<<dim3(eblocks, nc), NTHR, 0, st>>>(slab, slab_elems, 2, sexp);
        if (middle)
            for (int b = 1; b <= nbits; ++b)
                launch_gemm<N>(slab, slab_elems, nc, b - 1, b - 1, b, none, sexp, -1, st);
        k_lv_mirror<K><<<dim3(eblocks, nc * nused), NTHR, 0, st>>>(slab, slab_elems, nused);
        if (prof) cudaEventRecord(ev[1], st);
        k_lv_recur<K><<<2 * nc, NTHR, rec_smem, st>>>(slab, slab_elems, last_branch, lp, nT, S, Y);
        nl[1] += 1;
        fl[1] += f2 * 2.0 * nc * (nT - 1);
        if (prof) cudaEventRecord(ev[2], st);
        zd *cur_s = S, *oth_s = S2;
        if (middle) {
            for (int j = 1; j < pulse_num; ++j) {
                const int branch = j & 1;  // odd segments: B
                for (int b = 0; b < nbits; ++b) {
                    const int nact = count_bit(nT, b);
                    nl[2] += 1 + (nact > 0);
                    fl[2] += f2 * (double)nc * nact;
                    if (nact > 0) {
                        if constexpr (N >= 64) {
                            dim3 grid((N / 64) * ((nact + 63) / 64), nc);
                            k_lv_pass<N><<<grid, NTHR, 0, st>>>(slab, slab_elems, branch, b + 1, b, nact, nT,
                                                                cur_s, oth_s);
                        } else {
                            dim3 grid((unsigned)std::min<long>(1024, ((long)N * nact + NTHR - 1) / NTHR), nc);
                            k_lv_pass_small<N><<<grid, NTHR, 0, st>>>(slab, slab_elems, branch, b + 1, b, nact,
                                                                      nT, cur_s, oth_s);
                        }
                    }
                    {
                        dim3 grid((unsigned)std::min<long>(1024, ((long)N * nT + NTHR - 1) / NTHR), nc);
                        k_lv_pass_copy<<<grid, NTHR, 0, st>>>(N, b, nT, cur_s, oth_s);
                    }
                    std::swap(cur_s, oth_s);
                }
            }
        }
        if (prof) cudaEventRecord(ev[3], st);
        {
            const long warps = (long)nc * nT;
            const unsigned blocks = (unsigned)std::min<long>(4096, (warps + 7) / 8);
            k_lv_dot<<<blocks, NTHR, 0, st>>>(N, nT, nc, cur_s, Y, L + (size_t)c0 * nT);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
        float ms[3] = {0, 0, 0};
        if (prof && rc == OOPS_OK && cudaEventSynchronize(ev[3]) == cudaSuccess) {
            cudaEventElapsedTime(&ms[0], ev[0], ev[1]);
            cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
            cudaEventElapsedTime(&ms[2], ev[2], ev[3]);
        }
        lv_account(K, nl, fl, prof ? ms : nullptr, launches + nl[0] + nl[1] + nl[2]);
    }
    if (prof)
        for (auto &e : ev) cudaEventDestroy(e);
    cleanup();
    if (rc == OOPS_OK) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    }
    return rc;
}

}  // namespace

void oops_prof_reset_liouville()
{
    std::lock_guard<std::mutex> lk(g_lv_mu);
    for (int k = 0; k <= LV_MAX_K; ++k)
        for (int q = 0; q < 3; ++q) {
            g_lv_ms[k][q] = 0;
            g_lv_flop[k][q] = 0;
            g_lv_n[k][q] = 0;
        }
    g_lv_launches = 0;
}

extern "C" int oops_profile_liouville(int k, int phase, double *ms, long *launches, double *flop)
{
    if (k < 1 || k > LV_MAX_K || phase < 0 || phase > 2) return oops_set_status(OOPS_ERR_ARG, "k or phase");
    std::lock_guard<std::mutex> lk(g_lv_mu);
    if (ms) *ms = g_lv_ms[k][phase];
    if (launches) *launches = g_lv_n[k][phase];
    if (flop) *flop = g_lv_flop[k][phase];
    return OOPS_OK;
}

extern "C" long oops_liouville_launches(void)
{
    std::lock_guard<std::mutex> lk(g_lv_mu);
    return g_lv_launches;
}

extern "C" int oops_cce_coherence_liouville(const double *coords_dev, size_t nbath,
                                            const unsigned *clusters_dev, size_t ncl, int k,
                                            const oops_cce_params *p, const oops_cce_bath *bath,
                                            double *L_dev, void *stream)
{
    if (!coords_dev || !clusters_dev || !p || !bath || !L_dev)
        return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (k < 1 || k > LV_MAX_K)
        return oops_set_status(OOPS_ERR_SIZE, "cluster size must be 1..6 (Liouville path: 4^k x 4^k superoperators)");
    if (p->pulse_num < 1 || p->pulse_num > 64) return oops_set_status(OOPS_ERR_SIZE, "pulse_num must be 1..64");
    if (p->nT < 1 || p->nT > (1u << 24)) return oops_set_status(OOPS_ERR_SIZE, "nT out of range");
    if (!(bath->dephasing_rate >= 0.0) || !std::isfinite(bath->dephasing_rate))
        return oops_set_status(OOPS_ERR_ARG, "dephasing rate must be finite and >= 0");
    if (ncl == 0) return OOPS_OK;
    if (ncl > (1u << 30)) return oops_set_status(OOPS_ERR_SIZE, "too many clusters");
    (void)nbath;
    LvParams lp;
    lp.pp = phys_params(p);
    lp.gamma = 2.0 * PI_D * bath->dephasing_rate;
    const double *ax = bath->dephasing_axis;
    const double an = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    if (lp.gamma != 0.0 && !(an > 0.0)) return oops_set_status(OOPS_ERR_ARG, "zero dephasing axis");
    const double nx = an > 0 ? ax[0] / an : 0, ny = an > 0 ? ax[1] / an : 0, nz = an > 0 ? ax[2] / an : 0;
    lp.sg[0] = zmake(nz, 0.0);   // (0,0)
    lp.sg[1] = zmake(nx, ny);    // (1,0)
    lp.sg[2] = zmake(nx, -ny);   // (0,1)
    lp.sg[3] = zmake(-nz, 0.0);  // (1,1)
    for (int a = 0; a < 3; ++a) lp.pol[a] = bath->polarization[a];
    lp.tau = p->dt / (2.0 * p->pulse_num);
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)ncl, nT = (int)p->nT;
    switch (k) {
        case 1: return run_liouville<1>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
        case 2: return run_liouville<2>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
        case 3: return run_liouville<3>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
        case 4: return run_liouville<4>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
        case 5: return run_liouville<5>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
        default: return run_liouville<6>(coords_dev, clusters_dev, n, lp, p->pulse_num, nT, L_dev, st);
    }
}
