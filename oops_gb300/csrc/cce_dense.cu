// cce_dense.cu -- batched cluster-coherence propagation for clusters of up to
// six spin-1/2 nuclei (Hilbert dimension D = 2^k <= 64).
//
// Reference path being replaced: EnsembleCCE::cluster_evolution
// (src/source/app/ensemble_cce.cpp:33-55) -> PiecewiseFullMatrixVectorEvolution
// (src/source/quantum/QuantumEvolution/QuantumEvolutionAlgorithm.cpp:60-83),
// which exponentiates 4^k-dimensional Liouvillians with Pade (MatExp.cpp:
// 29-77) and then advances U_j^i = U_j U_j^{i-1} one product per time step.
// At zero bath polarisation and zero dephasing its observable
// L(t) = Re <d rho0, rho(t)> (ensemble_cce.cpp:104-113) equals
//   L(t) = Re Tr[B1(t)^+ B0(t)] / D,
//   B0 = U0(s0 t) U1(s1 t) U0(s2 t) ...,  B1 = the same with 0 <-> 1,
// with U_a(tau) = exp(-i H_a tau), H_0/H_1 the NV-conditional Hamiltonians and
// s_j the CPMG interval fractions (Pulse_Interval, misc.cpp:59-84).
//
// GB300 design:
//   1. assemble H_0 and H_1 directly from the resident bath coordinates
//      (dipolar pairs, Zeeman, hyperfine mean field: SpinInteraction.cpp,
//      misc.cpp:11-57), FP64 (k_assemble_eig: one CTA per Hamiltonian, from
//      a device work queue);
//   2. diagonalise both in shared memory: cyclic Jacobi in FP32, two
//      Newton-Schulz steps and V^H A V in FP64, cyclic Jacobi in FP64 to
//      rounding level (the FP64-heavy step: D^3 work once per cluster);
//   3. M = V0^+ V1 (FP64, plus an FP32 copy) and the per-cluster phase steps;
//   4. every time point independently: in the eigenbasis of H_0, U_0 is a
//      diagonal of phases and U_1 = M diag(e^{-i w1 tau}) M^+, so B0 and B1 are
//      short chains of D x D products (one warp per item for D <= 16, one CTA
//      per cluster and time slice for D = 32, 64; six-spin clusters in mixed
//      precision on the tensor cores, cce_tc.cu).  No power is carried from
//      one time point to the next, so rounding does not accumulate along the
//      grid; this is what lets step 4 run in FP32 (the "mixed" precision mode)
//      within 1e-6 of the FP64 oracle, while FP64 mode reproduces it to
//      ~1e-11.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "oops_cce.h"
#include "cce_phys.cuh"
#include "oops_common.cuh"
#include "oops_internal.h"

namespace {

// ---------------------------------------------------------------------------
// Kernel 2: per time point coherence from (w0, w1, M).  T = double or float.
// ---------------------------------------------------------------------------
template <typename T> struct cplx;
template <> struct cplx<double> { typedef double2 t; };
template <> struct cplx<float> { typedef float2 t; };

template <typename T, typename C>
__device__ inline C cmk(T r, T i)
{
    C z;
    z.x = r;
    z.y = i;
    return z;
}

// C = A * op(B), D x D column-major; op(B) = B or B^H.  Each thread owns a
// TR x TC output tile (TR = 4 at D = 64 keeps shared-memory loads at one per
// four FMAs; TC = 2 there when NTH = 512 threads share the product).
template <int D, bool BH, typename T, typename CT, int NTH = 256>
__device__ void cta_mm(const CT *A, const CT *B, CT *Cm)
{
    constexpr int TR = D >= 64 ? 4 : (D >= 32 ? 2 : 1);  // D = 16: one output per thread
    constexpr int TC = (D >= 64 && NTH >= 512) ? 2 : TR;
    constexpr int NT = (D / TR) * (D / TC);
    for (int tile = threadIdx.x; tile < NT; tile += blockDim.x) {
        const int r0 = (tile % (D / TR)) * TR, c0 = (tile / (D / TR)) * TC;
        T ar[TR][TC], ai[TR][TC];
#pragma unroll
        for (int a = 0; a < TR; ++a)
#pragma unroll
            for (int b = 0; b < TC; ++b) { ar[a][b] = 0; ai[a][b] = 0; }
#pragma unroll 4
        for (int l = 0; l < D; ++l) {
            CT av[TR], bv[TC];
#pragma unroll
            for (int a = 0; a < TR; ++a) av[a] = A[(r0 + a) + D * l];
#pragma unroll
            for (int b = 0; b < TC; ++b) {
                if (BH) {
                    CT q = B[(c0 + b) + D * l];
                    bv[b] = cmk<T, CT>(q.x, -q.y);
                } else {
                    bv[b] = B[l + D * (c0 + b)];
                }
            }
#pragma unroll
            for (int a = 0; a < TR; ++a)
#pragma unroll
                for (int b = 0; b < TC; ++b) {
                    ar[a][b] = fma(av[a].x, bv[b].x, ar[a][b]);
                    ar[a][b] = fma(-av[a].y, bv[b].y, ar[a][b]);
                    ai[a][b] = fma(av[a].x, bv[b].y, ai[a][b]);
                    ai[a][b] = fma(av[a].y, bv[b].x, ai[a][b]);
                }
        }
#pragma unroll
        for (int a = 0; a < TR; ++a)
#pragma unroll
            for (int b = 0; b < TC; ++b) Cm[(r0 + a) + D * (c0 + b)] = cmk<T, CT>(ar[a][b], ai[a][b]);
    }
    __syncthreads();
}

// G = V V^H (FP64, D x D column-major), which is Hermitian: only the 2 x 2
// tiles on and above the diagonal are computed, with cta_mm's FMA order per
// entry, and each tile above it is also written as its conjugate transpose.
// A warp's FP64 instruction holds its sub-partition's FP64 pipe for all 32
// lanes, so the tiles are dealt out in order and whole warps fall idle: at
// D = 64 the 528 tiles fill 16 warps of 512 threads and 16 lanes of a second
// round, and the busiest sub-partition runs 5 tiles' worth of FMAs where the
// full product (cta_mm, 4 x 2 tiles) runs 8.  Used at D = 64 only (below it
// the full product's tiles are already one per thread).
template <int D>
__device__ void herm_gram(const zd *V, zd *G)
{
    constexpr int NB = D / 2;
    constexpr int NTILE = NB * (NB + 1) / 2;
    for (int u = threadIdx.x; u < NTILE; u += blockDim.x) {
        int b = (int)((sqrtf(8.0f * (float)u + 1.0f) - 1.0f) * 0.5f);
        while (b * (b + 1) / 2 > u) --b;
        while ((b + 1) * (b + 2) / 2 <= u) ++b;
        const int a = u - b * (b + 1) / 2;  // a <= b
        const int r0 = 2 * a, c0 = 2 * b;
        double ar[2][2], ai[2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) { ar[i][j] = 0.0; ai[i][j] = 0.0; }
#pragma unroll 4
        for (int l = 0; l < D; ++l) {
            const zd av[2] = {V[r0 + D * l], V[r0 + 1 + D * l]};
            const zd y0 = V[c0 + D * l], y1 = V[c0 + 1 + D * l];
            const zd bv[2] = {zmake(y0.x, -y0.y), zmake(y1.x, -y1.y)};
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    ar[i][j] = fma(av[i].x, bv[j].x, ar[i][j]);
                    ar[i][j] = fma(-av[i].y, bv[j].y, ar[i][j]);
                    ai[i][j] = fma(av[i].x, bv[j].y, ai[i][j]);
                    ai[i][j] = fma(av[i].y, bv[j].x, ai[i][j]);
                }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int r = r0 + i, c = c0 + j;
                G[r + D * c] = zmake(ar[i][j], ai[i][j]);
                if (a < b) G[c + D * r] = zmake(ar[i][j], -ai[i][j]);
            }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Eigensolver building blocks (one CTA, matrices in shared memory)
// ---------------------------------------------------------------------------
template <typename T, int H2>
struct JacobiShared {
    T cs[H2], sn[H2];
    typename cplx<T>::t ph[H2];
    int pr[H2][2];
    int rot;
};

template <typename T, typename CT>
__device__ inline CT cmul(CT a, CT b)
{
    return cmk<T, CT>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// 1 / sqrt(x) and 1 / x for FP64 x within the FP32 range: an FP32 seed
// refined by two Newton steps, r <- r (3 - x r^2) / 2 and r <- r (2 - x r),
// each of which doubles the number of correct bits (23 -> 46 -> FP64
// rounding).  Only for values the FP32 seed can represent.
template <typename T>
__device__ inline T rsqrt_newton(T x)
{
    T r = (T)rsqrtf((float)x);
    r = r * ((T)1.5 - (T)0.5 * x * r * r);
    r = r * ((T)1.5 - (T)0.5 * x * r * r);
    return r;
}
template <typename T>
__device__ inline T rcp_newton(T x)
{
    T r = (T)(1.0f / (float)x);
    r = r * ((T)2 - x * r);
    r = r * ((T)2 - x * r);
    return r;
}

// (u, v) <- (c u - s (v e), s u + c (v e))
template <typename T, typename CT>
__device__ inline void rot_pair(CT &u, CT &v, T c, T s, CT e)
{
    const CT ve = cmul<T, CT>(v, e);
    const CT nu = cmk<T, CT>(c * u.x - s * ve.x, c * u.y - s * ve.y);
    v = cmk<T, CT>(s * u.x + c * ve.x, s * u.y + c * ve.y);
    u = nu;
}

// Cyclic Jacobi on the Hermitian D x D matrix A (column-major), rotations
// accumulated into V, round-robin disjoint pairs (D/2 rotations per round).
// A pair is rotated while |a_pq| > thresh and |a_pq| > rel |a_qq - a_pp|:
// with rel > 0 a pair whose rotation would move the eigenvectors by less
// than rel (and the eigenvalues by less than rel |a_pq|) is left alone.
// Returns 1 when a sweep rotated nothing, 0 after max_sweeps.
template <int D, typename T>
__device__ int jacobi_sweeps(typename cplx<T>::t *A, typename cplx<T>::t *V, T thresh,
                             int max_sweeps, JacobiShared<T, (D / 2 > 0 ? D / 2 : 1)> &js,
                             T rel = 0)
{
    typedef typename cplx<T>::t CT;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) js.rot = 0;
        __syncthreads();
        for (int rnd = 0; rnd < D - 1; ++rnd) {
            if (threadIdx.x < D / 2) {
                const int t = threadIdx.x;
                int p, q;
                if (t == 0) { p = D - 1; q = rnd; }
                else { p = (rnd + t) % (D - 1); q = (rnd - t + (D - 1)) % (D - 1); }
                if (p > q) { int s = p; p = q; q = s; }
                js.pr[t][0] = p;
                js.pr[t][1] = q;
                const CT apq = A[p + D * q];
                const T mag2 = apq.x * apq.x + apq.y * apq.y;
                const T app = A[p + D * p].x, aqq = A[q + D * q].x;
                // squared comparison: pairs below the threshold (all of them
                // in the final sweep) need no square root
                const T gap = aqq - app;
                if (!(mag2 > thresh * thresh) || mag2 < (T)(sizeof(T) == 4 ? 1e-30 : 1e-60) ||
                    !(mag2 > rel * rel * gap * gap)) {
                    js.cs[t] = 1;
                    js.sn[t] = 0;
                    js.ph[t] = cmk<T, CT>(1, 0);
                } else if (sizeof(T) == 8 && mag2 > 1e-30 && mag2 < 1e30) {
                    // FP64: reciprocals and inverse square roots by Newton's
                    // method from FP32 seeds (~40 FP64 instructions instead
                    // of ~140 for library divisions and square roots; FP64
                    // issues at 1/64 of the FP32 rate and this phase runs on
                    // one warp between barriers)
                    const T rinv = rsqrt_newton(mag2);                 // 1 / |a_pq|
                    T zeta = (aqq - app) * (T)0.5 * rinv;
                    T tt;
                    if (fabs(zeta) < (T)1e15) {
                        const T u = 1 + zeta * zeta;
                        tt = rcp_newton(fabs(zeta) + u * rsqrt_newton(u));
                    } else {
                        tt = (T)0.5 * rcp_newton(fabs(zeta));           // 1 / (2 |zeta|)
                    }
                    if (zeta < 0) tt = -tt;
                    const T c = rsqrt_newton(1 + tt * tt);
                    js.cs[t] = c;
                    js.sn[t] = tt * c;
                    js.ph[t] = cmk<T, CT>(apq.x * rinv, -apq.y * rinv);  // e^{-i phi}
                    js.rot = 1;
                } else if (sizeof(T) == 4) {
                    // FP32 phase: approximate eigenvectors only (the FP64
                    // phase re-orthonormalises V and rotates V^H A V from the
                    // original A), so hardware reciprocal square roots and
                    // fast divisions replace the IEEE sequences in this
                    // serial chain between barriers
                    const float rinv = rsqrtf((float)mag2);             // 1 / |a_pq|
                    const float zeta = ((float)aqq - (float)app) * 0.5f * rinv;
                    const float az = fabsf(zeta);
                    float tt;
                    if (az < 1e15f) {
                        const float u = fmaf(zeta, zeta, 1.0f);
                        tt = __fdividef(1.0f, az + u * rsqrtf(u));
                    } else {
                        tt = __fdividef(0.5f, az);
                    }
                    if (zeta < 0.0f) tt = -tt;
                    const float c = rsqrtf(fmaf(tt, tt, 1.0f));
                    js.cs[t] = (T)c;
                    js.sn[t] = (T)(tt * c);
                    js.ph[t] = cmk<T, CT>((T)((float)apq.x * rinv), (T)(-(float)apq.y * rinv));  // e^{-i phi}
                    js.rot = 1;
                } else {
                    const T mag = sqrt(mag2);
                    const T zeta = (aqq - app) / (2 * mag);
                    const T tt = (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt(1 + zeta * zeta));
                    const T c = 1 / sqrt(1 + tt * tt);
                    js.cs[t] = c;
                    js.sn[t] = tt * c;
                    js.ph[t] = cmk<T, CT>(apq.x / mag, -apq.y / mag);  // e^{-i phi}
                    js.rot = 1;
                }
            }
            __syncthreads();
            // A <- J^H A J, block by block: for the pairs a, b of this round
            // the 2 x 2 block of rows {p_a, q_a} and columns {p_b, q_b}
            // becomes J_a^H A_ab J_b, which depends on that block only
            // (J = [[c, s], [-s e, c e]] on columns p, q; e = e^{-i phi}).  A
            // is Hermitian, so only blocks a <= b are computed and block
            // (b, a) is written as their conjugate transpose: half the
            // arithmetic of separate column and row passes, one barrier
            // fewer.  V <- V J in the same pass.
            constexpr int NP = D / 2 > 0 ? D / 2 : 1;
            constexpr int NB = NP * (NP + 1) / 2;
            for (int e = threadIdx.x; e < NB + NP * D; e += blockDim.x) {
                if (e < NB) {
                    int b = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
                    while (b * (b + 1) / 2 > e) --b;
                    while ((b + 1) * (b + 2) / 2 <= e) ++b;
                    const int a = e - b * (b + 1) / 2;  // a <= b
                    const bool ra = js.sn[a] != 0, rb = js.sn[b] != 0;
                    if (!ra && !rb) continue;
                    const int pa = js.pr[a][0], qa = js.pr[a][1], pb = js.pr[b][0], qb = js.pr[b][1];
                    CT x00 = A[pa + D * pb], x01 = A[pa + D * qb];
                    CT x10 = A[qa + D * pb], x11 = A[qa + D * qb];
                    if (rb) {
                        const T c = js.cs[b], s = js.sn[b];
                        const CT ep = js.ph[b];
                        rot_pair<T, CT>(x00, x01, c, s, ep);  // row p_a, columns p_b, q_b
                        rot_pair<T, CT>(x10, x11, c, s, ep);  // row q_a
                    }
                    if (ra) {
                        const T c = js.cs[a], s = js.sn[a];
                        const CT epc = cmk<T, CT>(js.ph[a].x, -js.ph[a].y);  // conj(e)
                        rot_pair<T, CT>(x00, x10, c, s, epc);  // column p_b, rows p_a, q_a
                        rot_pair<T, CT>(x01, x11, c, s, epc);  // column q_b
                    }
                    A[pa + D * pb] = x00;
                    A[pa + D * qb] = x01;
                    A[qa + D * pb] = x10;
                    A[qa + D * qb] = x11;
                    if (a != b) {
                        A[pb + D * pa] = cmk<T, CT>(x00.x, -x00.y);
                        A[qb + D * pa] = cmk<T, CT>(x01.x, -x01.y);
                        A[pb + D * qa] = cmk<T, CT>(x10.x, -x10.y);
                        A[qb + D * qa] = cmk<T, CT>(x11.x, -x11.y);
                    }
                } else {
                    const int f = e - NB, t = f / D, row = f % D;
                    if (js.sn[t] == 0) continue;
                    const int p = js.pr[t][0], q = js.pr[t][1];
                    CT vp = V[row + D * p], vq = V[row + D * q];
                    rot_pair<T, CT>(vp, vq, js.cs[t], js.sn[t], js.ph[t]);
                    V[row + D * p] = vp;
                    V[row + D * q] = vq;
                }
            }
            __syncthreads();
        }
        const int rotated = js.rot;
        __syncthreads();
        if (!rotated) return 1;
    }
    return 0;
}

// X <- M X in place (FP64, D x D column-major): one warp per column of X, the
// column held in registers while the new one is formed.
template <int D>
__device__ void left_mul_inplace(const zd *M, zd *X)
{
    constexpr int E = (D + 31) / 32;
    static_assert(E <= 2, "D <= 64");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < D; j += nw) {
        zd v[E], o[E];
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const int r = lane + 32 * q;
            v[q] = r < D ? X[r + D * j] : zmake(0, 0);
            o[q] = zmake(0, 0);
        }
#pragma unroll 4
        for (int k = 0; k < D; ++k) {
            const zd vs = (E == 1 || k < 32) ? v[0] : v[E - 1];
            const zd vk = zmake(__shfl_sync(0xffffffffu, vs.x, k & 31), __shfl_sync(0xffffffffu, vs.y, k & 31));
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int r = lane + 32 * q;
                if (r < D) {
                    const zd m = M[r + D * k];
                    o[q].x = fma(m.x, vk.x, fma(-m.y, vk.y, o[q].x));
                    o[q].y = fma(m.x, vk.y, fma(m.y, vk.x, o[q].y));
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const int r = lane + 32 * q;
            if (r < D) X[r + D * j] = o[q];
        }
    }
    __syncthreads();
}

// W <- A V for a cluster Hamiltonian A (FP64, D = 2^K): A's entry (r, c) is
// zero unless r and c differ in at most two spins, so row r has the
// 1 + K + K(K-1)/2 nonzeros at c = r ^ m for the masks m of at most two bits
// (22 of 64 at K = 6).  One warp per column of V; a lane's 16-byte reads of A
// and V fall into distinct bank groups for distinct r mod 8.
template <int K>
__device__ void ham_mul(const zd *A, const zd *V, zd *W)
{
    constexpr int D = 1 << K;
    constexpr int E = (D + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < D; j += nw) {
#pragma unroll 1
        for (int q = 0; q < E; ++q) {
            const int r = lane + 32 * q;
            if (r >= D) continue;
            const zd *vj = V + D * j;
            zd o = zmake(0.0, 0.0);
            auto acc = [&](int c) {
                const zd a = A[r + D * c], v = vj[c];
                o.x = fma(a.x, v.x, fma(-a.y, v.y, o.x));
                o.y = fma(a.x, v.y, fma(a.y, v.x, o.y));
            };
            acc(r);
#pragma unroll
            for (int i = 0; i < K; ++i) {
                acc(r ^ (1 << i));
#pragma unroll
                for (int i2 = i + 1; i2 < K; ++i2) acc(r ^ (1 << i) ^ (1 << i2));
            }
            W[r + D * j] = o;
        }
    }
    __syncthreads();
}

// X <- X - (E X) / 2 in place (a Newton-Schulz step V <- (3I - V V^H) V / 2
// written as V - E V / 2 with E = V V^H - I): E is small (~1e-6, then
// ~1e-12), so the product E X needs only FP32 precision (its absolute error
// is ~1e-7 |E|), while E and the update of X stay FP64.  One warp per column
// of X, held in registers while the new one is formed.
template <int D>
__device__ void left_correct_inplace(const float2 *Em, zd *X)
{
    constexpr int E2 = (D + 31) / 32;
    static_assert(E2 <= 2, "D <= 64");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < D; j += nw) {
        zd v[E2];
        float2 vf[E2], o[E2];
#pragma unroll
        for (int q = 0; q < E2; ++q) {
            const int r = lane + 32 * q;
            v[q] = r < D ? X[r + D * j] : zmake(0, 0);
            vf[q] = make_float2((float)v[q].x, (float)v[q].y);
            o[q] = make_float2(0.f, 0.f);
        }
#pragma unroll 4
        for (int k = 0; k < D; ++k) {
            const float2 vs = (E2 == 1 || k < 32) ? vf[0] : vf[E2 - 1];
            const float2 vk = make_float2(__shfl_sync(0xffffffffu, vs.x, k & 31), __shfl_sync(0xffffffffu, vs.y, k & 31));
#pragma unroll
            for (int q = 0; q < E2; ++q) {
                const int r = lane + 32 * q;
                if (r < D) {
                    const float2 m = Em[r + D * k];
                    o[q].x = fmaf(m.x, vk.x, fmaf(-m.y, vk.y, o[q].x));
                    o[q].y = fmaf(m.x, vk.y, fmaf(m.y, vk.x, o[q].y));
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < E2; ++q) {
            const int r = lane + 32 * q;
            if (r < D) X[r + D * j] = zmake(v[q].x - 0.5 * (double)o[q].x, v[q].y - 0.5 * (double)o[q].y);
        }
    }
    __syncthreads();
}

// The D x D complex matrix G (FP64) rounded to FP32 into the first half of
// its own storage (each of the NTH threads stages its elements in
// registers).  Converting once spares the product that reads it a conversion
// per use (D per element).
template <int D, int NTH>
__device__ float2 *to_f32_inplace(zd *G)
{
    constexpr int PER = (D * D + NTH - 1) / NTH;
    zd v[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + NTH * i;
        if (e < D * D) v[i] = G[e];
    }
    __syncthreads();
    float2 *G32 = reinterpret_cast<float2 *>(G);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + NTH * i;
        if (e < D * D) G32[e] = make_float2((float)v[i].x, (float)v[i].y);
    }
    __syncthreads();
    return G32;
}

// (x, y) <- (c x - s f y, s conj(f) x + c y): columns p, q of X J for the
// rotation J = [[c, s conj(e)], [-s e, c]] with f = e, rows p, q of J^H X
// with f = conj(e)
__device__ inline void rot2f(float2 &x, float2 &y, float c, float s, float2 f)
{
    const float2 fy = make_float2(f.x * y.x - f.y * y.y, f.x * y.y + f.y * y.x);
    const float2 fx = make_float2(f.x * x.x + f.y * x.y, f.x * x.y - f.y * x.x);  // conj(f) x
    const float2 nx = make_float2(c * x.x - s * fy.x, c * x.y - s * fy.y);
    y = make_float2(s * fx.x + c * y.x, s * fx.y + c * y.y);
    x = nx;
}

// Mixed modes: the last Jacobi phase, on S = V^H A V, which the FP32 phase
// and the Newton-Schulz steps leave diagonal up to ~2^-22 ||A||_F.  The
// diagonal stays in FP64 (dg) and the off-diagonal part is held in FP32 (N,
// scaled by the power of two sc, zero diagonal): a rotation moves the
// diagonal by -+ t |s_pq| (an FP64 update of two entries) and mixes
// off-diagonal entries with each other, so their FP32 rounding is relative to
// the small entries themselves (~2^-24 of ~2^-22 ||A||_F), not to ||A||.
// Rotations J = [[c, s conj(e)], [-s e, c]] (e = e^{-i phi}; unlike
// jacobi_sweeps' form, column q is not rephased) accumulate into
// K = J_1 J_2 ... - I in FP32, which is small except on near-degenerate
// pairs; the caller forms V (I + K) = V + V K with the product in FP32.  The
// pair criterion is jacobi_sweeps' (thresh and rel on the scaled entries).
// Returns 1 when a sweep rotated nothing, 0 after max_sweeps.
template <int D>
__device__ int jacobi_refine32(float2 *N, float2 *Km, double *dg, double sc, float thresh, float rel,
                               int max_sweeps, JacobiShared<float, (D / 2 > 0 ? D / 2 : 1)> &js)
{
    constexpr int NP = D / 2 > 0 ? D / 2 : 1;
    constexpr int NB = NP * (NP + 1) / 2;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) js.rot = 0;
        __syncthreads();
        for (int rnd = 0; rnd < D - 1; ++rnd) {
            if (threadIdx.x < D / 2) {
                const int t = threadIdx.x;
                int p, q;
                if (t == 0) { p = D - 1; q = rnd; }
                else { p = (rnd + t) % (D - 1); q = (rnd - t + (D - 1)) % (D - 1); }
                if (p > q) { int s = p; p = q; q = s; }
                js.pr[t][0] = p;
                js.pr[t][1] = q;
                const float2 apq = N[p + D * q];
                const float mag2 = apq.x * apq.x + apq.y * apq.y;
                const float gap = (float)((dg[q] - dg[p]) * sc);
                if (!(mag2 > thresh * thresh) || mag2 < 1e-30f || !(mag2 > rel * rel * gap * gap)) {
                    js.cs[t] = 1.0f;
                    js.sn[t] = 0.0f;
                    js.ph[t] = make_float2(1.0f, 0.0f);
                } else {
                    // IEEE square roots and divisions: the rotation's
                    // unitarity error stays at FP32 rounding
                    const float mag = sqrtf(mag2);
                    const float zeta = gap * 0.5f / mag;
                    float tt = 1.0f / (fabsf(zeta) + sqrtf(fmaf(zeta, zeta, 1.0f)));
                    if (zeta < 0.0f) tt = -tt;
                    const float c = 1.0f / sqrtf(fmaf(tt, tt, 1.0f));
                    js.cs[t] = c;
                    js.sn[t] = tt * c;
                    js.ph[t] = make_float2(apq.x / mag, -apq.y / mag);  // e^{-i phi}
                    const double dd = (double)(tt * mag) / sc;
                    dg[p] -= dd;
                    dg[q] += dd;
                    js.rot = 1;
                }
            }
            __syncthreads();
            for (int e = threadIdx.x; e < NB + NP * D; e += blockDim.x) {
                if (e < NB) {
                    int b = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
                    while (b * (b + 1) / 2 > e) --b;
                    while ((b + 1) * (b + 2) / 2 <= e) ++b;
                    const int a = e - b * (b + 1) / 2;  // a <= b
                    const bool ra = js.sn[a] != 0.0f, rb = js.sn[b] != 0.0f;
                    if (!ra && !rb) continue;
                    const int pa = js.pr[a][0], qa = js.pr[a][1], pb = js.pr[b][0], qb = js.pr[b][1];
                    if (a == b) {  // the rotated pair's own entry is annihilated
                        N[pa + D * qa] = make_float2(0.0f, 0.0f);
                        N[qa + D * pa] = make_float2(0.0f, 0.0f);
                        continue;
                    }
                    float2 x00 = N[pa + D * pb], x01 = N[pa + D * qb];
                    float2 x10 = N[qa + D * pb], x11 = N[qa + D * qb];
                    if (rb) {  // columns p_b, q_b
                        const float c = js.cs[b], s = js.sn[b];
                        const float2 f = js.ph[b];
                        rot2f(x00, x01, c, s, f);
                        rot2f(x10, x11, c, s, f);
                    }
                    if (ra) {  // rows p_a, q_a
                        const float c = js.cs[a], s = js.sn[a];
                        const float2 f = make_float2(js.ph[a].x, -js.ph[a].y);
                        rot2f(x00, x10, c, s, f);
                        rot2f(x01, x11, c, s, f);
                    }
                    N[pa + D * pb] = x00;
                    N[pa + D * qb] = x01;
                    N[qa + D * pb] = x10;
                    N[qa + D * qb] = x11;
                    N[pb + D * pa] = make_float2(x00.x, -x00.y);
                    N[qb + D * pa] = make_float2(x01.x, -x01.y);
                    N[pb + D * qa] = make_float2(x10.x, -x10.y);
                    N[qb + D * qa] = make_float2(x11.x, -x11.y);
                } else {
                    // K <- (I + K) J - I: rotate columns p, q of K, then add
                    // (J - I)'s entries in rows p and q
                    const int f = e - NB, t = f / D, row = f % D;
                    const float s = js.sn[t];
                    if (s == 0.0f) continue;
                    const int p = js.pr[t][0], q = js.pr[t][1];
                    const float c = js.cs[t];
                    const float2 ph = js.ph[t];
                    float2 vp = Km[row + D * p], vq = Km[row + D * q];
                    rot2f(vp, vq, c, s, ph);
                    const float cm1 = -(s * s) / (1.0f + c);  // c - 1 without cancellation
                    if (row == p) {
                        vp.x += cm1;
                        vq.x += s * ph.x;
                        vq.y -= s * ph.y;
                    } else if (row == q) {
                        vp.x -= s * ph.x;
                        vp.y -= s * ph.y;
                        vq.x += cm1;
                    }
                    Km[row + D * p] = vp;
                    Km[row + D * q] = vq;
                }
            }
            __syncthreads();
        }
        const int rotated = js.rot;
        __syncthreads();
        if (!rotated) return 1;
    }
    return 0;
}

// V <- V + V32 K (V FP64, V32 its FP32 copy, K FP32): one warp per column j,
// K's column held in registers and broadcast by shuffles
template <int D>
__device__ void add_right_mul_f32(zd *V, const float2 *V32, const float2 *Km)
{
    constexpr int E = (D + 31) / 32;
    static_assert(E <= 2, "D <= 64");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < D; j += nw) {
        float2 kv[E], o[E];
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const int r = lane + 32 * q;
            kv[q] = r < D ? Km[r + D * j] : make_float2(0.f, 0.f);
            o[q] = make_float2(0.f, 0.f);
        }
#pragma unroll 4
        for (int k = 0; k < D; ++k) {
            const float2 ks = (E == 1 || k < 32) ? kv[0] : kv[E - 1];
            const float2 kk = make_float2(__shfl_sync(0xffffffffu, ks.x, k & 31), __shfl_sync(0xffffffffu, ks.y, k & 31));
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int r = lane + 32 * q;
                if (r < D) {
                    const float2 v = V32[r + D * k];
                    o[q].x = fmaf(v.x, kk.x, fmaf(-v.y, kk.y, o[q].x));
                    o[q].y = fmaf(v.x, kk.y, fmaf(v.y, kk.x, o[q].y));
                }
            }
        }
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const int r = lane + 32 * q;
            if (r < D) {
                V[r + D * j].x += (double)o[q].x;
                V[r + D * j].y += (double)o[q].y;
            }
        }
    }
    __syncthreads();
}

// Local spin frames.  Every spin's own field h_i (Zeeman + hyperfine mean
// field) dominates its couplings (dipolar pairs are ~1e-4 of ||H||_F on the
// CCE workloads), so in the product basis where each h_i points along z the
// Hamiltonian is diagonal up to the pair terms and the cyclic Jacobi starts
// close to convergence (numpy emulation on the CCE-6 workload: 4.1 FP32
// sweeps on average and at most 5 at six spins instead of 13.6 and 15; 3.2
// and 4 instead of 8 and 9 at four spins).  The basis change is exact: with
// u_i the 2 x 2 unitary whose columns are the eigenvectors |+n>, |-n> of
// n . sigma (n = h_i / |h_i|), u_i^H S_a u_i = sum_b Q_ab S_b for a real
// orthogonal Q, so U^H H U (U = u_0 (x) ... (x) u_{K-1}) has the couplings
// h'_i = Q_i^T h_i (= |h_i| z) and J'_ij = Q_i^T J_ij Q_j and is assembled
// by hamiltonian_elem like H itself; its eigenvectors V' give H's as U V'.

// u (row-major 2 x 2: u[2 row + col]) and Q (row-major 3 x 3) of one spin
__device__ void spin_frame(const double *hv, zd *u, double *Q)
{
    const double hx = hv[0], hy = hv[1], hz = hv[2];
    const double hn = sqrt(hx * hx + hy * hy + hz * hz);
    zd u00, u01, u10, u11;
    if (!(hn > 0.0)) {
        u00 = zmake(1.0, 0.0); u01 = zmake(0.0, 0.0);
        u10 = zmake(0.0, 0.0); u11 = zmake(1.0, 0.0);
    } else {
        const double nx = hx / hn, ny = hy / hn, nz = hz / hn;
        if (nz >= 0.0) {  // |+n> ~ (1 + nz, nx + i ny), |-n> ~ (-(nx - i ny), 1 + nz)
            const double s = 1.0 / sqrt(2.0 * (1.0 + nz));
            u00 = zmake((1.0 + nz) * s, 0.0); u10 = zmake(nx * s, ny * s);
            u01 = zmake(-nx * s, ny * s);     u11 = zmake((1.0 + nz) * s, 0.0);
        } else {          // |+n> ~ (nx - i ny, 1 - nz), |-n> ~ (-(1 - nz), nx + i ny)
            const double s = 1.0 / sqrt(2.0 * (1.0 - nz));
            u00 = zmake(nx * s, -ny * s);      u10 = zmake((1.0 - nz) * s, 0.0);
            u01 = zmake(-(1.0 - nz) * s, 0.0); u11 = zmake(nx * s, ny * s);
        }
    }
    u[0] = u00; u[1] = u01; u[2] = u10; u[3] = u11;
    // M_a = u^H sigma_a u = [[Q_az, Q_ax - i Q_ay], [Q_ax + i Q_ay, -Q_az]]:
    // its (0,0) and (0,1) entries from the columns c0 = (u00, u10), c1 = (u01, u11)
    auto cc = [](zd a, zd b) { return zmake(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); };  // conj(a) b
    auto add = [](zd a, zd b) { return zmake(a.x + b.x, a.y + b.y); };
    auto sub = [](zd a, zd b) { return zmake(a.x - b.x, a.y - b.y); };
    auto mi = [](zd a) { return zmake(a.y, -a.x); };   // -i a
    auto pi = [](zd a) { return zmake(-a.y, a.x); };   //  i a
    const zd m00[3] = {add(cc(u00, u10), cc(u10, u00)), add(cc(u00, mi(u10)), cc(u10, pi(u00))),
                       sub(cc(u00, u00), cc(u10, u10))};
    const zd m01[3] = {add(cc(u00, u11), cc(u10, u01)), add(cc(u00, mi(u11)), cc(u10, pi(u01))),
                       sub(cc(u00, u01), cc(u10, u11))};
    for (int a = 0; a < 3; ++a) {
        Q[3 * a + 0] = m01[a].x;
        Q[3 * a + 1] = -m01[a].y;
        Q[3 * a + 2] = m00[a].x;
    }
}

// h_i <- Q_i^T h_i and J_ij <- Q_i^T J_ij Q_j in place, by the first K * K
// threads (each owns one pair and at most one spin).  The caller
// synchronises before and after.
template <int K>
__device__ void rotate_couplings(double *J, double *h, const double *Q)
{
    if (threadIdx.x >= K * K) return;
    const int i = threadIdx.x / K, j = threadIdx.x % K;
    if (i < j) {
        double *Jij = J + (i * K + j) * 9;
        const double *Qi = Q + 9 * i, *Qj = Q + 9 * j;
        double T[9], R[9];
        for (int a = 0; a < 3; ++a)
            for (int d = 0; d < 3; ++d)
                T[3 * a + d] = Jij[3 * a] * Qj[d] + Jij[3 * a + 1] * Qj[3 + d] + Jij[3 * a + 2] * Qj[6 + d];
        for (int b = 0; b < 3; ++b)
            for (int d = 0; d < 3; ++d)
                R[3 * b + d] = Qi[b] * T[d] + Qi[3 + b] * T[3 + d] + Qi[6 + b] * T[6 + d];
        for (int q = 0; q < 9; ++q) Jij[q] = R[q];
    }
    if (threadIdx.x < K) {
        const int s = threadIdx.x;
        const double *Qs = Q + 9 * s;
        const double a0 = h[3 * s], a1 = h[3 * s + 1], a2 = h[3 * s + 2];
        for (int b = 0; b < 3; ++b) h[3 * s + b] = a0 * Qs[b] + a1 * Qs[3 + b] + a2 * Qs[6 + b];
    }
}

// V <- (u_0 (x) ... (x) u_{K-1}) V in place (FP64, D x D column-major, spin
// 0 the most significant bit): one pass per spin over the row pairs that
// differ in its bit
template <int K>
__device__ void apply_frames(zd *V, const zd *u)
{
    constexpr int D = 1 << K;
    for (int i = 0; i < K; ++i) {
        const int b = K - 1 - i;
        const zd a00 = u[4 * i], a01 = u[4 * i + 1], a10 = u[4 * i + 2], a11 = u[4 * i + 3];
        for (int t = threadIdx.x; t < D * D / 2; t += blockDim.x) {
            const int j = t / (D / 2), pr = t % (D / 2);
            const int x0 = ((pr >> b) << (b + 1)) | (pr & ((1 << b) - 1)), x1 = x0 | (1 << b);
            const zd v0 = V[x0 + D * j], v1 = V[x1 + D * j];
            V[x0 + D * j] = zmake(a00.x * v0.x - a00.y * v0.y + a01.x * v1.x - a01.y * v1.y,
                                  a00.x * v0.y + a00.y * v0.x + a01.x * v1.y + a01.y * v1.x);
            V[x1 + D * j] = zmake(a10.x * v0.x - a10.y * v0.y + a11.x * v1.x - a11.y * v1.y,
                                  a10.x * v0.y + a10.y * v0.x + a11.x * v1.y + a11.y * v1.x);
        }
        __syncthreads();
    }
}

// dg[p] = Re(v_p^H g_p) in FP64 for the columns v_p of V and g_p of G = A V:
// the Rayleigh quotients (V is unitary to FP64 rounding), the diagonal of
// S = V^H A V.  One warp per column, reduced with shuffles.
template <int D>
__device__ void rayleigh_diag(const zd *V, const zd *G, double *dg)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int p = warp; p < D; p += nw) {
        double s = 0.0;
        for (int r = lane; r < D; r += 32) {
            const zd v = V[r + D * p], g = G[r + D * p];
            s = fma(v.x, g.x, fma(v.y, g.y, s));
        }
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) dg[p] = s;
    }
    __syncthreads();
}

// N = V^H R for p < q (FP32), mirrored to the lower triangle as its
// conjugate, zero diagonal: VH holds V^H (VH[p + D r] = conj(V[r + D p])),
// R the residual columns.  One warp per column q of R, held in registers and
// broadcast by shuffles; lanes own rows p, so VH's reads are consecutive.
template <int D>
__device__ void herm_offdiag_f32(const float2 *VH, const float2 *R, float2 *N)
{
    constexpr int E = (D + 31) / 32;
    static_assert(E <= 2, "D <= 64");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = warp; q < D; q += nw) {
        float2 rv[E], o[E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int r = lane + 32 * i;
            rv[i] = r < D ? R[r + D * q] : make_float2(0.f, 0.f);
            o[i] = make_float2(0.f, 0.f);
        }
#pragma unroll 4
        for (int k = 0; k < D; ++k) {
            const float2 rs = (E == 1 || k < 32) ? rv[0] : rv[E - 1];
            const float2 rk = make_float2(__shfl_sync(0xffffffffu, rs.x, k & 31), __shfl_sync(0xffffffffu, rs.y, k & 31));
#pragma unroll
            for (int i = 0; i < E; ++i) {
                const int p = lane + 32 * i;
                if (p < D) {
                    const float2 a = VH[p + D * k];
                    o[i].x = fmaf(a.x, rk.x, fmaf(-a.y, rk.y, o[i].x));
                    o[i].y = fmaf(a.x, rk.y, fmaf(a.y, rk.x, o[i].y));
                }
            }
        }
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int p = lane + 32 * i;
            if (p < q) {
                N[p + D * q] = o[i];
                N[q + D * p] = make_float2(o[i].x, -o[i].y);
            } else if (p == q) {
                N[p + D * q] = make_float2(0.f, 0.f);
            }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Kernel 1: assemble H for (cluster, branch) and diagonalise it (FP64)
// ---------------------------------------------------------------------------
// Threads per CTA: one CTA per SM at D = 64 (its shared memory), so 512
// threads there (16 warps to hide the FP64 and shared-memory latencies of the
// dependent chains), 256 below; registers for two CTAs per SM at D = 32,
// four below.
template <int K>
constexpr int EIG_THREADS = K >= 6 ? 512 : 256;

template <int K>
__global__ void __launch_bounds__(EIG_THREADS<K>, K >= 6 ? 1 : (K == 5 ? 2 : 4))
k_assemble_eig(const double *__restrict__ coords, const unsigned *__restrict__ clusters,
               int ncl, PhysParams pp, const double *__restrict__ xfield,
               double *__restrict__ wout, zd *__restrict__ Vout,
               int *__restrict__ queue, int *__restrict__ fail, double rel_gap)
{
    constexpr int D = 1 << K;
    constexpr int H2 = D / 2 > 0 ? D / 2 : 1;
    extern __shared__ zd sm[];
    zd *A = sm;              // D x D, column-major
    zd *V = sm + D * D;      // eigenvectors
    zd *G = sm + 2 * D * D;  // FP64 scratch; holds A32 and V32 during the FP32 phase
    float2 *A32 = reinterpret_cast<float2 *>(G), *V32 = A32 + D * D;
    __shared__ double J[MAX_K * MAX_K * 9];  // pair tensors (i<j at i*K+j)
    __shared__ double h[MAX_K * 3];          // single-spin fields
    __shared__ JacobiShared<double, H2> js64;
    __shared__ JacobiShared<float, H2> js32;
    __shared__ int s_item;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= 2 * ncl) break;
        const int cl = item >> 1, br = item & 1;
        const unsigned *idx = clusters + (size_t)cl * K;
        cluster_couplings<K>(coords, idx, pp, br, J, h);
        __syncthreads();
        if (xfield) {  // mean field of the other bath spins (single-sample CCE)
            if (threadIdx.x < 3 * K) h[threadIdx.x] += xfield[(size_t)cl * 3 * K + threadIdx.x];
            __syncthreads();
        }
        // H' = U^H H U in the spins' local frames (spin_frame); V = U V' at the end
        __shared__ zd s_u[MAX_K * 4];
        __shared__ double s_Q[MAX_K * 9];
        if (threadIdx.x < K) spin_frame(h + 3 * threadIdx.x, s_u + 4 * threadIdx.x, s_Q + 9 * threadIdx.x);
        __syncthreads();
        rotate_couplings<K>(J, h, s_Q);
        __syncthreads();
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            const int r = e % D, c = e / D;
            A[e] = hamiltonian_elem<K>(r, c, J, h);
            V[e] = zmake(r == c ? 1.0 : 0.0, 0.0);
        }
        __syncthreads();
        // Eigendecomposition, FP64 result at a third of the FP64 work of a
        // plain FP64 Jacobi (FP64 issues at 1/64 of the FP32 rate here):
        //  1. cyclic Jacobi in FP32 until the off-diagonal is ~2^-22 ||A||_F
        //     (on four-spin Hamiltonians as many FP32 sweeps as 2^-20, ~7,
        //     but no item then needs a fourth FP64 sweep; the slowest item
        //     on an SM sets the kernel's duration);
        //  2. two Newton-Schulz steps V <- (3I - V V^H) V / 2 make the FP32
        //     eigenvectors unitary to FP64 rounding (V V^H in FP64, the small
        //     correction product in FP32);
        //  3. S = V^H (A V) (nearly diagonal; A V in FP64 with A's
        //     sparsity, 22 of 64 entries per row at six spins; V^H (A V) in
        //     FP64 in the FP64 mode, and in the mixed modes its diagonal in
        //     FP64 and its off-diagonal from the FP64 residual by an FP32
        //     product);
        //  4. cyclic Jacobi in FP64 on it, rotations accumulated into V, until a
        //     sweep rotates nothing: a pair is rotated while
        //     |a_pq| > 2^-51 ||A||_F (the Frobenius norm is invariant), so the
        //     off-diagonal ends at rounding level, which near-degenerate
        //     Zeeman-split spectra need for 1e-10 accuracy of the eigenvectors.
        //     The mixed modes (rel_gap > 0) run this phase as
        //     jacobi_refine32: FP64 diagonal, FP32 off-diagonal and rotation
        //     accumulator, and a pair is left alone once its rotation would
        //     move the eigenvectors by less than rel_gap -- the eigenvalues
        //     keep FP64 accuracy, the eigenvectors FP32 accuracy, which is
        //     what the FP32 overlaps M hold.
        // Steps 1-3 serve both modes: a single Newton-Schulz step leaves V
        // unitary only to ~1e-10, which moves the eigenvalues of V^H A V by
        // ~1e-10 ||A|| -- a phase error of ~1e-4 rad at 8 ms.
        __shared__ double s_fro;
        if (threadIdx.x == 0) s_fro = 0.0;
        __syncthreads();
        {
            double loc = 0.0;
            for (int e = threadIdx.x; e < D * D; e += blockDim.x)
                loc += A[e].x * A[e].x + A[e].y * A[e].y;
            for (int off = 16; off > 0; off >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, off);
            if ((threadIdx.x & 31) == 0) atomicAdd(&s_fro, loc);
        }
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            A32[e] = make_float2((float)A[e].x, (float)A[e].y);
            V32[e] = make_float2((e % D) == (e / D) ? 1.0f : 0.0f, 0.0f);
        }
        __syncthreads();
        const double fro = sqrt(s_fro);
        const double thresh = 0x1p-51 * fro;
        jacobi_sweeps<D, float>(A32, V32, (float)(0x1p-22 * fro), 20, js32);
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) V[e] = zmake(V32[e].x, V32[e].y);
        __syncthreads();
        for (int it = 0; it < 2; ++it) {
            if constexpr (D >= 64) herm_gram<D>(V, G);  // G = V V^H
            else cta_mm<D, true, double, zd, EIG_THREADS<K>>(V, V, G);
            for (int e = threadIdx.x; e < D * D; e += blockDim.x)
                if ((e % D) == (e / D)) G[e].x -= 1.0;  // E = V V^H - I, small
            __syncthreads();
            left_correct_inplace<D>(to_f32_inplace<D, EIG_THREADS<K>>(G), V);  // V <- V - E V / 2
        }
        // S = V^H (A V): G <- A V with A's sparsity, then A's storage takes
        // V^H and G <- V^H G
        ham_mul<K>(A, V, G);  // G = A V
        if (rel_gap > 0.0) {
            // mixed modes: S = V^H A V with its diagonal in FP64 (the
            // Rayleigh quotients dg) and its off-diagonal in FP32 from the
            // FP64 residual R = G - V diag(dg), which is small (~2^-22
            // ||A||_F): S_pq = v_p^H r_q + dg_q v_p^H v_q, and the last term
            // is ~1e-16 ||A|| once V is unitary, so the FP32 product's error
            // is relative to the small entries (numpy emulation on six-spin
            // Hamiltonians of the CCE-6 workload: within 4e-14 ||A||_F of the
            // FP64 product, eigenvalues of S within 1.3e-15 ||A||_F of
            // LAPACK's) and the full FP64 product V^H G is not needed.  The
            // last Jacobi phase then runs on FP64 diagonal and FP32
            // off-diagonal (jacobi_refine32); V^H and R in A's storage, N
            // and K in G's.
            __shared__ double dg[D];
            const double sc = fro > 0.0 ? ldexp(1.0, -ilogb(fro)) : 1.0;
            rayleigh_diag<D>(V, G, dg);
            float2 *VH32 = reinterpret_cast<float2 *>(A), *R32 = VH32 + D * D;
            for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
                const int r = e % D, q = e / D;
                const zd v = V[e], g = G[e];
                R32[e] = make_float2((float)((g.x - dg[q] * v.x) * sc), (float)((g.y - dg[q] * v.y) * sc));
                VH32[q + D * r] = make_float2((float)v.x, -(float)v.y);
            }
            __syncthreads();
            float2 *N32 = reinterpret_cast<float2 *>(G), *K32 = N32 + D * D;
            for (int e = threadIdx.x; e < D * D; e += blockDim.x) K32[e] = make_float2(0.f, 0.f);
            herm_offdiag_f32<D>(VH32, R32, N32);  // N = sc * offdiag(V^H R), Hermitian
            const int conv = jacobi_refine32<D>(N32, K32, dg, sc, (float)(thresh * sc), (float)rel_gap, 24, js32);
            if (!conv) {
                __shared__ float s_res32;
                if (threadIdx.x == 0) s_res32 = 0.0f;
                __syncthreads();
                float loc = 0.0f;
                for (int e = threadIdx.x; e < D * D; e += blockDim.x)
                    loc = fmaxf(loc, sqrtf(N32[e].x * N32[e].x + N32[e].y * N32[e].y));
                for (int off = 16; off > 0; off >>= 1) loc = fmaxf(loc, __shfl_down_sync(0xffffffffu, loc, off));
                if ((threadIdx.x & 31) == 0) atomicMax((int *)&s_res32, __float_as_int(loc));
                __syncthreads();
                if (threadIdx.x == 0 && (double)s_res32 > 64.0 * thresh * sc) atomicAdd(fail, 1);
            }
            // V^H and R are spent: A's storage takes V's FP32 copy for
            // V <- V (I + K)
            float2 *V32 = reinterpret_cast<float2 *>(A);
            for (int e = threadIdx.x; e < D * D; e += blockDim.x) V32[e] = make_float2((float)V[e].x, (float)V[e].y);
            __syncthreads();
            add_right_mul_f32<D>(V, V32, K32);
            apply_frames<K>(V, s_u);
            for (int e = threadIdx.x; e < D * D; e += blockDim.x)
                Vout[((size_t)cl * 2 + br) * D * D + e] = V[e];
            for (int d = threadIdx.x; d < D; d += blockDim.x) wout[((size_t)cl * 2 + br) * D + d] = dg[d];
            continue;
        }
        // FP64 mode: S = V^H G in FP64, A's storage takes V^H first
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            const zd v = V[(e / D) + D * (e % D)];
            A[e] = zmake(v.x, -v.y);  // V^H
        }
        __syncthreads();
        left_mul_inplace<D>(A, G);
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) A[e] = G[e];
        __syncthreads();
        const int converged = jacobi_sweeps<D, double>(A, V, thresh, 24, js64, rel_gap);
        if (!converged) {
            // accept a residual within a few roundings of the threshold
            __shared__ double s_res;
            if (threadIdx.x == 0) s_res = 0.0;
            __syncthreads();
            double loc = 0.0;
            for (int e = threadIdx.x; e < D * D; e += blockDim.x)
                if (e % D != e / D) loc = fmax(loc, zabs(A[e]));
            for (int off = 16; off > 0; off >>= 1) loc = fmax(loc, __shfl_down_sync(0xffffffffu, loc, off));
            if ((threadIdx.x & 31) == 0) atomicMax((unsigned long long *)&s_res, __double_as_longlong(loc));
            __syncthreads();
            if (threadIdx.x == 0 && s_res > 64.0 * thresh) atomicAdd(fail, 1);
        }
        apply_frames<K>(V, s_u);
        for (int e = threadIdx.x; e < D * D; e += blockDim.x)
            Vout[((size_t)cl * 2 + br) * D * D + e] = V[e];
        for (int d = threadIdx.x; d < D; d += blockDim.x)
            wout[((size_t)cl * 2 + br) * D + d] = A[d + D * d].x;
    }
}

// e^{-i x}: FP64 sincos for T = double; FP64 range reduction then FP32
// sincosf for T = float (|error| ~ 1e-7, the precision of that mode)
template <typename T, typename CT>
__device__ inline CT phase(double x)
{
    if (sizeof(T) == 8) {
        double s, c;
        sincos(-x, &s, &c);
        return cmk<T, CT>((T)c, (T)s);
    } else {
        const double twopi = 6.283185307179586476925286766559;
        double r = x - twopi * rint(x * (1.0 / twopi));
        float s, c;
        sincosf(-(float)r, &s, &c);
        return cmk<T, CT>((T)c, (T)s);
    }
}

// Phase advance per time step, once per cluster: phi[((cl*2 + br)*2 + f)*D + d]
// = frac(w_br[d] * dt * frac_f / 2 pi) as a 64-bit fixed-point fraction of a
// turn (f = 0: the half interval fh, f = 1: the full interval ff), for the FP32
// coherence kernels' phase_step_f.  53 significant bits; the phase of time
// point i is i * phi modulo one turn.
template <int K>
__global__ void k_phase_steps(const double *__restrict__ w, int ncl, double dt, double fh, double ff,
                              unsigned long long *__restrict__ phi)
{
    constexpr int D = 1 << K;
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (size_t)ncl * 4 * D) return;
    const int d = (int)(g % D);
    const size_t q = g / D;                 // (cl*2 + br)*2 + f
    const int f = (int)(q & 1);
    const size_t cb = q >> 1;               // cl*2 + br
    const double x = w[cb * D + d] * (dt * (f ? ff : fh)) * (1.0 / 6.283185307179586476925286766559);
    const double fr = x - floor(x);         // [0, 1)
    double m = rint(fr * 0x1p53);           // integer in [0, 2^53]
    if (m >= 0x1p53) m = 0.0;
    phi[g] = ((unsigned long long)m) << 11;
}

// L(t_i), i in the cluster's time slice.  Workspace per CTA: six D x D
// buffers (M, Y_h, Y_f and a pool of three for the two branch chains) in
// shared memory when they fit, else in gws (global, L2-resident).
template <int K, typename T>
__global__ void __launch_bounds__(256)
k_coherence(const double *__restrict__ w, const unsigned long long *__restrict__ phi,
            const zd *__restrict__ Mg, const float2 *__restrict__ Mg32, int ncl, int pulse_num,
            int nT, double dt, int tslices,
            double *__restrict__ L, int *__restrict__ queue, typename cplx<T>::t *__restrict__ gws,
            int use_smem)
{
    typedef typename cplx<T>::t CT;
    constexpr int D = 1 << K;
    constexpr int DD = D * D;
    extern __shared__ unsigned char smraw[];
    __shared__ double w0s[D], w1s[D];          // FP64 mode: eigenvalues
    __shared__ unsigned long long phs[4 * D];  // FP32 mode: phase steps [br][h, f][d]
    __shared__ CT e1h[D], e1f[D], e0h[D], e0f[D];
    __shared__ double frac_s[65];
    __shared__ int s_item;
    __shared__ T red[24];
    CT *ws = use_smem ? reinterpret_cast<CT *>(smraw) : gws + (size_t)blockIdx.x * 6 * DD;
    CT *Mx = ws, *Yh = ws + DD, *Yf = ws + 2 * DD;
    CT *pool[3] = {ws + 3 * DD, ws + 4 * DD, ws + 5 * DD};
    const int nseg = pulse_num + 1;
    if (threadIdx.x == 0) {
        double prev = 0.0;
        for (int i = 0; i < pulse_num; ++i) {
            double tt = (2.0 * i + 1.0) / (2.0 * pulse_num);
            frac_s[i] = tt - prev;
            prev = tt;
        }
        frac_s[pulse_num] = 1.0 - prev;
    }
    __syncthreads();
    const double fh = frac_s[0];
    const double ff = frac_s[nseg > 2 ? 1 : 0];
    const bool two = fh != ff;
    const int per = (nT + tslices - 1) / tslices;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= ncl * tslices) break;
        const int cl = item / tslices, sl = item % tslices;
        if constexpr (sizeof(T) == 8) {
            for (int d = threadIdx.x; d < D; d += blockDim.x) {
                w0s[d] = w[((size_t)cl * 2 + 0) * D + d];
                w1s[d] = w[((size_t)cl * 2 + 1) * D + d];
            }
        } else {
            for (int e = threadIdx.x; e < 4 * D; e += blockDim.x) phs[e] = phi[(size_t)cl * 4 * D + e];
        }
        for (int e = threadIdx.x; e < DD; e += blockDim.x) {
            if constexpr (sizeof(T) == 4) {
                const float2 m = Mg32[(size_t)cl * DD + e];  // FP32 copy: no FP64 conversion
                Mx[e] = cmk<T, CT>(m.x, m.y);
            } else {
                const zd m = Mg[(size_t)cl * DD + e];
                Mx[e] = cmk<T, CT>((T)m.x, (T)m.y);
            }
        }
        __syncthreads();
        const int i0 = sl * per, i1 = min(nT, i0 + per);
        for (int i = i0; i < i1; ++i) {
            if (i == 0) {
                if (threadIdx.x == 0) L[(size_t)cl * nT] = 1.0;
                continue;
            }
            const double t = (double)i * dt;
            for (int d = threadIdx.x; d < D; d += blockDim.x) {
                if constexpr (sizeof(T) == 8) {
                    e1h[d] = phase<T, CT>(w1s[d] * (t * fh));
                    e1f[d] = phase<T, CT>(w1s[d] * (t * ff));
                    e0h[d] = phase<T, CT>(w0s[d] * (t * fh));
                    e0f[d] = phase<T, CT>(w0s[d] * (t * ff));
                } else {
                    const float2 a = phase_step_f(phs[0 * D + d], i), b = phase_step_f(phs[1 * D + d], i);
                    const float2 c = phase_step_f(phs[2 * D + d], i), q = phase_step_f(phs[3 * D + d], i);
                    e0h[d] = cmk<T, CT>(a.x, a.y);
                    e0f[d] = cmk<T, CT>(b.x, b.y);
                    e1h[d] = cmk<T, CT>(c.x, c.y);
                    e1f[d] = cmk<T, CT>(q.x, q.y);
                }
            }
            __syncthreads();
            // Y = (M diag(e1)) M^+
            for (int e = threadIdx.x; e < DD; e += blockDim.x) {
                const int c = e / D;
                const CT m = Mx[e];
                CT a = e1h[c];
                pool[0][e] = cmk<T, CT>(m.x * a.x - m.y * a.y, m.x * a.y + m.y * a.x);
                if (two) {
                    a = e1f[c];
                    pool[1][e] = cmk<T, CT>(m.x * a.x - m.y * a.y, m.x * a.y + m.y * a.x);
                }
            }
            __syncthreads();
            cta_mm<D, true, T, CT>(pool[0], Mx, Yh);
            if (two) cta_mm<D, true, T, CT>(pool[1], Mx, Yf);
            CT *res[2] = {nullptr, nullptr};
            int freebuf[3] = {0, 1, 2};
            for (int br = 0; br < 2; ++br) {
                CT *cur = pool[freebuf[br == 0 ? 0 : 1]];
                CT *tmp = pool[freebuf[br == 0 ? 1 : 2]];
                // a chain that starts with U0 is diag(dstart) until its first
                // Y factor, which then is a row scaling, not a product
                bool started = false;
                const CT *dstart = nullptr;
                for (int j = 0; j < nseg; ++j) {
                    const bool outer = (j == 0 || j == nseg - 1);
                    if (((j + br) & 1) == 0) {  // U0 segment: diagonal phases
                        const CT *e0 = outer ? e0h : e0f;
                        if (!started) {
                            dstart = e0;
                        } else {
                            for (int e = threadIdx.x; e < DD; e += blockDim.x) {
                                const CT d = e0[e / D];
                                const CT x = cur[e];
                                cur[e] = cmk<T, CT>(x.x * d.x - x.y * d.y, x.x * d.y + x.y * d.x);
                            }
                            __syncthreads();
                        }
                    } else {  // U1 segment: Y factor
                        const CT *Y = (outer || !two) ? Yh : Yf;
                        if (!started) {
                            for (int e = threadIdx.x; e < DD; e += blockDim.x) cur[e] = Y[e];
                            __syncthreads();
                        } else if (dstart) {
                            for (int e = threadIdx.x; e < DD; e += blockDim.x) {
                                const CT d = dstart[e % D], y = Y[e];
                                cur[e] = cmk<T, CT>(d.x * y.x - d.y * y.y, d.x * y.y + d.y * y.x);
                            }
                            dstart = nullptr;
                            __syncthreads();
                        } else {
                            cta_mm<D, false, T, CT>(cur, Y, tmp);
                            CT *sw = cur;
                            cur = tmp;
                            tmp = sw;
                        }
                    }
                    started = true;
                }
                if (dstart) {  // a chain of one diagonal factor
                    for (int e = threadIdx.x; e < DD; e += blockDim.x)
                        cur[e] = (e % D == e / D) ? dstart[e % D] : cmk<T, CT>(0, 0);
                    __syncthreads();
                }
                res[br] = cur;
                if (br == 0) {
                    // branch 1 works in the two pool buffers that do not hold res[0]
                    int k2 = 0;
                    for (int q = 0; q < 3; ++q)
                        if (pool[q] != res[0]) freebuf[1 + k2++] = q;
                }
            }
            // L = Re Tr(B1^+ B0) / D in the normalised difference form
            // (coherence_from_sums): the error stays proportional to
            // sqrt(1 - L) -- most clusters have L_C close to 1, and their
            // product over thousands of clusters would otherwise collect every
            // cluster's absolute rounding error -- and a common norm drift of
            // the FP32 chains cancels.
            // per-thread partial sums in T (FP32 mode: DD/256 entries per
            // thread), the cross-thread reduction in FP64
            T tr = 0, t0 = 0, t1 = 0;
            for (int e = threadIdx.x; e < DD; e += blockDim.x) {
                const CT b1 = res[1][e], b0 = res[0][e];
                const T dr = b0.x - b1.x, di = b0.y - b1.y;
                tr = fma(dr, dr, fma(di, di, tr));
                t0 = fma(b0.x, b0.x, fma(b0.y, b0.y, t0));
                t1 = fma(b1.x, b1.x, fma(b1.y, b1.y, t1));
            }
            // FP32 mode: cross-thread sums and the defect in FP32, 1 - x in
            // FP64; FP64 mode: all in FP64 (T = double)
            for (int off = 16; off > 0; off >>= 1) {
                tr += __shfl_down_sync(0xffffffffu, tr, off);
                t0 += __shfl_down_sync(0xffffffffu, t0, off);
                t1 += __shfl_down_sync(0xffffffffu, t1, off);
            }
            if ((threadIdx.x & 31) == 0) {
                red[threadIdx.x >> 5] = tr;
                red[8 + (threadIdx.x >> 5)] = t0;
                red[16 + (threadIdx.x >> 5)] = t1;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                T sum = 0, s0 = 0, s1 = 0;
                for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
                    sum += red[q];
                    s0 += red[8 + q];
                    s1 += red[16 + q];
                }
                if constexpr (sizeof(T) == 4)
                    L[(size_t)cl * nT + i] = 1.0 - (double)coherence_defect_f(s0, s1, sum);
                else
                    L[(size_t)cl * nT + i] = coherence_from_sums(s0, s1, sum);
            }
            __syncthreads();
        }
    }
}

// Clusters of up to four spins (D <= 16): one warp per (cluster, time point)
// for D >= 8, one group of D*D lanes per item for D = 2, 4 (8 or 2 items per
// warp); matrices in a group-private slice of shared memory, warp-level
// synchronisation only.  A 256-thread CTA per item would leave most threads
// idle at D = 2..8 and pay a CTA barrier per product at D = 16.
template <int D, typename T, typename CT>
__device__ inline void warp_mm(const CT *A, const CT *B, CT *Cm, bool bh)
{
    if constexpr (D * D >= 32) {
        // register tile: each lane owns R consecutive rows of one column, so
        // one B element and R A elements are loaded per k step (R complex
        // multiply-adds per B load instead of one)
        constexpr int R = D * D / 32;
        constexpr int LPC = D / R;
        const int lane = threadIdx.x & 31;
        const int c = lane / LPC, r0 = (lane % LPC) * R;
        T ar[R], ai[R];
#pragma unroll
        for (int i = 0; i < R; ++i) ar[i] = ai[i] = 0;
#pragma unroll
        for (int l = 0; l < D; ++l) {
            CT b;
            if (bh) {
                const CT q = B[c + D * l];
                b = cmk<T, CT>(q.x, -q.y);
            } else {
                b = B[l + D * c];
            }
            CT av[R];
            if constexpr (sizeof(CT) == 8 && R % 2 == 0) {
                // FP32: two complex entries per 16-byte load (r0 is a multiple
                // of R, the buffers 16-byte aligned)
                const float4 *ap = reinterpret_cast<const float4 *>(A + r0 + D * l);
#pragma unroll
                for (int i = 0; i < R / 2; ++i) {
                    const float4 q = ap[i];
                    av[2 * i] = cmk<T, CT>(q.x, q.y);
                    av[2 * i + 1] = cmk<T, CT>(q.z, q.w);
                }
            } else {
#pragma unroll
                for (int i = 0; i < R; ++i) av[i] = A[r0 + i + D * l];
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const CT a = av[i];
                ar[i] = fma(a.x, b.x, ar[i]);
                ar[i] = fma(-a.y, b.y, ar[i]);
                ai[i] = fma(a.x, b.y, ai[i]);
                ai[i] = fma(a.y, b.x, ai[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) Cm[r0 + i + D * c] = cmk<T, CT>(ar[i], ai[i]);
        __syncwarp();
        return;
    }
    // D*D < 32: lanes are in groups of D*D (one item per group), one element each
    {
        const int e = (threadIdx.x & 31) % (D * D);
        const int r = e % D, c = e / D;
        T ar = 0, ai = 0;
#pragma unroll
        for (int l = 0; l < D; ++l) {
            const CT a = A[r + D * l];
            CT b;
            if (bh) {
                const CT q = B[c + D * l];
                b = cmk<T, CT>(q.x, -q.y);
            } else {
                b = B[l + D * c];
            }
            ar = fma(a.x, b.x, ar);
            ar = fma(-a.y, b.y, ar);
            ai = fma(a.x, b.y, ai);
            ai = fma(a.y, b.x, ai);
        }
        Cm[e] = cmk<T, CT>(ar, ai);
    }
    __syncwarp();
}

template <int K, typename T>
constexpr int warp_kernel_warps()
{
    // dynamic shared memory stays under ~100 KB per CTA (two CTAs per SM)
    return (6 * (1 << (2 * K)) * (int)sizeof(typename cplx<T>::t) * 8 <= 100 * 1024) ? 8 : 4;
}
// lanes per item
template <int K>
constexpr int warp_group()
{
    return (1 << (2 * K)) >= 32 ? 32 : (1 << (2 * K));
}
template <int K, typename T>
constexpr size_t warp_kernel_smem()
{
    return (size_t)warp_kernel_warps<K, T>() * (32 / warp_group<K>()) * 6 * (1 << (2 * K)) *
           sizeof(typename cplx<T>::t);
}

// D = 16: two CTAs per SM at most (the warp-private matrices take ~100 KB of
// shared memory per CTA), so up to 128 registers per thread; smaller D: four
// CTAs per SM, up to 64 registers
template <int K, typename T>
__global__ void __launch_bounds__(256, K >= 4 ? 2 : 4)
k_coherence_warp(const double *__restrict__ w, const unsigned long long *__restrict__ phi,
                 const zd *__restrict__ Mg, const float2 *__restrict__ Mg32, int ncl, int pulse_num,
                 int nT, double dt,
                 double *__restrict__ L)
{
    typedef typename cplx<T>::t CT;
    constexpr int D = 1 << K;
    constexpr int DD = D * D;
    constexpr int WARPS = warp_kernel_warps<K, T>();
    constexpr int G = warp_group<K>();
    constexpr int IPW = 32 / G;
    extern __shared__ unsigned char wsmraw[];
    CT(*buf)[6 * DD] = reinterpret_cast<CT(*)[6 * DD]>(wsmraw);
    __shared__ CT ph[WARPS * IPW][4 * D];
    __shared__ double frac_s[65];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int glane = lane % G, slot = wid * IPW + lane / G;
    if (threadIdx.x == 0) {
        double prev = 0.0;
        for (int i = 0; i < pulse_num; ++i) {
            double tt = (2.0 * i + 1.0) / (2.0 * pulse_num);
            frac_s[i] = tt - prev;
            prev = tt;
        }
        frac_s[pulse_num] = 1.0 - prev;
    }
    __syncthreads();
    const int nseg = pulse_num + 1;
    const double fh = frac_s[0];
    const double ff = frac_s[nseg > 2 ? 1 : 0];
    const bool two = fh != ff;
    CT *Mx = buf[slot], *Yh = Mx + DD, *Yf = Mx + 2 * DD;
    CT *pool[3] = {Mx + 3 * DD, Mx + 4 * DD, Mx + 5 * DD};
    CT *e1h = ph[slot], *e1f = e1h + D, *e0h = e1h + 2 * D, *e0f = e1h + 3 * D;
    const long long total = (long long)ncl * nT;
    // D >= 8 (one item per warp): each warp takes a contiguous run of items,
    // mostly time points of one cluster, so M is loaded once per cluster and
    // not once per time point (the launch is one wave sized by occupancy).
    // D <= 4 (several items per warp): warp-strided items; every group of a
    // warp runs the same number of iterations (warp-wide __syncwarp), a group
    // past the end recomputes the last item and does not store it.
    long long b0, b_end, b_step;
    if constexpr (G == 32) {
        const long long nw = (long long)gridDim.x * WARPS;
        const long long chunk = (total + nw - 1) / nw;
        b0 = ((long long)blockIdx.x * WARPS + wid) * chunk;
        b_end = b0 + chunk < total ? b0 + chunk : total;
        b_step = 1;
    } else {
        b0 = ((long long)blockIdx.x * WARPS + wid) * IPW;
        b_end = total;
        b_step = (long long)gridDim.x * WARPS * IPW;
    }
    int m_cl = -1;  // cluster whose M is in Mx
    for (long long base = b0; base < b_end; base += b_step) {
        const long long item0 = base + lane / G;
        const bool valid = item0 < total;
        const long long item = valid ? item0 : total - 1;
        const int cl = (int)(item / nT), i = (int)(item % nT);
        const double t = (double)i * dt;
        const double *w0 = w + ((size_t)cl * 2 + 0) * D, *w1 = w + ((size_t)cl * 2 + 1) * D;
        if (cl != m_cl) {
            for (int e = glane; e < DD; e += G) {
                if constexpr (sizeof(T) == 4) {
                    const float2 m = Mg32[(size_t)cl * DD + e];  // FP32 copy: no FP64 conversion
                    Mx[e] = cmk<T, CT>(m.x, m.y);
                } else {
                    const zd m = Mg[(size_t)cl * DD + e];
                    Mx[e] = cmk<T, CT>((T)m.x, (T)m.y);
                }
            }
            m_cl = cl;
        }
        if (glane < D) {
            if constexpr (sizeof(T) == 8) {
                e1h[glane] = phase<T, CT>(w1[glane] * (t * fh));
                e1f[glane] = phase<T, CT>(w1[glane] * (t * ff));
                e0h[glane] = phase<T, CT>(w0[glane] * (t * fh));
                e0f[glane] = phase<T, CT>(w0[glane] * (t * ff));
            } else {
                const unsigned long long *pc = phi + (size_t)cl * 4 * D + glane;  // [br][h, f][d]
                const float2 a = phase_step_f(pc[0], i), b = phase_step_f(pc[D], i);
                const float2 c = phase_step_f(pc[2 * D], i), q = phase_step_f(pc[3 * D], i);
                e0h[glane] = cmk<T, CT>(a.x, a.y);
                e0f[glane] = cmk<T, CT>(b.x, b.y);
                e1h[glane] = cmk<T, CT>(c.x, c.y);
                e1f[glane] = cmk<T, CT>(q.x, q.y);
            }
        }
        __syncwarp();
        for (int e = glane; e < DD; e += G) {
            const int c = e / D;
            const CT m = Mx[e];
            CT a = e1h[c];
            pool[0][e] = cmk<T, CT>(m.x * a.x - m.y * a.y, m.x * a.y + m.y * a.x);
            if (two) {
                a = e1f[c];
                pool[1][e] = cmk<T, CT>(m.x * a.x - m.y * a.y, m.x * a.y + m.y * a.x);
            }
        }
        __syncwarp();
        warp_mm<D, T, CT>(pool[0], Mx, Yh, true);
        if (two) warp_mm<D, T, CT>(pool[1], Mx, Yf, true);
        CT *res[2] = {nullptr, nullptr};
        int fb1 = 1, fb2 = 2;
        for (int br = 0; br < 2; ++br) {
            CT *cur = br == 0 ? pool[0] : pool[fb1];
            CT *tmp = br == 0 ? pool[1] : pool[fb2];
            // a chain that starts with U0 is diag(dstart) until its first Y
            // factor, which then is a row scaling, not a product (a Hahn
            // echo needs one product per time point: Y)
            bool started = false;
            const CT *dstart = nullptr;
            for (int j = 0; j < nseg; ++j) {
                const bool outer = (j == 0 || j == nseg - 1);
                if (((j + br) & 1) == 0) {
                    const CT *e0 = outer ? e0h : e0f;
                    if (!started) {
                        dstart = e0;
                    } else {
                        for (int e = glane; e < DD; e += G) {
                            const CT d = e0[e / D];
                            const CT x = cur[e];
                            cur[e] = cmk<T, CT>(x.x * d.x - x.y * d.y, x.x * d.y + x.y * d.x);
                        }
                        __syncwarp();
                    }
                } else {
                    const CT *Y = (outer || !two) ? Yh : Yf;
                    if (!started) {
                        for (int e = glane; e < DD; e += G) cur[e] = Y[e];
                        __syncwarp();
                    } else if (dstart) {
                        for (int e = glane; e < DD; e += G) {
                            const CT d = dstart[e % D], y = Y[e];
                            cur[e] = cmk<T, CT>(d.x * y.x - d.y * y.y, d.x * y.y + d.y * y.x);
                        }
                        dstart = nullptr;
                        __syncwarp();
                    } else {
                        warp_mm<D, T, CT>(cur, Y, tmp, false);
                        CT *sw = cur;
                        cur = tmp;
                        tmp = sw;
                    }
                }
                started = true;
            }
            if (dstart) {  // a chain of one diagonal factor
                for (int e = glane; e < DD; e += G)
                    cur[e] = (e % D == e / D) ? dstart[e % D] : cmk<T, CT>(0, 0);
                __syncwarp();
            }
            res[br] = cur;
            if (br == 0) {
                if (cur == pool[0]) { fb1 = 1; fb2 = 2; }
                else { fb1 = 0; fb2 = 2; }
            }
        }
        // per-lane partial sums in T (FP32 mode: a few entries per lane,
        // relative error ~1e-7), the cross-lane reduction in FP64
        T tr = 0, t0 = 0, t1 = 0;
        for (int e = glane; e < DD; e += G) {
            const CT b1 = res[1][e], b0 = res[0][e];
            const T dr = b0.x - b1.x, di = b0.y - b1.y;
            tr = fma(dr, dr, fma(di, di, tr));
            t0 = fma(b0.x, b0.x, fma(b0.y, b0.y, t0));
            t1 = fma(b1.x, b1.x, fma(b1.y, b1.y, t1));
        }
        if constexpr (sizeof(T) == 4) {
            // FP32 mode: cross-lane sums and the defect in FP32, 1 - x in FP64
            for (int off = G / 2; off > 0; off >>= 1) {
                tr += __shfl_xor_sync(0xffffffffu, tr, off);
                t0 += __shfl_xor_sync(0xffffffffu, t0, off);
                t1 += __shfl_xor_sync(0xffffffffu, t1, off);
            }
            if (valid && glane == 0)
                L[(size_t)cl * nT + i] = i == 0 ? 1.0 : 1.0 - (double)coherence_defect_f(t0, t1, tr);
        } else {
            double lr = tr, l0 = t0, l1 = t1;
            for (int off = G / 2; off > 0; off >>= 1) {
                lr += __shfl_xor_sync(0xffffffffu, lr, off);
                l0 += __shfl_xor_sync(0xffffffffu, l0, off);
                l1 += __shfl_xor_sync(0xffffffffu, l1, off);
            }
            if (valid && glane == 0) L[(size_t)cl * nT + i] = i == 0 ? 1.0 : coherence_from_sums(l0, l1, lr);
        }
        __syncwarp();
    }
}

// flag clusters whose coherence drops below tau at any time point
__global__ void k_flag_low(const double *__restrict__ L, int ncl, int nT, double tau,
                           int *__restrict__ flag)
{
    const int cl = blockIdx.x;
    if (cl >= ncl) return;
    int low = 0;
    for (int i = threadIdx.x; i < nT; i += blockDim.x)
        if (!(L[(size_t)cl * nT + i] >= tau)) low = 1;
    low = __syncthreads_or(low);
    if (threadIdx.x == 0) flag[cl] = low;
}

// gather (w, M) of the listed clusters; scatter their recomputed curves back
template <int K>
__global__ void k_gather_wm(const double *__restrict__ w, const zd *__restrict__ M,
                            const int *__restrict__ list, int n, double *__restrict__ w2,
                            zd *__restrict__ M2)
{
    constexpr int D = 1 << K;
    const int q = blockIdx.x;
    if (q >= n) return;
    const int cl = list[q];
    for (int e = threadIdx.x; e < 2 * D; e += blockDim.x) w2[(size_t)q * 2 * D + e] = w[(size_t)cl * 2 * D + e];
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) M2[(size_t)q * D * D + e] = M[(size_t)cl * D * D + e];
}

__global__ void k_scatter_rows(const double *__restrict__ Lsub, const int *__restrict__ list, int n,
                               int nT, double *__restrict__ L)
{
    const int q = blockIdx.x;
    if (q >= n) return;
    for (int i = threadIdx.x; i < nT; i += blockDim.x)
        L[(size_t)list[q] * nT + i] = Lsub[(size_t)q * nT + i];
}

// M = V0^+ V1 per cluster (FP64)
// M = V0^H V1 per cluster (FP64), and its FP32 copy M32 for the FP32
// coherence kernels when M32 is not null
template <int K>
__global__ void k_overlap(const zd *__restrict__ V, int ncl, zd *__restrict__ M,
                          float2 *__restrict__ M32)
{
    constexpr int D = 1 << K;
    const int cl = blockIdx.x;
    if (cl >= ncl) return;
    const zd *V0 = V + ((size_t)cl * 2) * D * D, *V1 = V0 + D * D;
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
        const int r = e % D, c = e / D;
        zd acc = zmake(0, 0);
        for (int l = 0; l < D; ++l) {
            const zd a = V0[l + D * r], b = V1[l + D * c];
            // conj(a) * b
            acc.x = fma(a.x, b.x, acc.x);
            acc.x = fma(a.y, b.y, acc.x);
            acc.y = fma(a.x, b.y, acc.y);
            acc.y = fma(-a.y, b.x, acc.y);
        }
        M[(size_t)cl * D * D + e] = acc;
        if (M32) M32[(size_t)cl * D * D + e] = make_float2((float)acc.x, (float)acc.y);
    }
}

// ---------------------------------------------------------------------------
// Single-sample CCE (SingleSampleCCE, src/source/app/single_sample_cce.cpp):
// the bath is a pure product state, each spin up or down along z
// (prepare_bath_state, :35-46); every cluster spin feels the mean dipolar
// field of the bath spins outside the cluster (DipolarField with the cluster
// masked out, SpinInteraction.cpp:150-165; DipolarFieldInteractionCoeff,
// SpinInteractionComponent.cpp:433-451; dipole_field, misc.cpp:50-57), and
// L(t) = Re <psi_1(t) | psi_2(t)> with psi_a the cluster's basis state
// propagated through riffle(H_a, H_{1-a}) (:48-127).
// ---------------------------------------------------------------------------

// xfield[cl][i][a] = sum_{j not in cluster} T_ij[a][z] m_j, m_j = +1/2 (state
// 0) or -1/2 (state 1): one CTA per cluster, threads over bath spins.
template <int K>
__global__ void __launch_bounds__(256)
k_bath_field(const double *__restrict__ coords, int nbath, const unsigned char *__restrict__ state,
             const unsigned *__restrict__ clusters, int ncl, double gb, double *__restrict__ xfield)
{
    __shared__ double red[8][3 * MAX_K];
    const int cl = blockIdx.x;
    if (cl >= ncl) return;
    const unsigned *idx = clusters + (size_t)cl * K;
    double acc[3 * K];
#pragma unroll
    for (int q = 0; q < 3 * K; ++q) acc[q] = 0.0;
    for (int j = threadIdx.x; j < nbath; j += blockDim.x) {
        bool in = false;
#pragma unroll
        for (int s = 0; s < K; ++s) in |= idx[s] == (unsigned)j;
        if (in) continue;
        const double m = state[j] ? -0.5 : 0.5;
#pragma unroll
        for (int s = 0; s < K; ++s) {
            double t9[9];
            dipole_tensor(coords + 3 * idx[s], coords + 3 * (size_t)j, gb, gb, t9);
#pragma unroll
            for (int a = 0; a < 3; ++a) acc[3 * s + a] += t9[6 + a] * m;  // T[a][z] (symmetric)
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < 3 * K; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3 * K) {
        double v = 0.0;
        for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) v += red[w8][threadIdx.x];
        xfield[(size_t)cl * 3 * K + threadIdx.x] = v;
    }
}

// L(t_i) = Re <psi_1 | psi_2> (normalised) in the eigenbasis of H_0: the initial state is
// x0 = V0^H e_b (b = the cluster spins' basis state, spin 0 the most
// significant bit); an H_0 segment multiplies by e^{-i w0 tau}, an H_1
// segment by M diag(e^{-i w1 tau}) M^H.  One warp per time point, M and M^H
// of the CTA's cluster in shared memory.  T = double: FP64 throughout; T =
// float: FP32 products and fixed-point phase steps (mixed mode).
template <int K, typename T>
constexpr size_t state_kernel_smem()
{
    constexpr int D = 1 << K;
    return (size_t)(2 * D * D + D + 8 * 2 * D) * sizeof(typename cplx<T>::t) + 2 * D * sizeof(double);
}

template <int K, typename T>
__global__ void __launch_bounds__(256)
k_state_coherence(const double *__restrict__ w, const unsigned long long *__restrict__ phi,
                  const zd *__restrict__ Mg, const float2 *__restrict__ Mg32, const zd *__restrict__ V,
                  const unsigned *__restrict__ clusters, const unsigned char *__restrict__ state,
                  int ncl, int pulse_num, int nT, double dt, double fh, double ff,
                  double *__restrict__ L)
{
    typedef typename cplx<T>::t CT;
    constexpr int D = 1 << K, DD = D * D, R = (D + 31) / 32;
    extern __shared__ unsigned char sraw[];
    double *wsh = reinterpret_cast<double *>(sraw);   // w0[D], w1[D]
    CT *Ms = reinterpret_cast<CT *>(wsh + 2 * D);      // M (column-major)
    CT *Mh = Ms + DD;                                  // M^H
    CT *x0 = Mh + DD;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    CT *buf = x0 + D + warp * 2 * D;
    for (int cl = blockIdx.x; cl < ncl; cl += gridDim.x) {
        __syncthreads();
        for (int e = threadIdx.x; e < DD; e += blockDim.x) {
            CT m;
            if constexpr (sizeof(T) == 8) m = Mg[(size_t)cl * DD + e];
            else m = Mg32[(size_t)cl * DD + e];
            const int r = e % D, c = e / D;
            Ms[e] = m;
            Mh[c + D * r] = cmk<T, CT>(m.x, -m.y);
        }
        int b = 0;
        for (int s = 0; s < K; ++s) b |= (state[clusters[(size_t)cl * K + s]] ? 1 : 0) << (K - 1 - s);
        const zd *V0 = V + (size_t)cl * 2 * DD;
        for (int m = threadIdx.x; m < D; m += blockDim.x) {
            const zd v = V0[b + D * m];
            x0[m] = cmk<T, CT>((T)v.x, (T)-v.y);
            wsh[m] = w[(size_t)cl * 2 * D + m];
            wsh[D + m] = w[(size_t)cl * 2 * D + D + m];
        }
        __syncthreads();
        for (int i = warp; i < nT; i += nw) {
            // phase factors of this time point: [br][f][q]
            CT ph[2][2][R];
#pragma unroll
            for (int br = 0; br < 2; ++br)
#pragma unroll
                for (int f = 0; f < 2; ++f)
#pragma unroll
                    for (int q = 0; q < R; ++q) {
                        const int m = lane + 32 * q;
                        if (m >= D) {
                            ph[br][f][q] = cmk<T, CT>(1, 0);
                        } else if constexpr (sizeof(T) == 8) {
                            double sn, cs;
                            sincos(wsh[br * D + m] * ((f ? ff : fh) * dt * (double)i), &sn, &cs);
                            ph[br][f][q] = cmk<T, CT>(cs, -sn);
                        } else {
                            ph[br][f][q] = phase_step_f(phi[(((size_t)cl * 2 + br) * 2 + f) * D + m], i);
                        }
                    }
            CT fin[2][R];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                CT xr[R];
#pragma unroll
                for (int q = 0; q < R; ++q) {
                    const int m = lane + 32 * q;
                    xr[q] = m < D ? x0[m] : cmk<T, CT>(0, 0);
                }
                for (int j = 0; j <= pulse_num; ++j) {
                    const int hsel = (j + a) & 1, f = (j == 0 || j == pulse_num) ? 0 : 1;
                    if (hsel == 0) {
#pragma unroll
                        for (int q = 0; q < R; ++q) {
                            const CT p = ph[0][f][q], x = xr[q];
                            xr[q] = cmk<T, CT>(x.x * p.x - x.y * p.y, x.x * p.y + x.y * p.x);
                        }
                        continue;
                    }
                    CT *xs = buf + a * D;
#pragma unroll
                    for (int q = 0; q < R; ++q)
                        if (lane + 32 * q < D) xs[lane + 32 * q] = xr[q];
                    __syncwarp();
                    CT yr[R];
#pragma unroll
                    for (int q = 0; q < R; ++q) {
                        const int m = lane + 32 * q;
                        T ar = 0, ai = 0;
                        if (m < D)
                            for (int c = 0; c < D; ++c) {
                                const CT g = Mh[m + D * c], x = xs[c];
                                ar = fma(g.x, x.x, ar);
                                ar = fma(-g.y, x.y, ar);
                                ai = fma(g.x, x.y, ai);
                                ai = fma(g.y, x.x, ai);
                            }
                        const CT p = ph[1][f][q];
                        yr[q] = cmk<T, CT>(ar * p.x - ai * p.y, ar * p.y + ai * p.x);
                    }
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < R; ++q)
                        if (lane + 32 * q < D) xs[lane + 32 * q] = yr[q];
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < R; ++q) {
                        const int m = lane + 32 * q;
                        T ar = 0, ai = 0;
                        if (m < D)
                            for (int c = 0; c < D; ++c) {
                                const CT g = Ms[m + D * c], x = xs[c];
                                ar = fma(g.x, x.x, ar);
                                ar = fma(-g.y, x.y, ar);
                                ai = fma(g.x, x.y, ai);
                                ai = fma(g.y, x.x, ai);
                            }
                        xr[q] = cmk<T, CT>(ar, ai);
                    }
                    __syncwarp();
                }
#pragma unroll
                for (int q = 0; q < R; ++q) fin[a][q] = xr[q];
            }
            // normalised difference form (as the trace kernels): n0 = |x1|^2,
            // n1 = |x2|^2, d = |x1 - x2|^2 cancel the norm drift of reduced-
            // precision chains (an FP32 M is unitary only to ~1e-7 and is
            // applied up to 2n times)
            T n0 = 0, n1 = 0, dd = 0;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const CT u = fin[0][q], v = fin[1][q];
                n0 += u.x * u.x + u.y * u.y;
                n1 += v.x * v.x + v.y * v.y;
                dd += (u.x - v.x) * (u.x - v.x) + (u.y - v.y) * (u.y - v.y);
            }
            for (int o = 16; o > 0; o >>= 1) {
                n0 += __shfl_xor_sync(0xffffffffu, n0, o);
                n1 += __shfl_xor_sync(0xffffffffu, n1, o);
                dd += __shfl_xor_sync(0xffffffffu, dd, o);
            }
            if (lane == 0) {
                if constexpr (sizeof(T) == 4) L[(size_t)cl * nT + i] = 1.0 - (double)coherence_defect_f(n0, n1, dd);
                else L[(size_t)cl * nT + i] = coherence_from_sums(n0, n1, dd);
            }
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Opt-in kernel timing (CUDA events on the launching stream around the
// per-time-point coherence kernel), read by bench.py for the roofline.  The
// events are only recorded during a run; they are resolved (waited for and
// destroyed) when the counters are read, so timing adds no host
// synchronisation to the runs it measures.
typedef oops_prof_event ProfPending;
static std::mutex g_prof_mu;
static int g_prof_on = 0;
// index k: coherence kernel of size class k; index 8 + k: its eigensolver
// phase (assembly, diagonalisation, overlaps, phase steps)
static double g_prof_ms[16] = {0};
static long g_prof_n[16] = {0};
static double g_prof_flop[16] = {0};
static long g_prof_corr[8] = {0};
static std::vector<ProfPending> g_prof_pending;
static thread_local std::vector<oops_prof_event> *t_prof_sink = nullptr;

bool oops_prof_enabled() { return g_prof_on != 0; }
void oops_prof_set_sink(std::vector<oops_prof_event> *sink) { t_prof_sink = sink; }
void oops_prof_accumulate(const oops_prof_event &e, float ms)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (e.k < 0 || e.k >= 16) return;
    g_prof_ms[e.k] += ms;
    g_prof_n[e.k] += 1;
    g_prof_flop[e.k] += e.flop;
}

// a timing event on st; while st is being captured into a graph, an external
// record node, which every replay of the graph records
static void prof_record(cudaEvent_t ev, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    else
        cudaEventRecord(ev, st);
}

static void prof_push(cudaEvent_t ev0, cudaEvent_t ev1, int k, double flop)
{
    if (t_prof_sink) {
        t_prof_sink->push_back({ev0, ev1, k, flop});
        return;
    }
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_pending.push_back({ev0, ev1, k, flop});
}

static void prof_resolve(bool keep)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (const ProfPending &p : g_prof_pending) {
        float ms = 0;
        if (keep && cudaEventSynchronize(p.ev1) == cudaSuccess &&
            cudaEventElapsedTime(&ms, p.ev0, p.ev1) == cudaSuccess) {
            g_prof_ms[p.k] += ms;
            g_prof_n[p.k] += 1;
            g_prof_flop[p.k] += p.flop;
        }
        cudaEventDestroy(p.ev0);
        cudaEventDestroy(p.ev1);
    }
    g_prof_pending.clear();
}

extern "C" int oops_profile_enable(int on)
{
    prof_resolve(false);
    g_prof_on = on;
    oops_prof_reset_liouville();
    for (int q = 0; q < 16; ++q) {
        g_prof_ms[q] = 0;
        g_prof_n[q] = 0;
        g_prof_flop[q] = 0;
        if (q < 8) g_prof_corr[q] = 0;
    }
    return OOPS_OK;
}
extern "C" int oops_profile_corrected(int k, long *count)
{
    if (k < 0 || k >= 8 || !count) return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    *count = g_prof_corr[k];
    return OOPS_OK;
}
extern "C" int oops_profile_read(int k, double *ms_total, long *launches, double *flop)
{
    if (k < 0 || k >= 8 || !ms_total || !launches || !flop) return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    prof_resolve(true);
    *ms_total = g_prof_ms[k];
    *launches = g_prof_n[k];
    *flop = g_prof_flop[k];
    return OOPS_OK;
}
extern "C" int oops_profile_read_eig(int k, double *ms_total, long *launches)
{
    if (k < 0 || k >= 8 || !ms_total || !launches) return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    prof_resolve(true);
    *ms_total = g_prof_ms[8 + k];
    *launches = g_prof_n[8 + k];
    return OOPS_OK;
}

// complex D x D products per time point of the SIMT coherence kernels (Y
// factors built, then chain products; a chain's first Y after a diagonal
// start is a row scaling), times 8 D^3 real flops each
static double coherence_flop(int D, int pulse_num, int nT, int ncl)
{
    const int nseg = pulse_num + 1;
    double fh = 0.5 / pulse_num, ff = pulse_num > 1 ? 1.0 / pulse_num : fh;
    int gem = (fh != ff) ? 2 : 1;
    for (int br = 0; br < 2; ++br) {
        bool started = false, diag = false;
        for (int j = 0; j < nseg; ++j) {
            const bool u1 = ((j + br) & 1) == 1;
            if (!started) diag = !u1;
            else if (u1 && diag) diag = false;  // row scaling, not a product
            else if (u1) gem++;
            started = true;
        }
    }
    return (double)gem * 8.0 * D * D * D * (double)(nT - 1) * ncl;
}

namespace {

// Recompute in FP64 the clusters whose mixed-precision coherence falls below
// tau at some time point (their L_C enters the CCE reduction as a divisor, so
// their absolute rounding error becomes a large relative error).
// The last Jacobi phase of k_assemble_eig: FP64 mode (rel_gap 0) runs it in
// FP64 and rotates every pair above the absolute threshold (eigenvectors to
// FP64 rounding, which the 1e-10 per-cluster parity needs).  The mixed modes
// keep the overlaps M in FP32 (rounding 6e-8), so they run it with an FP32
// off-diagonal (jacobi_refine32) and leave a pair alone once its rotation
// would move the eigenvectors by less than 2^-30 (and the eigenvalues by
// less than 2^-30 |a_pq|).  A mixed run with an FP64 correction threshold
// (tau > 0) recomputes clusters in FP64 from the same eigenbasis, so it
// takes the FP64 phase.
static double eig_rel_gap(int precision, double tau = 0.0)
{
    return precision == OOPS_PREC_FP64 || tau > 0.0 ? 0.0 : 0x1p-30;
}

// ---------------------------------------------------------------------------
// Launch tuning (oops_tune_*): per device and cluster size, the CTAs per SM
// of the eigensolver and of the block coherence kernels, and the time-slice
// multiplier that splits a class's time grid when it has few clusters.  Zero
// means the built-in default; the autotuner (oops_gb300/tune.py) measures
// candidates and sets the winners from its on-disk cache.
// ---------------------------------------------------------------------------
static int g_tune[64][OOPS_TUNE_NPARAM][8] = {};

static int tune_value(int param, int k, int def)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return def;
    }
    const int v = g_tune[dev][param][k & 7];
    return v > 0 ? v : def;
}
static int tune_eig_per_sm(int K)
{
    const int D = 1 << K;
    return tune_value(OOPS_TUNE_EIG_PER_SM, K, D >= 64 ? 1 : (D >= 32 ? 4 : 8));
}
static int tune_coh_per_sm(int K, bool fp64)
{
    const int D = 1 << K;
    return tune_value(OOPS_TUNE_COH_PER_SM, K, fp64 ? (D >= 32 ? 1 : 4) : (D >= 64 ? 1 : (D >= 32 ? 2 : 4)));
}
static int tune_tslice_mult(int K, int def) { return tune_value(OOPS_TUNE_TSLICE_MULT, K, def); }

}  // namespace

extern "C" int oops_tune_set(int param, int k, int value)
{
    if (param < 0 || param >= OOPS_TUNE_NPARAM || k < 1 || k > MAX_K || value < 0 || value > 64)
        return oops_set_status(OOPS_ERR_ARG, "oops_tune_set: parameter 0..2, k 1..6, value 0..64");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return oops_set_status(OOPS_ERR_CUDA, "oops_tune_set: no current CUDA device");
    }
    g_tune[dev][param][k] = value;
    return OOPS_OK;
}

extern "C" int oops_tune_get(int param, int k, int *value)
{
    if (param < 0 || param >= OOPS_TUNE_NPARAM || k < 1 || k > MAX_K || !value)
        return oops_set_status(OOPS_ERR_ARG, "oops_tune_get: parameter 0..2, k 1..6");
    switch (param) {
        case OOPS_TUNE_EIG_PER_SM: *value = tune_eig_per_sm(k); break;
        case OOPS_TUNE_COH_PER_SM: *value = tune_coh_per_sm(k, false); break;
        default: *value = tune_tslice_mult(k, k >= 5 ? 2 : 4); break;  // k >= 5: the tensor-core kernels' default
    }
    return OOPS_OK;
}

namespace {

// One wave of the warp coherence kernel: as many CTAs as fit on the GPU at
// once (each warp then takes a contiguous run of items), never more than the
// items need
template <typename F>
static int warp_grid(F *kernel, int threads, size_t smem, long long items, int ipc, int sms)
{
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess || occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    return (int)std::max<long long>(1, std::min<long long>((items + ipc - 1) / ipc, (long long)sms * occ));
}

// CPMG interval fractions of the outer (half) and inner (full) segments, by
// the same arithmetic as the kernels' frac_s table (Pulse_Interval,
// misc.cpp:59-84)
static void interval_fractions(int pulse_num, double *fh, double *ff)
{
    double prev = 0.0, f0 = 0.0, f1 = 0.0;
    for (int i = 0; i < pulse_num; ++i) {
        const double tt = (2.0 * i + 1.0) / (2.0 * pulse_num);
        if (i == 0) f0 = tt - prev;
        if (i == 1) f1 = tt - prev;
        prev = tt;
    }
    *fh = f0;
    *ff = pulse_num > 1 ? f1 : f0;
}

template <int K>
void launch_phase_steps(const double *w, int ncl, int pulse_num, double dt, unsigned long long *phi,
                        cudaStream_t st)
{
    constexpr int D = 1 << K;
    double fh, ff;
    interval_fractions(pulse_num, &fh, &ff);
    const size_t n = (size_t)ncl * 4 * D;
    k_phase_steps<K><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(w, ncl, dt, fh, ff, phi);
}

template <int K>
int correct_fp64(const double *w, const zd *M, int ncl, int pulse_num, int nT, double dt,
                 double tau, double *L, cudaStream_t st, long *ncorr)
{
    constexpr int D = 1 << K;
    const int sms = oops_sm_count();
    *ncorr = 0;
    int *flag = nullptr;
    if (cudaMallocAsync((void **)&flag, (size_t)ncl * sizeof(int), st) != cudaSuccess) {
        cudaGetLastError();
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (FP64 correction flags)");
    }
    k_flag_low<<<ncl, 128, 0, st>>>(L, ncl, nT, tau, flag);
    std::vector<int> hf(ncl);
    cudaMemcpyAsync(hf.data(), flag, (size_t)ncl * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(flag, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    std::vector<int> list;
    for (int c = 0; c < ncl; ++c)
        if (hf[c]) list.push_back(c);
    const int n = (int)list.size();
    *ncorr = n;
    if (n == 0) return OOPS_OK;
    int *dlist = nullptr, *q = nullptr;
    double *w2 = nullptr, *Lsub = nullptr;
    zd *M2 = nullptr;
    void *gws = nullptr;
    const int tslices = std::max(1, std::min(nT, (sms * 4 + n - 1) / n));
    size_t smem = (size_t)6 * D * D * sizeof(double2);
    const int use_smem = smem <= 200 * 1024;
    const int grid = std::max(1, std::min(n * tslices, sms * (D >= 32 ? 1 : 4)));
    if (cudaMallocAsync((void **)&dlist, (size_t)n * sizeof(int), st) != cudaSuccess ||
        cudaMallocAsync((void **)&q, 4 * sizeof(int), st) != cudaSuccess ||
        cudaMallocAsync((void **)&w2, (size_t)n * 2 * D * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&M2, (size_t)n * D * D * sizeof(zd), st) != cudaSuccess ||
        cudaMallocAsync((void **)&Lsub, (size_t)n * nT * sizeof(double), st) != cudaSuccess ||
        (!use_smem && cudaMallocAsync(&gws, (size_t)grid * smem, st) != cudaSuccess)) {
        cudaGetLastError();
        if (dlist) cudaFreeAsync(dlist, st);
        if (q) cudaFreeAsync(q, st);
        if (w2) cudaFreeAsync(w2, st);
        if (M2) cudaFreeAsync(M2, st);
        if (Lsub) cudaFreeAsync(Lsub, st);
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (FP64 correction)");
    }
    cudaMemcpyAsync(dlist, list.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(q, 0, 4 * sizeof(int), st);
    k_gather_wm<K><<<n, 128, 0, st>>>(w, M, dlist, n, w2, M2);
    if constexpr (K <= 4) {
        constexpr int W = warp_kernel_warps<K, double>();
        constexpr size_t sm = warp_kernel_smem<K, double>();
        cudaFuncSetAttribute(k_coherence_warp<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        const long long items = (long long)n * nT;
        constexpr int IPC = W * (32 / warp_group<K>());   // items per CTA pass
        int g = warp_grid(k_coherence_warp<K, double>, W * 32, sm, items, IPC, sms);
        k_coherence_warp<K, double><<<g, W * 32, sm, st>>>(w2, nullptr, M2, nullptr, n, pulse_num, nT, dt, Lsub);
    } else {
        if (!use_smem) smem = 0;
        cudaFuncSetAttribute(k_coherence<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_coherence<K, double><<<grid, 256, smem, st>>>(w2, nullptr, M2, nullptr, n, pulse_num, nT, dt, tslices, Lsub, q,
                                                        (double2 *)gws, use_smem);
    }
    k_scatter_rows<<<n, 128, 0, st>>>(Lsub, dlist, n, nT, L);
    cudaFreeAsync(dlist, st);
    cudaFreeAsync(q, st);
    cudaFreeAsync(w2, st);
    cudaFreeAsync(M2, st);
    cudaFreeAsync(Lsub, st);
    if (gws) cudaFreeAsync(gws, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    return OOPS_OK;
}

// ext_ctr: null -> the call allocates its counters, waits for the stream and
// checks the error flags before returning.  Non-null (8 zeroed device ints the
// caller owns) -> the call only enqueues work (unless the FP64 correction
// needs the host), and the caller checks ext_ctr[3] (eigensolver
// failure) and ext_ctr[5] (tensor-core status) after its own synchronisation.
template <int K>
int run_class(const double *coords, const unsigned *clusters, int ncl, const PhysParams &pp,
              int pulse_num, int nT, double dt, int precision, double tau, double *L,
              cudaStream_t st, int *ext_ctr)
{
    constexpr int D = 1 << K;
    const int sms = oops_sm_count();
    double *w = nullptr;
    zd *V = nullptr, *M = nullptr;
    unsigned long long *phi = nullptr;
    float2 *M32 = nullptr;
    int *ctr = nullptr;
    void *gws = nullptr;
    int rc = OOPS_OK;
    const bool fp32 = precision != OOPS_PREC_FP64;
    // stream-ordered allocations: no device-wide synchronisation, so batches
    // on different streams overlap
    auto cleanup = [&]() {
        if (w) cudaFreeAsync(w, st);
        if (V) cudaFreeAsync(V, st);
        if (M) cudaFreeAsync(M, st);
        if (phi) cudaFreeAsync(phi, st);
        if (M32) cudaFreeAsync(M32, st);
        if (ctr && !ext_ctr) cudaFreeAsync(ctr, st);
        if (gws) cudaFreeAsync(gws, st);
    };
    if (ext_ctr) ctr = ext_ctr;
    if (cudaMallocAsync((void **)&w, (size_t)ncl * 2 * D * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&V, (size_t)ncl * 2 * D * D * sizeof(zd), st) != cudaSuccess ||
        cudaMallocAsync((void **)&M, (size_t)ncl * D * D * sizeof(zd), st) != cudaSuccess ||
        (fp32 && cudaMallocAsync((void **)&phi, (size_t)ncl * 4 * D * sizeof(unsigned long long), st) != cudaSuccess) ||
        (fp32 && cudaMallocAsync((void **)&M32, (size_t)ncl * D * D * sizeof(float2), st) != cudaSuccess) ||
        (!ext_ctr && cudaMallocAsync((void **)&ctr, 8 * sizeof(int), st) != cudaSuccess)) {
        cudaGetLastError();
        cleanup();
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (cluster workspace)");
    }
    if (!ext_ctr) cudaMemsetAsync(ctr, 0, 8 * sizeof(int), st);
    cudaEvent_t eg0 = nullptr, eg1 = nullptr;
    if (g_prof_on) {
        cudaEventCreate(&eg0);
        cudaEventCreate(&eg1);
        prof_record(eg0, st);
    }
    // 1. assemble + diagonalise (work queue over 2*ncl items)
    {
        size_t smem = (size_t)3 * D * D * sizeof(zd);
        cudaFuncSetAttribute(k_assemble_eig<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = tune_eig_per_sm(K);
        int grid = std::max(1, std::min(2 * ncl, sms * per_sm));
        k_assemble_eig<K><<<grid, EIG_THREADS<K>, smem, st>>>(coords, clusters, ncl, pp, nullptr, w, V, ctr + 0, ctr + 3,
                                                    eig_rel_gap(precision, tau));
    }
    k_overlap<K><<<ncl, 256, 0, st>>>(V, ncl, M, M32);
    if (fp32) launch_phase_steps<K>(w, ncl, pulse_num, dt, phi, st);
    if (g_prof_on) {
        prof_record(eg1, st);
        prof_push(eg0, eg1, 8 + K, 0.0);
    }
    // 2. per time point coherence
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (g_prof_on) {
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
        prof_record(ev0, st);
    }
    const int tslices = std::max(1, std::min(nT, (sms * tune_tslice_mult(K, 4) + ncl - 1) / std::max(1, ncl)));
    bool done_small = false;
    if constexpr (K <= 4) {
        const long long items = (long long)ncl * nT;
        if (precision == OOPS_PREC_FP64) {
            constexpr int W = warp_kernel_warps<K, double>();
            constexpr size_t sm = warp_kernel_smem<K, double>();
            cudaFuncSetAttribute(k_coherence_warp<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            constexpr int IPC = W * (32 / warp_group<K>());   // items per CTA pass
            int grid = warp_grid(k_coherence_warp<K, double>, W * 32, sm, items, IPC, sms);
            k_coherence_warp<K, double><<<grid, W * 32, sm, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, L);
        } else {
            constexpr int W = warp_kernel_warps<K, float>();
            constexpr size_t sm = warp_kernel_smem<K, float>();
            cudaFuncSetAttribute(k_coherence_warp<K, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            constexpr int IPC = W * (32 / warp_group<K>());   // items per CTA pass
            int grid = warp_grid(k_coherence_warp<K, float>, W * 32, sm, items, IPC, sms);
            k_coherence_warp<K, float><<<grid, W * 32, sm, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, L);
        }
        done_small = true;
    }
    const bool use_tc = K >= 5 && precision == OOPS_PREC_MIXED && oops_tc64_supported(pulse_num);
    if (done_small) {
    } else if (use_tc) {
        rc = K == 6 ? oops_coherence_tc64(phi, M32, ncl, pulse_num, nT, L, ctr + 4, ctr + 5, tune_tslice_mult(K, 2), st)
                    : oops_coherence_tc32(phi, M32, ncl, pulse_num, nT, L, ctr + 4, ctr + 5, tune_tslice_mult(K, 2), st);
        if (rc) {
            cleanup();
            return rc;
        }
    } else if (precision == OOPS_PREC_FP64) {
        size_t smem = (size_t)6 * D * D * sizeof(double2);
        int use_smem = smem <= 200 * 1024;
        int grid = std::max(1, std::min(ncl * tslices, sms * tune_coh_per_sm(K, true)));
        if (!use_smem) {
            if (cudaMallocAsync(&gws, (size_t)grid * smem, st) != cudaSuccess) {
                cudaGetLastError();
                cleanup();
                return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (FP64 workspace)");
            }
            smem = 0;
        }
        cudaFuncSetAttribute(k_coherence<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_coherence<K, double><<<grid, 256, smem, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, tslices, L,
                                                        ctr + 1, (double2 *)gws, use_smem);
    } else {
        size_t smem = (size_t)6 * D * D * sizeof(float2);
        int grid = std::max(1, std::min(ncl * tslices, sms * tune_coh_per_sm(K, false)));
        cudaFuncSetAttribute(k_coherence<K, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_coherence<K, float><<<grid, 256, smem, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, tslices, L,
                                                       ctr + 2, nullptr, 1);
    }
    if (g_prof_on) prof_record(ev1, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    if (!rc && tau > 0.0 && precision != OOPS_PREC_FP64) {
        long ncorr = 0;
        rc = correct_fp64<K>(w, M, ncl, pulse_num, nT, dt, tau, L, st, &ncorr);
        g_prof_corr[K] += ncorr;
    }
    if (!rc && !ext_ctr) {
        int flags[8] = {0};
        cudaMemcpyAsync(flags, ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
        else if (flags[3]) rc = oops_set_status(OOPS_ERR_NUMERIC, "Jacobi eigensolver did not converge");
        else if (flags[5]) rc = oops_set_status(flags[5], "tensor-core coherence kernel failed (bounded wait expired)");
    }
    if (g_prof_on) {
        if (!rc) prof_push(ev0, ev1, K, coherence_flop(D, pulse_num, nT, ncl));
        else {
            cudaEventDestroy(ev0);
            cudaEventDestroy(ev1);
        }
    }
    cleanup();
    return rc;
}

// Single-sample coherence of one size class (see k_state_coherence).
// ext_ctr as run_class: null -> wait for the stream and check the flags;
// non-null (8 zeroed device ints) -> enqueue only, the caller checks
// ext_ctr[3] after synchronising.
template <int K>
int run_class_state(const double *coords, int nbath, const unsigned char *state,
                    const unsigned *clusters, int ncl, const PhysParams &pp, int pulse_num, int nT,
                    double dt, int precision, double *L, cudaStream_t st, int *ext_ctr)
{
    constexpr int D = 1 << K;
    const int sms = oops_sm_count();
    const bool fp32 = precision != OOPS_PREC_FP64;
    double *w = nullptr, *xf = nullptr;
    zd *V = nullptr, *M = nullptr;
    unsigned long long *phi = nullptr;
    float2 *M32 = nullptr;
    int *ctr = nullptr;
    auto cleanup = [&]() {
        if (w) cudaFreeAsync(w, st);
        if (xf) cudaFreeAsync(xf, st);
        if (V) cudaFreeAsync(V, st);
        if (M) cudaFreeAsync(M, st);
        if (phi) cudaFreeAsync(phi, st);
        if (M32) cudaFreeAsync(M32, st);
        if (ctr && !ext_ctr) cudaFreeAsync(ctr, st);
    };
    if (ext_ctr) ctr = ext_ctr;
    if (cudaMallocAsync((void **)&w, (size_t)ncl * 2 * D * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&xf, (size_t)ncl * 3 * K * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void **)&V, (size_t)ncl * 2 * D * D * sizeof(zd), st) != cudaSuccess ||
        cudaMallocAsync((void **)&M, (size_t)ncl * D * D * sizeof(zd), st) != cudaSuccess ||
        (fp32 && cudaMallocAsync((void **)&phi, (size_t)ncl * 4 * D * sizeof(unsigned long long), st) != cudaSuccess) ||
        (fp32 && cudaMallocAsync((void **)&M32, (size_t)ncl * D * D * sizeof(float2), st) != cudaSuccess) ||
        (!ext_ctr && cudaMallocAsync((void **)&ctr, 8 * sizeof(int), st) != cudaSuccess)) {
        cudaGetLastError();
        cleanup();
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (single-sample workspace)");
    }
    if (!ext_ctr) cudaMemsetAsync(ctr, 0, 8 * sizeof(int), st);
    k_bath_field<K><<<ncl, 256, 0, st>>>(coords, nbath, state, clusters, ncl, pp.gb, xf);
    {
        size_t smem = (size_t)3 * D * D * sizeof(zd);
        cudaFuncSetAttribute(k_assemble_eig<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = tune_eig_per_sm(K);
        int grid = std::max(1, std::min(2 * ncl, sms * per_sm));
        k_assemble_eig<K><<<grid, EIG_THREADS<K>, smem, st>>>(coords, clusters, ncl, pp, xf, w, V, ctr + 0, ctr + 3,
                                                    eig_rel_gap(precision));
    }
    k_overlap<K><<<ncl, 256, 0, st>>>(V, ncl, M, M32);
    if (fp32) launch_phase_steps<K>(w, ncl, pulse_num, dt, phi, st);
    double fh, ff;
    interval_fractions(pulse_num, &fh, &ff);
    auto launch = [&](auto kern, size_t smem) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int bps = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 256, smem);
        const int grid = std::max(1, std::min(ncl, sms * std::max(1, bps)));
        kern<<<grid, 256, smem, st>>>(w, phi, M, M32, V, clusters, state, ncl, pulse_num, nT, dt, fh, ff, L);
    };
    if (fp32) launch(k_state_coherence<K, float>, state_kernel_smem<K, float>());
    else launch(k_state_coherence<K, double>, state_kernel_smem<K, double>());
    if (ext_ctr) {
        cleanup();
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? OOPS_OK : oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    }
    int flags[8] = {0};
    cudaMemcpyAsync(flags, ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, st);
    cleanup();
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    if (flags[3]) return oops_set_status(OOPS_ERR_NUMERIC, "Jacobi eigensolver did not converge");
    return OOPS_OK;
}

}  // namespace

extern "C" int oops_cce_coherence_state(const double *coords_dev, size_t nbath,
                                        const unsigned char *state_dev, const unsigned *clusters_dev,
                                        size_t ncl, int k, const oops_cce_params *p, int precision,
                                        double *L_dev, void *stream)
{
    return oops_cce_coherence_state_enqueue(coords_dev, nbath, state_dev, clusters_dev, ncl, k, p,
                                            precision, L_dev, stream, nullptr);
}

int oops_cce_coherence_state_enqueue(const double *coords_dev, size_t nbath,
                                     const unsigned char *state_dev, const unsigned *clusters_dev,
                                     size_t ncl, int k, const oops_cce_params *p, int precision,
                                     double *L_dev, void *stream, int *ext_ctr)
{
    if (!coords_dev || !state_dev || !clusters_dev || !p || !L_dev)
        return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (k < 1 || k > MAX_K) return oops_set_status(OOPS_ERR_SIZE, "cluster size must be 1..6 (dense path)");
    if (p->pulse_num < 1 || p->pulse_num > 64) return oops_set_status(OOPS_ERR_SIZE, "pulse_num must be 1..64");
    if (p->nT < 1 || p->nT > (1u << 24)) return oops_set_status(OOPS_ERR_SIZE, "nT out of range");
    if (nbath < (size_t)k || nbath > (1u << 30)) return oops_set_status(OOPS_ERR_SIZE, "nbath out of range");
    if (precision != OOPS_PREC_FP64 && precision != OOPS_PREC_MIXED && precision != OOPS_PREC_MIXED_SIMT)
        return oops_set_status(OOPS_ERR_ARG, "unknown precision");
    if (ncl == 0) return OOPS_OK;
    if (ncl > (1u << 30)) return oops_set_status(OOPS_ERR_SIZE, "too many clusters");
    const PhysParams pp = phys_params(p);
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)ncl, nT = (int)p->nT, nb = (int)nbath;
    switch (k) {
        case 1: return run_class_state<1>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
        case 2: return run_class_state<2>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
        case 3: return run_class_state<3>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
        case 4: return run_class_state<4>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
        case 5: return run_class_state<5>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
        default: return run_class_state<6>(coords_dev, nb, state_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st, ext_ctr);
    }
}

extern "C" int oops_cce_coherence(const double *coords_dev, size_t nbath,
                                  const unsigned *clusters_dev, size_t ncl, int k,
                                  const oops_cce_params *p, int precision, double *L_dev,
                                  void *stream)
{
    return oops_cce_coherence_enqueue(coords_dev, nbath, clusters_dev, ncl, k, p, precision,
                                      L_dev, stream, nullptr);
}

int oops_cce_coherence_enqueue(const double *coords_dev, size_t nbath,
                               const unsigned *clusters_dev, size_t ncl, int k,
                               const oops_cce_params *p, int precision, double *L_dev,
                               void *stream, int *ext_ctr)
{
    if (!coords_dev || !clusters_dev || !p || !L_dev) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (k < 1 || k > MAX_K) return oops_set_status(OOPS_ERR_SIZE, "cluster size must be 1..6 (dense path)");
    if (p->pulse_num < 1 || p->pulse_num > 64) return oops_set_status(OOPS_ERR_SIZE, "pulse_num must be 1..64");
    if (p->nT < 1 || p->nT > (1u << 24)) return oops_set_status(OOPS_ERR_SIZE, "nT out of range");
    if (precision != OOPS_PREC_FP64 && precision != OOPS_PREC_MIXED &&
        precision != OOPS_PREC_MIXED_SIMT)
        return oops_set_status(OOPS_ERR_ARG, "unknown precision");
    if (ncl == 0) return OOPS_OK;
    if (ncl > (1u << 30)) return oops_set_status(OOPS_ERR_SIZE, "too many clusters");
    (void)nbath;
    const PhysParams pp = phys_params(p);
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)ncl, nT = (int)p->nT;
    if (precision != OOPS_PREC_FP64 && k <= p->fp64_max_k) precision = OOPS_PREC_FP64;
    switch (k) {
        case 1: return run_class<1>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
        case 2: return run_class<2>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
        case 3: return run_class<3>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
        case 4: return run_class<4>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
        case 5: return run_class<5>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
        default: return run_class<6>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, p->fp64_below, L_dev, st, ext_ctr);
    }
}

// ---------------------------------------------------------------------------
// oops_cce_coherence_noalloc: the same computation with no device allocation.
//
// Some callers cannot allocate device memory during a run: a host application
// whose own allocator reserved the device memory up front (fixed memory
// budgets, pools owned by an MPI or Fortran host code), or a serving loop that
// must not let cudaMalloc/cudaFree synchronise the device between requests.
// This entry point takes its scratch (eigenvalues, eigenvectors, overlaps and
// work-queue counters) from one file-scope device array of
// OOPS_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds
// until the process exits.  Requests whose scratch would not fit are rejected
// with OOPS_ERR_SIZE.  The caller still provides inputs and outputs.
//
// Every call looks up the array's device address on the current device with
// cudaGetSymbolAddress (host code cannot use the array's name as a device
// address), and ends by reading a failure counter back and synchronising
// `stream`, so a call cannot be captured into a CUDA graph.  The first call
// on a device loads the module and should come before any stream capture on
// that device.  All calls share the array and it keeps the last call's
// contents; the counters are cleared on every call, and calls that overlap on
// the GPU (other streams, other host threads) race on the array: serialise
// them.  Mixed precision runs every cluster size on the FP32 CUDA-core
// kernels (OOPS_PREC_MIXED and OOPS_PREC_MIXED_SIMT are the same here);
// fp64_max_k switches small clusters to FP64 as in oops_cce_coherence, and
// fp64_below > 0 in a mixed mode is OOPS_ERR_UNSUPPORTED (its recomputation
// needs buffers sized by the number of flagged clusters).
// ---------------------------------------------------------------------------
#define OOPS_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[OOPS_NOALLOC_SCRATCH_BYTES];

namespace {

void *noalloc_base(int *rc)
{
    // looked up on every call: the address belongs to the current device's
    // context and is not cached across calls, devices or context teardowns
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        *rc = oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
        return nullptr;
    }
    *rc = OOPS_OK;
    return p;
}

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

template <int K>
int run_class_noalloc(const double *coords, const unsigned *clusters, int ncl, const PhysParams &pp,
                      int pulse_num, int nT, double dt, int precision, double *L, cudaStream_t st)
{
    constexpr int D = 1 << K;
    const int sms = oops_sm_count();
    const int tslices = std::max(1, std::min(nT, (sms * 4 + ncl - 1) / std::max(1, ncl)));
    size_t fp64_smem = (size_t)6 * D * D * sizeof(double2);
    const bool gws_needed = precision == OOPS_PREC_FP64 && fp64_smem > 200 * 1024;
    const int grid64 = std::max(1, std::min(ncl * tslices, sms * (D >= 32 ? 1 : 4)));
    const size_t b_ctr = 256;
    const size_t b_w = up256((size_t)ncl * 2 * D * sizeof(double));
    const size_t b_V = up256((size_t)ncl * 2 * D * D * sizeof(zd));
    const size_t b_M = up256((size_t)ncl * D * D * sizeof(zd));
    const size_t b_g = gws_needed ? up256((size_t)grid64 * fp64_smem) : 0;
    const size_t b_p = precision != OOPS_PREC_FP64 ? up256((size_t)ncl * 4 * D * sizeof(unsigned long long)) : 0;
    const size_t b_m32 = precision != OOPS_PREC_FP64 ? up256((size_t)ncl * D * D * sizeof(float2)) : 0;
    const size_t need = b_ctr + b_w + b_V + b_M + b_g + b_p + b_m32;
    if (need > OOPS_NOALLOC_SCRATCH_BYTES)
        return oops_set_status(OOPS_ERR_SIZE,
                               "oops_cce_coherence_noalloc: the batch needs more scratch than the "
                               "32 MiB static array; pass fewer clusters per call");
    int rc = OOPS_OK;
    unsigned char *base = (unsigned char *)noalloc_base(&rc);
    if (rc) return rc;
    int *ctr = (int *)base;
    double *w = (double *)(base + b_ctr);
    zd *V = (zd *)(base + b_ctr + b_w);
    zd *M = (zd *)(base + b_ctr + b_w + b_V);
    double2 *gws = gws_needed ? (double2 *)(base + b_ctr + b_w + b_V + b_M) : nullptr;
    unsigned long long *phi = b_p ? (unsigned long long *)(base + b_ctr + b_w + b_V + b_M + b_g) : nullptr;
    float2 *M32 = b_m32 ? (float2 *)(base + b_ctr + b_w + b_V + b_M + b_g + b_p) : nullptr;
    // work-queue and failure counters must start at zero on every call
    cudaError_t e = cudaMemsetAsync(ctr, 0, 4 * sizeof(int), st);
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    {
        size_t smem = (size_t)3 * D * D * sizeof(zd);
        cudaFuncSetAttribute(k_assemble_eig<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = tune_eig_per_sm(K);
        int grid = std::max(1, std::min(2 * ncl, sms * per_sm));
        k_assemble_eig<K><<<grid, EIG_THREADS<K>, smem, st>>>(coords, clusters, ncl, pp, nullptr, w, V, ctr + 0, ctr + 3,
                                                    eig_rel_gap(precision));
    }
    k_overlap<K><<<ncl, 256, 0, st>>>(V, ncl, M, M32);
    if (phi) launch_phase_steps<K>(w, ncl, pulse_num, dt, phi, st);
    if (precision == OOPS_PREC_FP64) {
        size_t smem = gws_needed ? 0 : fp64_smem;
        cudaFuncSetAttribute(k_coherence<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_coherence<K, double><<<grid64, 256, smem, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, tslices, L,
                                                          ctr + 1, gws, gws_needed ? 0 : 1);
    } else {
        size_t smem = (size_t)6 * D * D * sizeof(float2);
        int grid = std::max(1, std::min(ncl * tslices, sms * (D >= 64 ? 1 : (D >= 32 ? 2 : 4))));
        cudaFuncSetAttribute(k_coherence<K, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_coherence<K, float><<<grid, 256, smem, st>>>(w, phi, M, M32, ncl, pulse_num, nT, dt, tslices, L,
                                                       ctr + 2, nullptr, 1);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    int fails = 0;
    cudaMemcpyAsync(&fails, ctr + 3, sizeof(int), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    if (fails) return oops_set_status(OOPS_ERR_NUMERIC, "Jacobi eigensolver did not converge");
    return OOPS_OK;
}

}  // namespace

extern "C" int oops_cce_coherence_noalloc(const double *coords_dev, size_t nbath,
                                          const unsigned *clusters_dev, size_t ncl, int k,
                                          const oops_cce_params *p, int precision, double *L_dev,
                                          void *stream)
{
    if (!coords_dev || !clusters_dev || !p || !L_dev) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (k < 1 || k > MAX_K) return oops_set_status(OOPS_ERR_SIZE, "cluster size must be 1..6 (dense path)");
    if (p->pulse_num < 1 || p->pulse_num > 64) return oops_set_status(OOPS_ERR_SIZE, "pulse_num must be 1..64");
    if (p->nT < 1 || p->nT > (1u << 24)) return oops_set_status(OOPS_ERR_SIZE, "nT out of range");
    if (precision != OOPS_PREC_FP64 && precision != OOPS_PREC_MIXED &&
        precision != OOPS_PREC_MIXED_SIMT)
        return oops_set_status(OOPS_ERR_ARG, "unknown precision");
    if (precision != OOPS_PREC_FP64 && p->fp64_below > 0.0)
        return oops_set_status(OOPS_ERR_UNSUPPORTED,
                               "oops_cce_coherence_noalloc: fp64_below is not supported (its FP64 "
                               "recomputation allocates per flagged cluster)");
    if (ncl == 0) return OOPS_OK;
    if (ncl > (1u << 24)) return oops_set_status(OOPS_ERR_SIZE, "too many clusters");
    (void)nbath;
    const PhysParams pp = phys_params(p);
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)ncl, nT = (int)p->nT;
    if (precision != OOPS_PREC_FP64 && k <= p->fp64_max_k) precision = OOPS_PREC_FP64;
    if (precision == OOPS_PREC_MIXED_SIMT) precision = OOPS_PREC_MIXED;
    switch (k) {
        case 1: return run_class_noalloc<1>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
        case 2: return run_class_noalloc<2>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
        case 3: return run_class_noalloc<3>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
        case 4: return run_class_noalloc<4>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
        case 5: return run_class_noalloc<5>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
        default: return run_class_noalloc<6>(coords_dev, clusters_dev, n, pp, p->pulse_num, nT, p->dt, precision, L_dev, st);
    }
}
