// cce_tc.cu -- tensor-core (tcgen05) per-time-point coherence for clusters
// of six spin-1/2 nuclei (D = 64), mixed precision.
//
// Same observable as k_coherence<6,float> in cce_dense.cu:
//   L(t) = Re Tr(B1^+ B0) / D (normalised difference form, coherence_from_sums),
//   B0 = U0(s0 t) U1(s1 t) ..., B1 = 0 <-> 1,
// in the eigenbasis of H_0: U0(tau) = E0(tau) = diag(e^{-i w0 tau}) and
// U1(tau) = Y(tau) = M E1(tau) M^+.  Every complex 64x64 product runs on the
// 5th-generation tensor cores:
//   * operands are split hi + lo in FP16 (|entries| <= 1: the pair carries
//     ~22 bits, absolute error ~3e-8) and each product is the three passes
//     hi*hi + hi*lo + lo*hi with FP32 accumulation in tensor memory;
//   * A = [Re X ; Im X] (128 x 64, K-major) and B = Re G^T, Im G^T (64 x 64,
//     K-major): D1 = A Re G, D2 = A Im G in TMEM columns 0..63 and 64..127,
//     one tcgen05.mma (M=128, N=64, K=16) per pass, half and K slice: 24 per
//     product, issued by one thread, completion through an mbarrier;
//   * the epilogue (tcgen05.ld) pairs thread t with t^64 so that each thread
//     owns complete complex entries of 16 columns of one row, splits them
//     into the next operand and never needs a cross-thread complex product:
//     every diagonal phase factor of the pulse sequence is folded into a
//     "group" operand G = Y(y) E0(d) or into the chain's first factor.
// FP64 stays in the eigendecomposition, the per-cluster phase steps and the
// cross-thread trace sums.  Shared memory: two A operands (hi/lo, 32 KB each,
// also the epilogues' exchange buffers) and four complex B slots (M^H and up
// to three groups, 32 KB each).  One CTA of 256 threads per SM (each thread
// owns 16 columns of one row of every product), TMEM 256 columns: the two
// branch chains (and the two Y builds) are software-pipelined, each with its
// own A operand, accumulator and mbarrier, so one branch's products run on
// the tensor cores while the threads run the other branch's epilogue and
// operand packing.  Operand rows are packed into 16-byte shared stores (8
// FP16 values along K, one core-matrix row); group operands are transposed
// in registers by 8-lane shuffles first.
// Supported pulse sequences: Hahn (n = 1) and CPMG with even n; the caller
// uses the FP32 CUDA-core kernel otherwise.  Every wait is bounded; on
// timeout the CTA records OOPS_ERR_TIMEOUT, waits (bounded) for its products
// in flight, frees its TMEM and exits.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "oops_common.cuh"
#include "oops_internal.h"

namespace {

constexpr int D = 64;
constexpr int NT = 256;                  // threads per CTA (8 warps)
constexpr int CW = 16;                   // output columns per thread
constexpr int OP_BYTES = 128 * 64 * 2;   // one FP16 128x64 operand (16 KB)
constexpr int HALF_OP = 64 * 64 * 2;     // one FP16 64x64 operand (8 KB)
constexpr int SLOT_BYTES = 4 * HALF_OP;  // Re hi, Re lo, Im hi, Im lo (32 KB)
constexpr int NSLOT = 4;
constexpr int ABUF_BYTES = 2 * OP_BYTES;  // one A operand, hi | lo (32 KB)
constexpr int SMEM_DYN = 2 * ABUF_BYTES + NSLOT * SLOT_BYTES;  // 196608
constexpr int TMEM_COLS = 256;           // two accumulators of 128 columns
constexpr long SPIN_LIMIT = 20000000;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// K-major canonical layout without swizzle: core matrices of 8 rows x 16 bytes
// (8 fp16 along K), core (rb, kb) at ((rb * 8) + kb) * 128 bytes (K = 64).
__device__ __forceinline__ int kmaj_off(int row, int k)
{
    return (((row >> 3) * 8 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2) >> 1;  // in halves
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    // LBO = 128 B (next core matrix along K), SBO = 1024 B (next 8 rows)
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// idesc: D f32, A/B f16, K-major both, N = 64, M = 128
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(64 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void split16(float x, __half &hi, __half &lo)
{
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

struct Smem {
    __half *A[2];  // two A operands: [hi 16K | lo 16K] each
    __half *slot;  // NSLOT x 32 KB
};

__device__ __forceinline__ uint32_t pack2(__half lo_k, __half hi_k)
{
    __half2 p = __halves2half2(lo_k, hi_k);
    return *reinterpret_cast<uint32_t *>(&p);
}

// hi + lo split of two values at once: hi = x rounded to FP16's 11
// significant bits in FP32 integer arithmetic (add half an FP16 ulp to the
// magnitude bits, clear the 13 dropped bits), lo = x - hi exactly in FP32,
// each pair converted by one packed cvt.  Three conversions per value become
// one per value; the pair sums to x within an FP16 ulp of lo (~2^-22 |x|),
// as split16's does (values below FP16's normal range, |x| < 2^-14, keep an
// absolute error of ~2^-25 either way).
__device__ __forceinline__ void split16x2(float a, float b, uint32_t &hi2, uint32_t &lo2)
{
    const float ha = __uint_as_float((__float_as_uint(a) + 0x1000u) & 0xFFFFE000u);
    const float hb = __uint_as_float((__float_as_uint(b) + 0x1000u) & 0xFFFFE000u);
    __half2 h = __floats2half2_rn(ha, hb);
    __half2 l = __floats2half2_rn(a - ha, b - hb);
    hi2 = *reinterpret_cast<uint32_t *>(&h);
    lo2 = *reinterpret_cast<uint32_t *>(&l);
}

// Thread layout (256 threads): thread t reads TMEM lane l = t & 127 (row l
// of the 128-row accumulator [Re X; Im X] G), columns of quarter q = t >> 7,
// and after the exchange in the epilogue owns row r = l & 63 of the complex
// product at columns cbase .. cbase+15, cbase = 32 q + 16 (l >> 6).  Within a
// warp q and l >> 6 are uniform, so TMEM loads are warp-uniform.
__device__ __forceinline__ int col_base(int t) { return 32 * (t >> 7) + 16 * ((t >> 6) & 1); }

// Row r of a complex 64 x 64 factor, columns cbase .. cbase+15 (v[j] = entry
// at column cbase + j), into A operand `A`: Re at row r, Im at row 64 + r, hi
// and lo parts.  Eight consecutive K values of one row are one 16-byte
// core-matrix row: 8 vector stores per call, four wavefronts each across a
// warp (its 32 rows fill four core-matrix columns).
__device__ __forceinline__ void put_A_row(__half *A, int r, int cbase, const float2 *v)
{
#pragma unroll
    for (int kb = 0; kb < CW / 8; ++kb) {
        uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float2 a = v[8 * kb + 2 * p], b = v[8 * kb + 2 * p + 1];
            split16x2(a.x, b.x, rh[p], rl[p]);
            split16x2(a.y, b.y, ih[p], il[p]);
        }
        const int k0 = cbase + 8 * kb;
        const int oRe = kmaj_off(r, k0), oIm = kmaj_off(64 + r, k0);  // halves, 16-byte aligned
        *reinterpret_cast<uint4 *>(A + oRe) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
        *reinterpret_cast<uint4 *>(A + OP_BYTES / 2 + oRe) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
        *reinterpret_cast<uint4 *>(A + oIm) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
        *reinterpret_cast<uint4 *>(A + OP_BYTES / 2 + oIm) = make_uint4(il[0], il[1], il[2], il[3]);
    }
}

// Entries G[r][cbase + j] (j < 16, this thread's row r) of a group operand
// into slot s, transposed (B[n = c][k = r], K-major).  The eight lanes that
// hold rows r0 .. r0+7 transpose each 8 x 8 block with a three-stage
// shuffle butterfly (static register indices through selects), after which
// lane i holds column cbase + 8 blk + i for rows r0 .. r0+7: one 16-byte
// store per part instead of eight 2-byte stores, four wavefronts per warp.
__device__ __forceinline__ void put_B_rows(Smem &S, int s, int r, int cbase, const float2 *v)
{
    __half *b = S.slot + (size_t)s * (SLOT_BYTES / 2);
    const int lane8 = threadIdx.x & 7;
    const int r0 = r & ~7;
#pragma unroll
    for (int blk = 0; blk < CW / 8; ++blk) {
        float2 a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = v[8 * blk + k];
#pragma unroll
        for (int bit = 4; bit >= 1; bit >>= 1) {
            const bool hi = (lane8 & bit) != 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k & bit) continue;
                const float2 send = hi ? a[k] : a[k | bit];
                float2 recv;
                recv.x = __shfl_xor_sync(0xffffffffu, send.x, bit);
                recv.y = __shfl_xor_sync(0xffffffffu, send.y, bit);
                if (hi) a[k] = recv;
                else a[k | bit] = recv;
            }
        }
        // a[k] = G[r0 + k][c], c = cbase + 8 blk + lane8
        uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            split16x2(a[2 * p].x, a[2 * p + 1].x, rh[p], rl[p]);
            split16x2(a[2 * p].y, a[2 * p + 1].y, ih[p], il[p]);
        }
        const int o = kmaj_off(cbase + 8 * blk + lane8, r0);  // halves, 16-byte aligned
        *reinterpret_cast<uint4 *>(b + o) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
        *reinterpret_cast<uint4 *>(b + HALF_OP / 2 + o) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
        *reinterpret_cast<uint4 *>(b + 2 * (HALF_OP / 2) + o) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
        *reinterpret_cast<uint4 *>(b + 3 * (HALF_OP / 2) + o) = make_uint4(il[0], il[1], il[2], il[3]);
    }
}

// one complex product A x slot s -> TMEM columns tmem .. tmem+127 (issued by
// thread 0), completion signalled on mbar
__device__ __forceinline__ void issue_product(const Smem &S, const __half *A, int s, uint32_t tmem,
                                              uint32_t mbar)
{
    const uint32_t a0 = smem_u32(A);
    const uint32_t b0 = smem_u32(S.slot) + (uint32_t)s * SLOT_BYTES;
    // passes: (A hi, B hi), (A hi, B lo), (A lo, B hi)
    const uint32_t aoff[3] = {0u, 0u, (uint32_t)OP_BYTES};
    const uint32_t boff[3] = {0u, (uint32_t)HALF_OP, 0u};
    for (int part = 0; part < 2; ++part) {           // Re G -> cols 0..63, Im G -> 64..127
        const uint32_t dcol = tmem + (uint32_t)(part * 64);
        const uint32_t bpart = b0 + (uint32_t)(part * 2 * HALF_OP);
        for (int p = 0; p < 3; ++p)
            for (int kk = 0; kk < 4; ++kk) {
                const uint64_t ad = sdesc(a0 + aoff[p] + (uint32_t)kk * 256u);
                const uint64_t bd = sdesc(bpart + boff[p] + (uint32_t)kk * 256u);
                const uint32_t acc = (p > 0 || kk > 0) ? 1u : 0u;
                asm volatile("{\n.reg .pred q;\nsetp.ne.u32 q, %4, 0;\n"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}" ::"r"(dcol),
                             "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
            }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

// bounded wait for mbarrier phase `parity`; returns false on timeout
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t parity)
{
    for (long it = 0; it < SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(mbar), "r"(parity));
        if (done) return true;
    }
    return false;
}

// load 16 TMEM columns starting at taddr for this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Epilogue: out[j] = C[r][cbase + j], C = X G the complex product in TMEM
// columns tmem .. tmem+127 (Re G part in the first 64, Im G part in the next
// 64).  Thread t reads lane t & 127, which holds (Re X G) for t & 64 == 0 and
// (Im X G) otherwise; t and t ^ 64 swap the 16 columns the other one owns
// through the A operand `A` (free: the product that read it is complete).
// All reads of this accumulator are complete when it returns.
__device__ void epilogue(__half *A, uint32_t tmem, float2 *out)
{
    const int t = threadIdx.x;
    const int warp = t >> 5;
    const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    float *X = reinterpret_cast<float *>(A);  // 256 x 32 floats, rotated columns
    const int p = (t >> 6) & 1;                  // 0: Re X row, 1: Im X row
    const int keep = col_base(t);
    const int give = 32 * (t >> 7) + (p == 0 ? 16 : 0);  // the partner's columns
    {
        float g[16];
        tmem_ld16(lane_addr + give, g);
#pragma unroll
        for (int j = 0; j < 16; ++j) X[t * 32 + ((2 * j + t) & 31)] = g[j];
        tmem_ld16(lane_addr + 64 + give, g);
#pragma unroll
        for (int j = 0; j < 16; ++j) X[t * 32 + ((2 * j + 1 + t) & 31)] = g[j];
    }
    __syncthreads();
    float k1[16], k2[16];
    tmem_ld16(lane_addr + keep, k1);
    tmem_ld16(lane_addr + 64 + keep, k2);
    asm volatile("tcgen05.fence::before_thread_sync;");
    const int pt = t ^ 64;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float pr = X[pt * 32 + ((2 * j + pt) & 31)];
        const float pi = X[pt * 32 + ((2 * j + 1 + pt) & 31)];
        // p = 0: own = (Xr Gr, Xr Gi), partner = (Xi Gr, Xi Gi); p = 1: swapped
        const float xrgr = p == 0 ? k1[j] : pr;
        const float xrgi = p == 0 ? k2[j] : pi;
        const float xigr = p == 0 ? pr : k1[j];
        const float xigi = p == 0 ? pi : k2[j];
        out[j] = make_float2(xrgr - xigi, xrgi + xigr);
    }
    __syncthreads();  // exchange reads done: A may be rewritten
}

__global__ void __launch_bounds__(NT, 1)
k_coherence_tc64(const unsigned long long *__restrict__ phi, const float2 *__restrict__ Mg, int ncl,
                 int pulse_num, int nT, int tslices, double *__restrict__ L, int *__restrict__ queue,
                 int *__restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_item, s_abort;
    __shared__ float2 e0h[D], e0f[D], e1h[D], e1f[D];
    __shared__ unsigned long long phs[4 * D];  // phase steps [branch][h, f][d]
    __shared__ float red[3][NT / 32];
    // group program: per branch, lead diagonal type (-1 none, 0 h, 1 f) and
    // groups (y, d) with y in {0 h, 1 f}, d in {-1 none, 0 h, 1 f}
    __shared__ int g_lead[2], g_n[2], g_y[2][40], g_d[2][40], g_slot[2][40];
    __shared__ int s_need[2][3];  // slot of group (y, d) keyed (y, d+1); -1 if unused
    Smem S;
    S.A[0] = reinterpret_cast<__half *>(smraw);
    S.A[1] = reinterpret_cast<__half *>(smraw + ABUF_BYTES);
    S.slot = reinterpret_cast<__half *>(smraw + 2 * ABUF_BYTES);
    const int t = threadIdx.x;
    const int r = t & 63, cb = col_base(t);
    const int nseg = pulse_num + 1;
    if (t == 0) {
        s_abort = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 3; ++b) s_need[a][b] = -1;
        int next_slot = 1;  // slot 0 holds M^H
        for (int br = 0; br < 2; ++br) {
            int j = 0, n = 0;
            g_lead[br] = -1;
            if (((0 + br) & 1) == 0) {  // first factor is U0
                g_lead[br] = 0;         // segment 0 has fraction h
                j = 1;
            }
            while (j < nseg && n < 40) {
                const int y = (j == 0 || j == nseg - 1) ? 0 : 1;
                int d = -1;
                if (j + 1 < nseg) d = (j + 1 == nseg - 1) ? 0 : 1;
                g_y[br][n] = y;
                g_d[br][n] = d;
                ++n;
                j += (d >= 0) ? 2 : 1;
            }
            if (j < nseg) s_abort = 2;  // longer program than the tables
            g_n[br] = n;
        }
        for (int br = 0; br < 2; ++br)
            for (int q = 0; q < g_n[br]; ++q) {
                g_slot[br][q] = -1;
                if (q == 0) continue;  // the first group is the chain's start (A)
                int &sl = s_need[g_y[br][q]][g_d[br][q] + 1];
                if (sl < 0) sl = next_slot++;
                g_slot[br][q] = sl;
            }
        if (next_slot > NSLOT) s_abort = 2;  // more distinct groups than slots
        for (int b = 0; b < 2; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[b])));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "n"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const uint32_t mb[2] = {smem_u32(&mbar[0]), smem_u32(&mbar[1])};
    uint32_t phase[2] = {0, 0};
    bool inflight[2] = {false, false};  // a committed product not yet waited for (uniform)
    const double frac_h = 0.5 / pulse_num, frac_f = pulse_num > 1 ? 1.0 / pulse_num : frac_h;
    const bool two = frac_f != frac_h;
    if (s_abort == 2) {
        if (t == 0) atomicCAS(status, 0, OOPS_ERR_UNSUPPORTED);
        goto done;
    }
    {
        const int per = (nT + tslices - 1) / tslices;
        int cur_cl = -1;
        for (;;) {
            __syncthreads();
            if (t == 0) s_item = atomicAdd(queue, 1);
            __syncthreads();
            const int item = s_item;
            if (item >= ncl * tslices || s_abort) break;
            const int cl = item / tslices, sl = item % tslices;
            const float2 *M = Mg + (size_t)cl * D * D;  // FP32 copy of M
            if (cl != cur_cl) {
                cur_cl = cl;
                for (int e = t; e < 4 * D; e += NT) phs[e] = phi[(size_t)cl * 4 * D + e];
                // slot 0: M^H as a B operand: B[n][k] = (M^H)[k][n] = conj(M[n][k])
                __half *b = S.slot;
                for (int e = t; e < D * D; e += NT) {
                    const int n = e % D, k = e / D;   // M column-major: M[n][k] = Mg[n + D k]
                    const float2 m = M[n + (size_t)D * k];
                    const int o = kmaj_off(n, k);
                    __half hh, ll;
                    split16(m.x, hh, ll);
                    b[o] = hh;
                    b[HALF_OP / 2 + o] = ll;
                    split16(-m.y, hh, ll);
                    b[2 * (HALF_OP / 2) + o] = hh;
                    b[3 * (HALF_OP / 2) + o] = ll;
                }
            }
            const int i0 = sl * per, i1 = min(nT, i0 + per);
            for (int i = i0; i < i1 && !s_abort; ++i) {
                if (i == 0) {
                    if (t == 0) L[(size_t)cl * nT] = 1.0;
                    continue;
                }
                __syncthreads();
                if (t < D) {
                    e0h[t] = phase_step_f(phs[t], i);
                    e0f[t] = phase_step_f(phs[D + t], i);
                    e1h[t] = phase_step_f(phs[2 * D + t], i);
                    e1f[t] = phase_step_f(phs[3 * D + t], i);
                }
                __syncthreads();
                float2 cur[2][CW];  // the two chains: row r, columns cb .. cb+15
                // ---- Y(h) (y = 0, A operand 0) and Y(f) (y = 1, A operand 1),
                // both products issued before either epilogue
                {
                    float2 v[CW];
#pragma unroll
                    for (int y = 0; y < 2; ++y) {
                        if (y == 1 && !two) break;
                        const float2 *e1 = y == 0 ? e1h : e1f;
#pragma unroll
                        for (int j = 0; j < CW; ++j) {
                            const int k = cb + j;
                            v[j] = cmulf(M[r + (size_t)D * k], e1[k]);
                        }
                        put_A_row(S.A[y], r, cb, v);
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;");
                __syncthreads();
                asm volatile("tcgen05.fence::after_thread_sync;");
                if (t == 0) {
                    issue_product(S, S.A[0], 0, tmem, mb[0]);
                    if (two) issue_product(S, S.A[1], 0, tmem + 128, mb[1]);
                }
                inflight[0] = true;
                inflight[1] = two;
#pragma unroll
                for (int y = 0; y < 2; ++y) {
                    if (y == 1 && !two) break;
                    if (!wait_phase(mb[y], phase[y])) s_abort = 1;
                    __syncthreads();  // the abort flag is uniform from here
                    if (s_abort) break;
                    phase[y] ^= 1;
                    inflight[y] = false;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    float2 Yv[CW];
                    epilogue(S.A[y], tmem + (uint32_t)(128 * y), Yv);
                    // groups with this y into their slots; chain starts to registers
#pragma unroll
                    for (int dd = -1; dd <= 1; ++dd) {
                        const int s = s_need[y][dd + 1];
                        if (s < 0) continue;  // uniform: s_need is shared
                        const float2 *e0 = dd == 0 ? e0h : e0f;
                        float2 g[CW];
#pragma unroll
                        for (int j = 0; j < CW; ++j) g[j] = dd < 0 ? Yv[j] : cmulf(Yv[j], e0[cb + j]);
                        put_B_rows(S, s, r, cb, g);
                    }
#pragma unroll
                    for (int br = 0; br < 2; ++br) {
                        if (g_y[br][0] != y && two) continue;
                        const int dd = g_d[br][0];
#pragma unroll
                        for (int j = 0; j < CW; ++j) {
                            const int c = cb + j;
                            float2 v = dd < 0 ? Yv[j] : cmulf(Yv[j], dd == 0 ? e0h[c] : e0f[c]);
                            if (g_lead[br] >= 0) v = cmulf(g_lead[br] == 0 ? e0h[r] : e0f[r], v);
                            cur[br][j] = v;
                        }
                    }
                }
                if (s_abort) break;
                // ---- the two chains, pipelined: while one branch's product
                // runs, the threads finish the other branch's epilogue and
                // pack its next operand
                int q[2] = {1, 1};
#pragma unroll
                for (int br = 0; br < 2; ++br)
                    if (q[br] < g_n[br]) put_A_row(S.A[br], r, cb, cur[br]);
                asm volatile("fence.proxy.async.shared::cta;");
                __syncthreads();
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int br = 0; br < 2; ++br) {
                    if (q[br] < g_n[br]) {
                        if (t == 0) issue_product(S, S.A[br], g_slot[br][q[br]], tmem + (uint32_t)(128 * br), mb[br]);
                        inflight[br] = true;
                    }
                }
                while (inflight[0] || inflight[1]) {
#pragma unroll
                    for (int br = 0; br < 2; ++br) {
                        if (!inflight[br] || s_abort) continue;
                        if (!wait_phase(mb[br], phase[br])) s_abort = 1;
                        __syncthreads();  // the abort flag is uniform from here
                        if (s_abort) continue;
                        phase[br] ^= 1;
                        inflight[br] = false;
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        epilogue(S.A[br], tmem + (uint32_t)(128 * br), cur[br]);
                        ++q[br];
                        if (q[br] < g_n[br]) {
                            put_A_row(S.A[br], r, cb, cur[br]);
                            asm volatile("fence.proxy.async.shared::cta;");
                            __syncthreads();
                            asm volatile("tcgen05.fence::after_thread_sync;");
                            if (t == 0) issue_product(S, S.A[br], g_slot[br][q[br]], tmem + (uint32_t)(128 * br), mb[br]);
                            inflight[br] = true;
                        }
                    }
                    if (s_abort) break;
                }
                if (s_abort) break;
                // the trace sums in FP32 (relative error ~1e-6, which moves
                // L by ~1e-6 (1 - L))
                float fr = 0.f, f0 = 0.f, f1 = 0.f;
#pragma unroll
                for (int j = 0; j < CW; ++j) {
                    const float dr = cur[0][j].x - cur[1][j].x, di = cur[0][j].y - cur[1][j].y;
                    fr = fmaf(dr, dr, fmaf(di, di, fr));
                    f0 = fmaf(cur[0][j].x, cur[0][j].x, fmaf(cur[0][j].y, cur[0][j].y, f0));
                    f1 = fmaf(cur[1][j].x, cur[1][j].x, fmaf(cur[1][j].y, cur[1][j].y, f1));
                }
                for (int off = 16; off > 0; off >>= 1) {
                    fr += __shfl_down_sync(0xffffffffu, fr, off);
                    f0 += __shfl_down_sync(0xffffffffu, f0, off);
                    f1 += __shfl_down_sync(0xffffffffu, f1, off);
                }
                if ((t & 31) == 0) {
                    red[0][t >> 5] = fr;
                    red[1][t >> 5] = f0;
                    red[2][t >> 5] = f1;
                }
                __syncthreads();
                if (t == 0) {
                    float sum = 0, s0 = 0, s1 = 0;
                    for (int qq = 0; qq < NT / 32; ++qq) {
                        sum += red[0][qq];
                        s0 += red[1][qq];
                        s1 += red[2][qq];
                    }
                    // the defect in FP32, 1 - x in FP64
                    L[(size_t)cl * nT + i] = 1.0 - (double)coherence_defect_f(s0, s1, sum);
                }
            }
        }
    }
done:
    if (s_abort == 1) {
        // a product did not complete in time: give every product still in
        // flight one more bounded wait before the tensor memory is released
        for (int b = 0; b < 2; ++b)
            if (inflight[b]) wait_phase(mb[b], phase[b]);
        if (t == 0) atomicCAS(status, 0, OOPS_ERR_TIMEOUT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TMEM_COLS));
}

}  // namespace

bool oops_tc64_supported(int pulse_num) { return pulse_num == 1 || (pulse_num % 2 == 0); }

// Launch the tensor-core coherence for ncl six-spin clusters (phi: phase
// steps, 4*64 per cluster; M: FP32 overlaps, 64x64 per cluster; L: ncl x nT).  queue and
// status are device ints that start at zero; the time grid is split so that
// about sms * tslice_mult items exist.
int oops_coherence_tc64(const unsigned long long *phi, const float2 *M, int ncl, int pulse_num,
                        int nT, double *L, int *queue, int *status, int tslice_mult, cudaStream_t st)
{
    if (!oops_tc64_supported(pulse_num))
        return oops_set_status(OOPS_ERR_UNSUPPORTED, "tensor-core path: Hahn or even CPMG only");
    const int sms = oops_sm_count();
    const int tslices = std::max(1, std::min(nT, (sms * std::max(1, tslice_mult) + ncl - 1) / std::max(1, ncl)));
    const int grid = std::max(1, std::min(ncl * tslices, sms));
    cudaFuncSetAttribute(k_coherence_tc64, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_DYN);
    k_coherence_tc64<<<grid, NT, SMEM_DYN, st>>>(phi, M, ncl, pulse_num, nT, tslices, L, queue, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    return OOPS_OK;
}
