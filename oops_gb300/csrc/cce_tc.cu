// cce_tc.cu -- tensor-core (tcgen05) per-time-point coherence for clusters
// of six spin-1/2 nuclei (D = 64), mixed precision.
//
// Same observable as k_coherence<6,float> in cce_dense.cu:
//   L(t) = Re Tr(B1^+ B0) / D (normalised difference form, coherence_from_sums),
//   B0 = U0(s0 t) U1(s1 t) ..., B1 = 0 <-> 1,
// in the eigenbasis of H_0: U0(tau) = E0(tau) = diag(e^{-i w0 tau}) and
// U1(tau) = Y(tau) = M E1(tau) M^+.  Every complex 64x64 product runs on the
// 5th-generation tensor cores:
//   * operands hold 2^8 times the factor (entries <= 256) split hi + lo in
//     FP16 (the pair carries ~22 bits, relative error ~2^-22, absolute floor
//     2^-33 of the unscaled entry) and each product is the three passes
//     hi*hi + hi*lo + lo*hi with FP32 accumulation in tensor memory;
//   * A = the rows of Re X and Im X (128 x 64, K-major; interleaved in blocks
//     of 16 rows, see row_of) and B = Re G^T, Im G^T (64 x 64,
//     K-major): D1 = A Re G, D2 = A Im G in TMEM columns 0..63 and 64..127,
//     one tcgen05.mma (M=128, N=64, K=16) per pass, half and K slice: 24 per
//     product, issued by one thread, completion through an mbarrier;
//   * the epilogue (tcgen05.ld) pairs thread t with t^16 (warp shuffles) so
//     that each thread owns complete complex entries of 16 columns of one
//     row, splits them
//     into the next operand and never needs a cross-thread complex product:
//     every diagonal phase factor of the pulse sequence is folded into a
//     "group" operand G = Y(y) E0(d) or into the chain's first factor.
// FP64 stays in the eigendecomposition, the per-cluster phase steps and the
// cross-thread trace sums.  Shared memory: two A operands (hi/lo, 32 KB each)
// and four complex B slots (M^H and up
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

// Operand scaling: every A and B operand holds its factor times OP_SCALE =
// 2^8 (entries |x| <= 1 become <= 256, far inside FP16's range), so the
// accumulators hold 2^16 times the product and the chains carry that scale;
// an operand built from a chain value is split with OP_UNSCALE = 2^-8.  The
// scale keeps the hi parts of entries down to 2^-22 in FP16's normal range
// (the packed split below is exact there) and lowers the absolute error floor
// of the split from FP16's subnormal spacing, 2^-25, to 2^-33.  Powers of two:
// exact.  The trace form L = 1 - (d - (sqrt n0 - sqrt n1)^2) / (2 sqrt(n0 n1))
// is invariant under the common scale.
constexpr float OP_SCALE = 256.0f, OP_UNSCALE = 1.0f / 256.0f;

// hi + lo split of two values at once, each first multiplied by `scale`: hi
// = x rounded to FP16's 11 significant bits in FP32 integer arithmetic (add
// half an FP16 ulp to the magnitude bits, clear the 13 dropped bits; ties
// away from zero), exactly representable in FP16 when |x| >= 2^-14, so lo =
// x - hi is exact in FP32 and the pair sums to x within an FP16 ulp of lo
// (~2^-22 |x|), as split16's does; each pair is converted by one packed cvt,
// one conversion per value instead of split16's three.
__device__ __forceinline__ void split16x2(float a, float b, uint32_t &hi2, uint32_t &lo2, float scale)
{
    a *= scale;
    b *= scale;
    const float ha = __uint_as_float((__float_as_uint(a) + 0x1000u) & 0xFFFFE000u);
    const float hb = __uint_as_float((__float_as_uint(b) + 0x1000u) & 0xFFFFE000u);
    __half2 h = __floats2half2_rn(ha, hb);
    __half2 l = __floats2half2_rn(a - ha, b - hb);
    hi2 = *reinterpret_cast<uint32_t *>(&h);
    lo2 = *reinterpret_cast<uint32_t *>(&l);
}

// Thread layout (256 threads).  The A operand holds the rows of Re X and
// Im X interleaved in blocks of 16: A row 32 (r >> 4) + (r & 15) is Re X row
// r and the row 16 below it Im X row r, so TMEM lanes l and l ^ 16 of the
// accumulator hold (Re X) G and (Im X) G of the same row r, in the same warp.
// Thread t reads lane l = t & 127 (part p = (t >> 4) & 1: 0 Re, 1 Im), the
// columns of quarter q = t >> 7, and after the exchange with thread t ^ 16
// (warp shuffles) owns row r = 16 ((t >> 5) & 3) + (t & 15) of the complex
// product at columns cbase .. cbase+15, cbase = 32 q + 16 p.  TMEM load
// addresses are warp-uniform (q is uniform in a warp; both halves of the
// quarter are loaded and the thread keeps its own).  Eight consecutive
// threads hold eight consecutive rows at the same columns (put_B_rows).
__device__ __forceinline__ int row_of(int t) { return 16 * ((t >> 5) & 3) + (t & 15); }
__device__ __forceinline__ int col_base(int t) { return 32 * (t >> 7) + 16 * ((t >> 4) & 1); }
__device__ __forceinline__ int a_row(int r) { return 32 * (r >> 4) + (r & 15); }  // Re; Im at + 16

// Row r of a complex 64 x 64 factor, columns cbase .. cbase+15 (v[j] = entry
// at column cbase + j), into A operand `A`: Re at row a_row(r), Im 16 rows
// below it, hi
// and lo parts.  Eight consecutive K values of one row are one 16-byte
// core-matrix row: 8 vector stores per call, four wavefronts each across a
// warp (its 32 rows fill four core-matrix columns).
__device__ __forceinline__ void put_A_row(__half *A, int r, int cbase, const float2 *v, float scale)
{
#pragma unroll
    for (int kb = 0; kb < CW / 8; ++kb) {
        uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float2 a = v[8 * kb + 2 * p], b = v[8 * kb + 2 * p + 1];
            split16x2(a.x, b.x, rh[p], rl[p], scale);
            split16x2(a.y, b.y, ih[p], il[p], scale);
        }
        const int k0 = cbase + 8 * kb;
        const int oRe = kmaj_off(a_row(r), k0), oIm = kmaj_off(a_row(r) + 16, k0);  // halves, 16-byte aligned
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
__device__ __forceinline__ void put_B_rows(Smem &S, int s, int r, int cbase, const float2 *v, float scale)
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
            split16x2(a[2 * p].x, a[2 * p + 1].x, rh[p], rl[p], scale);
            split16x2(a[2 * p].y, a[2 * p + 1].y, ih[p], il[p], scale);
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

// load 8 TMEM columns starting at taddr for this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// Epilogue: out[j] = C[r][cbase + j], C = X G the complex product in TMEM
// columns tmem .. tmem+127 (Re G part in the first 64, Im G part in the next
// 64).  Thread t reads lane t & 127, which holds (Re X) G for part p = 0 and
// (Im X) G for p = 1, at all 32 columns of its quarter; it keeps the 16 it
// owns and trades the other 16 with thread t ^ 16 (the other part of the same
// row) by warp shuffles, so no shared memory and no CTA barrier is involved.
// All reads of this accumulator are complete (tcgen05.wait::ld, then
// fence::before_thread_sync) when it returns; the next product into it is
// issued after a CTA barrier.
__device__ void epilogue(uint32_t tmem, float2 *out)
{
    const int t = threadIdx.x;
    const uint32_t lane_addr = tmem + ((uint32_t)(((t >> 5) & 3) * 32) << 16);
    const bool p = ((t >> 4) & 1) != 0;
    const uint32_t q32 = 32u * (uint32_t)(t >> 7);
    float lo[16], hi[16], own_r[16], oth_r[16];
    tmem_ld16(lane_addr + q32, lo);  // Re G part, columns 32 q .. 32 q + 15
    tmem_ld16(lane_addr + q32 + 16, hi);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        own_r[j] = p ? hi[j] : lo[j];
        oth_r[j] = __shfl_xor_sync(0xffffffffu, p ? lo[j] : hi[j], 16);
    }
    tmem_ld16(lane_addr + 64 + q32, lo);  // Im G part
    tmem_ld16(lane_addr + 64 + q32 + 16, hi);
    asm volatile("tcgen05.fence::before_thread_sync;");
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float own_i = p ? hi[j] : lo[j];
        const float oth_i = __shfl_xor_sync(0xffffffffu, p ? lo[j] : hi[j], 16);
        // p = 0: own = (Xr Gr, Xr Gi), other = (Xi Gr, Xi Gi); p = 1: swapped
        const float xrgr = p ? oth_r[j] : own_r[j], xigr = p ? own_r[j] : oth_r[j];
        const float xrgi = p ? oth_i : own_i, xigi = p ? own_i : oth_i;
        out[j] = make_float2(xrgr - xigi, xrgi + xigr);
    }
}

// The products of a pulse sequence with nseg = pulse_num + 1 segments, per
// branch (B0 starts with U0, B1 with U1): an optional leading diagonal
// lead[br] (-1 none, 0 h, 1 f), then n[br] groups (y, d) = Y(y) E0(d) with y in
// {0 h, 1 f} and d in {-1 none, 0 h, 1 f}.  The first group starts the chain
// (registers); every later group is a B operand in slot[br][q], one slot per
// distinct (y, d) (need[y][d + 1]); slot 0 holds M^H.
struct ChainProg {
    int lead[2], n[2], y[2][40], d[2][40], slot[2][40];
    int need[2][3];
};

// thread 0 only; false when the program does not fit the tables or slots
__device__ bool build_chain_prog(ChainProg &P, int nseg)
{
    bool ok = true;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 3; ++b) P.need[a][b] = -1;
    int next_slot = 1;  // slot 0 holds M^H
    for (int br = 0; br < 2; ++br) {
        int j = 0, n = 0;
        P.lead[br] = -1;
        if (((0 + br) & 1) == 0) {  // first factor is U0
            P.lead[br] = 0;         // segment 0 has fraction h
            j = 1;
        }
        while (j < nseg && n < 40) {
            const int y = (j == 0 || j == nseg - 1) ? 0 : 1;
            int d = -1;
            if (j + 1 < nseg) d = (j + 1 == nseg - 1) ? 0 : 1;
            P.y[br][n] = y;
            P.d[br][n] = d;
            ++n;
            j += (d >= 0) ? 2 : 1;
        }
        if (j < nseg) ok = false;  // longer program than the tables
        P.n[br] = n;
    }
    for (int br = 0; br < 2; ++br)
        for (int q = 0; q < P.n[br]; ++q) {
            P.slot[br][q] = -1;
            if (q == 0) continue;  // the first group is the chain's start (A)
            int &sl = P.need[P.y[br][q]][P.d[br][q] + 1];
            if (sl < 0) sl = next_slot++;
            P.slot[br][q] = sl;
        }
    if (next_slot > NSLOT) ok = false;  // more distinct groups than slots
    return ok;
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
    __shared__ ChainProg P;
    Smem S;
    S.A[0] = reinterpret_cast<__half *>(smraw);
    S.A[1] = reinterpret_cast<__half *>(smraw + ABUF_BYTES);
    S.slot = reinterpret_cast<__half *>(smraw + 2 * ABUF_BYTES);
    const int t = threadIdx.x;
    const int r = row_of(t), cb = col_base(t);
    const int nseg = pulse_num + 1;
    if (t == 0) {
        s_abort = build_chain_prog(P, nseg) ? 0 : 2;
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
                    split16(m.x * OP_SCALE, hh, ll);
                    b[o] = hh;
                    b[HALF_OP / 2 + o] = ll;
                    split16(-m.y * OP_SCALE, hh, ll);
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
                        put_A_row(S.A[y], r, cb, v, OP_SCALE);
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
                    epilogue(tmem + (uint32_t)(128 * y), Yv);
                    // groups with this y into their slots; chain starts to registers
#pragma unroll
                    for (int dd = -1; dd <= 1; ++dd) {
                        const int s = P.need[y][dd + 1];
                        if (s < 0) continue;  // uniform: s_need is shared
                        const float2 *e0 = dd == 0 ? e0h : e0f;
                        float2 g[CW];
#pragma unroll
                        for (int j = 0; j < CW; ++j) g[j] = dd < 0 ? Yv[j] : cmulf(Yv[j], e0[cb + j]);
                        put_B_rows(S, s, r, cb, g, OP_UNSCALE);
                    }
#pragma unroll
                    for (int br = 0; br < 2; ++br) {
                        if (P.y[br][0] != y && two) continue;
                        const int dd = P.d[br][0];
#pragma unroll
                        for (int j = 0; j < CW; ++j) {
                            const int c = cb + j;
                            float2 v = dd < 0 ? Yv[j] : cmulf(Yv[j], dd == 0 ? e0h[c] : e0f[c]);
                            if (P.lead[br] >= 0) v = cmulf(P.lead[br] == 0 ? e0h[r] : e0f[r], v);
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
                    if (q[br] < P.n[br]) put_A_row(S.A[br], r, cb, cur[br], OP_UNSCALE);
                asm volatile("fence.proxy.async.shared::cta;");
                __syncthreads();
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int br = 0; br < 2; ++br) {
                    if (q[br] < P.n[br]) {
                        if (t == 0) issue_product(S, S.A[br], P.slot[br][q[br]], tmem + (uint32_t)(128 * br), mb[br]);
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
                        epilogue(tmem + (uint32_t)(128 * br), cur[br]);
                        ++q[br];
                        if (q[br] < P.n[br]) {
                            put_A_row(S.A[br], r, cb, cur[br], OP_UNSCALE);
                            asm volatile("fence.proxy.async.shared::cta;");
                            __syncthreads();
                            asm volatile("tcgen05.fence::after_thread_sync;");
                            if (t == 0) issue_product(S, S.A[br], P.slot[br][q[br]], tmem + (uint32_t)(128 * br), mb[br]);
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

// ---------------------------------------------------------------------------
// Five-spin clusters (D = 32): two time points per product
// ---------------------------------------------------------------------------
// A complex 32 x 32 product is too small for an M = 128 MMA, so every product
// carries two time points h = 0, 1 of one cluster as a block-diagonal
// operand: A row 64 h + r holds Re X_h row r and row 64 h + 32 + r holds Im X_h
// row r, in K columns 32 h .. 32 h + 31 (zeros in the other half, written
// once); B (N = 64: Re G in rows n < 32, Im G in rows 32 + n) holds G_h^T in K
// columns 32 h .. 32 h + 31.  The operands then have the six-spin kernel's
// shapes and layouts (A 128 x 64, B 64 x 64, K-major, no swizzle), a product
// is 12 MMAs (four K slices, three passes) into 64 accumulator columns, and
// lane 64 h + 32 p + r of the accumulator holds row r of
// (p ? Im X_h : Re X_h) [Re G_h | Im G_h].
namespace tc32 {
constexpr int D = 32;
constexpr int XB_STRIDE = 17;                // exchange: 16 floats per thread, padded
constexpr int SLOT_BYTES = 2 * HALF_OP;      // B hi | lo, 8 KB each
constexpr int SMEM_DYN = 2 * ABUF_BYTES + NSLOT * SLOT_BYTES + NT * XB_STRIDE * 4;  // 148480
constexpr int TMEM_COLS = 128;               // two accumulators of 64 columns

// Thread roles (256 threads): warp w reads accumulator lanes 32 (w & 3) ..
// + 31, so thread t stands for time point h = (w >> 1) & 1, part p = w & 1
// (Re or Im row), row r = t & 31, and column half c2 = w >> 2; after the
// exchange it owns the complex entries of row r, columns n0 .. n0 + 7,
// n0 = 16 c2 + 8 p, of time point h's product.
__device__ __forceinline__ int t_h(int t) { return (t >> 6) & 1; }
__device__ __forceinline__ int t_p(int t) { return (t >> 5) & 1; }
__device__ __forceinline__ int t_n0(int t) { return 16 * (t >> 7) + 8 * ((t >> 5) & 1); }

// Row r of time point h's factor, columns n0 .. n0 + 7, into A operand `A`
// (scaled, split hi | lo): one 16-byte core-matrix row per part.
__device__ __forceinline__ void put_A(__half *A, int h, int r, int n0, const float2 *v, float scale)
{
    uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        split16x2(v[2 * q].x, v[2 * q + 1].x, rh[q], rl[q], scale);
        split16x2(v[2 * q].y, v[2 * q + 1].y, ih[q], il[q], scale);
    }
    const int k0 = 32 * h + n0;
    const int oRe = kmaj_off(64 * h + r, k0), oIm = kmaj_off(64 * h + 32 + r, k0);
    *reinterpret_cast<uint4 *>(A + oRe) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
    *reinterpret_cast<uint4 *>(A + OP_BYTES / 2 + oRe) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
    *reinterpret_cast<uint4 *>(A + oIm) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
    *reinterpret_cast<uint4 *>(A + OP_BYTES / 2 + oIm) = make_uint4(il[0], il[1], il[2], il[3]);
}

// Entries G_h[r][n0 + j] (j < 8) of a group operand into slot `b`, transposed
// (B[n][k = 32 h + r]): the eight lanes holding rows r0 .. r0 + 7 transpose
// their 8 x 8 block with a three-stage shuffle butterfly, after which lane i
// holds column n0 + i for rows r0 .. r0 + 7, one 16-byte row per part.
__device__ __forceinline__ void put_B(__half *b, int h, int r, int n0, const float2 *v, float scale)
{
    const int lane8 = threadIdx.x & 7;
    const int r0 = r & ~7;
    float2 a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = v[k];
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
    // a[k] = G_h[r0 + k][n0 + lane8]
    uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        split16x2(a[2 * q].x, a[2 * q + 1].x, rh[q], rl[q], scale);
        split16x2(a[2 * q].y, a[2 * q + 1].y, ih[q], il[q], scale);
    }
    const int oRe = kmaj_off(n0 + lane8, 32 * h + r0), oIm = kmaj_off(32 + n0 + lane8, 32 * h + r0);
    *reinterpret_cast<uint4 *>(b + oRe) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
    *reinterpret_cast<uint4 *>(b + HALF_OP / 2 + oRe) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
    *reinterpret_cast<uint4 *>(b + oIm) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
    *reinterpret_cast<uint4 *>(b + HALF_OP / 2 + oIm) = make_uint4(il[0], il[1], il[2], il[3]);
}

// one block-diagonal product A x slot -> TMEM columns tmem .. tmem + 63
// (issued by thread 0), completion signalled on mbar
__device__ __forceinline__ void issue(const __half *A, const __half *slot, uint32_t tmem, uint32_t mbar)
{
    const uint32_t a0 = smem_u32(A), b0 = smem_u32(slot);
    // passes: (A hi, B hi), (A hi, B lo), (A lo, B hi)
    const uint32_t aoff[3] = {0u, 0u, (uint32_t)OP_BYTES};
    const uint32_t boff[3] = {0u, (uint32_t)HALF_OP, 0u};
    for (int p = 0; p < 3; ++p)
        for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = sdesc(a0 + aoff[p] + (uint32_t)kk * 256u);
            const uint64_t bd = sdesc(b0 + boff[p] + (uint32_t)kk * 256u);
            const uint32_t acc = (p > 0 || kk > 0) ? 1u : 0u;
            asm volatile("{\n.reg .pred q;\nsetp.ne.u32 q, %4, 0;\n"
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}" ::"r"(tmem),
                         "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
        }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

// Epilogue: out[j] = C_h[r][n0 + j] from the accumulator at tmem (64 columns).
// Thread t holds its row kind (p) times [Re G | Im G] at columns 16 c2 ..
// 16 c2 + 15; it keeps 8 of them and swaps the other 8 with thread t ^ 32
// (the other row kind, same row and columns) through XB.  All reads of the
// accumulator are complete when it returns.
__device__ void epilogue(float *XB, uint32_t tmem, float2 *out)
{
    const int t = threadIdx.x;
    const int warp = t >> 5;
    const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const int p = t_p(t);
    const int col0 = 16 * (t >> 7);
    const uint32_t give = (uint32_t)(col0 + 8 * (1 - p)), keep = (uint32_t)(col0 + 8 * p);
    {
        float gr[8], gi[8];
        tmem_ld8(lane_addr + give, gr);
        tmem_ld8(lane_addr + 32 + give, gi);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            XB[t * XB_STRIDE + 2 * j] = gr[j];
            XB[t * XB_STRIDE + 2 * j + 1] = gi[j];
        }
    }
    __syncthreads();
    float kr[8], ki[8];
    tmem_ld8(lane_addr + keep, kr);
    tmem_ld8(lane_addr + 32 + keep, ki);
    asm volatile("tcgen05.fence::before_thread_sync;");
    const int pt = t ^ 32;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float pr = XB[pt * XB_STRIDE + 2 * j], pi = XB[pt * XB_STRIDE + 2 * j + 1];
        // p = 0: own = (Xr Gr, Xr Gi), partner = (Xi Gr, Xi Gi); p = 1: swapped
        const float xrgr = p == 0 ? kr[j] : pr;
        const float xrgi = p == 0 ? ki[j] : pi;
        const float xigr = p == 0 ? pr : kr[j];
        const float xigi = p == 0 ? pi : ki[j];
        out[j] = make_float2(xrgr - xigi, xrgi + xigr);
    }
    __syncthreads();  // exchange reads done: XB may be rewritten
}
}  // namespace tc32

__global__ void __launch_bounds__(NT, 1)
k_coherence_tc32(const unsigned long long *__restrict__ phi, const float2 *__restrict__ Mg, int ncl,
                 int pulse_num, int nT, int tslices, double *__restrict__ L, int *__restrict__ queue,
                 int *__restrict__ status)
{
    using namespace tc32;
    constexpr int DD = tc32::D;
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_item, s_abort;
    __shared__ float2 e0h[2][DD], e0f[2][DD], e1h[2][DD], e1f[2][DD];  // per time point h
    __shared__ unsigned long long phs[4 * DD];  // phase steps [branch][h, f][d]
    __shared__ float red[3][NT / 32];
    __shared__ ChainProg P;
    __half *Aop[2] = {reinterpret_cast<__half *>(smraw), reinterpret_cast<__half *>(smraw + ABUF_BYTES)};
    __half *slots = reinterpret_cast<__half *>(smraw + 2 * ABUF_BYTES);
    float *XB = reinterpret_cast<float *>(smraw + 2 * ABUF_BYTES + NSLOT * tc32::SLOT_BYTES);
    const int t = threadIdx.x;
    const int h = t_h(t), r = t & 31, n0 = t_n0(t);
    const int nseg = pulse_num + 1;
    // the A operands' off-diagonal K halves stay zero: nothing else writes them
    for (int e = t; e < 2 * ABUF_BYTES / 16; e += NT) reinterpret_cast<uint4 *>(smraw)[e] = make_uint4(0, 0, 0, 0);
    if (t == 0) {
        s_abort = build_chain_prog(P, nseg) ? 0 : 2;
        for (int b = 0; b < 2; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[b])));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "n"(tc32::TMEM_COLS));
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
            const float2 *M = Mg + (size_t)cl * DD * DD;  // FP32 copy of M
            if (cl != cur_cl) {
                cur_cl = cl;
                for (int e = t; e < 4 * DD; e += NT) phs[e] = phi[(size_t)cl * 4 * DD + e];
                // slot 0: M^H in both K halves, B[n][k] = conj(M[n][k mod 32])
                __half *b = slots;
                for (int e = t; e < DD * DD; e += NT) {
                    const int n = e % DD, k = e / DD;  // M column-major: M[n][k] = Mg[n + D k]
                    const float2 m = M[n + (size_t)DD * k];
                    __half rh, rl, ih, il;
                    split16(m.x * OP_SCALE, rh, rl);
                    split16(-m.y * OP_SCALE, ih, il);
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh) {
                        const int o = kmaj_off(n, 32 * hh + k), o2 = kmaj_off(32 + n, 32 * hh + k);
                        b[o] = rh;
                        b[HALF_OP / 2 + o] = rl;
                        b[o2] = ih;
                        b[HALF_OP / 2 + o2] = il;
                    }
                }
            }
            int i0 = sl * per;
            const int i1 = min(nT, i0 + per);
            if (i0 == 0) {
                if (t == 0 && i1 > 0) L[(size_t)cl * nT] = 1.0;
                i0 = 1;
            }
            for (int i = i0; i < i1 && !s_abort; i += 2) {
                const bool pair = i + 1 < i1;  // else time point h = 1 repeats i, unwritten
                __syncthreads();
                if (t < 2 * DD) {
                    const int hh = t >> 5, d = t & 31;
                    const int ti = i + (hh && pair ? 1 : 0);
                    e0h[hh][d] = phase_step_f(phs[d], ti);
                    e0f[hh][d] = phase_step_f(phs[DD + d], ti);
                    e1h[hh][d] = phase_step_f(phs[2 * DD + d], ti);
                    e1f[hh][d] = phase_step_f(phs[3 * DD + d], ti);
                }
                __syncthreads();
                float2 cur[2][8];  // the two chains: row r, columns n0 .. n0 + 7 of time point h
                // ---- Y(h) (A operand 0) and Y(f) (A operand 1) for both time points
                {
                    float2 v[8];
#pragma unroll
                    for (int y = 0; y < 2; ++y) {
                        if (y == 1 && !two) break;
                        const float2 *e1 = y == 0 ? e1h[h] : e1f[h];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int k = n0 + j;
                            v[j] = cmulf(M[r + (size_t)DD * k], e1[k]);
                        }
                        put_A(Aop[y], h, r, n0, v, OP_SCALE);
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;");
                __syncthreads();
                asm volatile("tcgen05.fence::after_thread_sync;");
                if (t == 0) {
                    tc32::issue(Aop[0], slots, tmem, mb[0]);
                    if (two) tc32::issue(Aop[1], slots, tmem + 64, mb[1]);
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
                    float2 Yv[8];
                    tc32::epilogue(XB, tmem + (uint32_t)(64 * y), Yv);
                    // groups with this y into their slots; chain starts to registers
#pragma unroll
                    for (int dd = -1; dd <= 1; ++dd) {
                        const int s = P.need[y][dd + 1];
                        if (s < 0) continue;  // uniform: P is shared
                        const float2 *e0 = dd == 0 ? e0h[h] : e0f[h];
                        float2 g[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) g[j] = dd < 0 ? Yv[j] : cmulf(Yv[j], e0[n0 + j]);
                        put_B(slots + (size_t)s * (tc32::SLOT_BYTES / 2), h, r, n0, g, OP_UNSCALE);
                    }
#pragma unroll
                    for (int br = 0; br < 2; ++br) {
                        if (P.y[br][0] != y && two) continue;
                        const int dd = P.d[br][0];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int c = n0 + j;
                            float2 v = dd < 0 ? Yv[j] : cmulf(Yv[j], dd == 0 ? e0h[h][c] : e0f[h][c]);
                            if (P.lead[br] >= 0) v = cmulf(P.lead[br] == 0 ? e0h[h][r] : e0f[h][r], v);
                            cur[br][j] = v;
                        }
                    }
                }
                if (s_abort) break;
                // ---- the two chains, pipelined as in the six-spin kernel
                int q[2] = {1, 1};
#pragma unroll
                for (int br = 0; br < 2; ++br)
                    if (q[br] < P.n[br]) put_A(Aop[br], h, r, n0, cur[br], OP_UNSCALE);
                asm volatile("fence.proxy.async.shared::cta;");
                __syncthreads();
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int br = 0; br < 2; ++br) {
                    if (q[br] < P.n[br]) {
                        if (t == 0)
                            tc32::issue(Aop[br], slots + (size_t)P.slot[br][q[br]] * (tc32::SLOT_BYTES / 2),
                                        tmem + (uint32_t)(64 * br), mb[br]);
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
                        tc32::epilogue(XB, tmem + (uint32_t)(64 * br), cur[br]);
                        ++q[br];
                        if (q[br] < P.n[br]) {
                            put_A(Aop[br], h, r, n0, cur[br], OP_UNSCALE);
                            asm volatile("fence.proxy.async.shared::cta;");
                            __syncthreads();
                            asm volatile("tcgen05.fence::after_thread_sync;");
                            if (t == 0)
                                tc32::issue(Aop[br], slots + (size_t)P.slot[br][q[br]] * (tc32::SLOT_BYTES / 2),
                                            tmem + (uint32_t)(64 * br), mb[br]);
                            inflight[br] = true;
                        }
                    }
                    if (s_abort) break;
                }
                if (s_abort) break;
                // trace sums per time point in FP32 (warps 0, 1, 4, 5: h = 0)
                float fr = 0.f, f0 = 0.f, f1 = 0.f;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
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
                if (t < 2 && (t == 0 || pair)) {
                    float sum = 0, s0 = 0, s1 = 0;
                    for (int w = 0; w < NT / 32; ++w) {
                        if (((w >> 1) & 1) != t) continue;
                        sum += red[0][w];
                        s0 += red[1][w];
                        s1 += red[2][w];
                    }
                    // the defect in FP32, 1 - x in FP64
                    L[(size_t)cl * nT + i + t] = 1.0 - (double)coherence_defect_f(s0, s1, sum);
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
    if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(tc32::TMEM_COLS));
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

// Launch the tensor-core coherence for ncl five-spin clusters (as
// oops_coherence_tc64: phi 4*32 phase steps and M 32x32 FP32 overlaps per
// cluster; each CTA runs two time points per product).
int oops_coherence_tc32(const unsigned long long *phi, const float2 *M, int ncl, int pulse_num,
                        int nT, double *L, int *queue, int *status, int tslice_mult, cudaStream_t st)
{
    if (!oops_tc64_supported(pulse_num))
        return oops_set_status(OOPS_ERR_UNSUPPORTED, "tensor-core path: Hahn or even CPMG only");
    const int sms = oops_sm_count();
    const int tslices = std::max(1, std::min(nT, (sms * std::max(1, tslice_mult) + ncl - 1) / std::max(1, ncl)));
    const int grid = std::max(1, std::min(ncl * tslices, sms));
    cudaFuncSetAttribute(k_coherence_tc32, cudaFuncAttributeMaxDynamicSharedMemorySize, tc32::SMEM_DYN);
    k_coherence_tc32<<<grid, NT, tc32::SMEM_DYN, st>>>(phi, M, ncl, pulse_num, nT, tslices, L, queue, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    return OOPS_OK;
}
