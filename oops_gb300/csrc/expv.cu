// expv.cu -- device-resident Krylov expv for a block of state vectors.
//
// Restates the algorithm of the reference's GPU driver ZGEXPV_CACHE
// (src/expv/source/zgexpv_cache.f:226-690) and its CPU twin
// HAMVEC_ZGEXPV_W_MKL_PROFILE (src/expv/source/hamvec_zgexpv_w_mkl_profile.f:
// 186-538): a k-step Lanczos + power-iteration estimate of ||H||, then
// Arnoldi with the corrected (m+2) scheme, an irreducible Pade(6,6)
// exponential of the Hessenberg matrix (ZGPADM, expokit.f:762-933), the local
// error estimate, step rejection (delta 1.2, gamma 0.9) and outputs at every
// requested time.  Differences from the reference, by design:
//   - nothing crosses PCIe per matvec (the reference copies v to the device
//     and w back around every matvec, zgexpv_cache.f:470-479);
//   - orthogonalisation is classical Gram-Schmidt applied twice (CGS2), with
//     the dot products of one pass fused into one kernel and reduced with warp
//     shuffles; the reference runs modified Gram-Schmidt with host BLAS;
//   - every column of the block carries its own step control (the columns
//     share the Arnoldi matvec launches);
//   - sgn = +1 and the norm-estimate seed restarts at (0,0,0,5) each call
//     (the Fortran reads an uninitialised t and SAVEs the seed);
//   - a zero Hamiltonian or a zero column returns the input unchanged instead
//     of dividing by zero; step rejection and power iteration are capped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "oops_common.cuh"
#include "oops_internal.h"

namespace {

constexpr int RED_THREADS = 256;
constexpr int DOT_CHUNK = 8;
constexpr double BREAK_TOL = 1.0e-7;
constexpr double DELTA = 1.2, GAMMA = 0.9;
constexpr int MAX_REJECT = 10000;

struct VState {
    double t_now, t_new, t_step, beta, vnorm, hump, xm, err_loc, s_error, x_error;
    double step_min, step_max, tbrkdwn, avnorm, inv;
    int k1, mbrkdwn, tt, out_first, out_last, status;
    long nstep, nexph, nscale, nreject, nmult, ibrkflag;
};

// ---------------------------------------------------------------- scalar math
__host__ __device__ inline double f_nint(double x)
{
    return x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5);
}
__host__ __device__ inline double f_aint(double x) { return x >= 0 ? floor(x) : -floor(-x); }
__host__ __device__ inline double f_pow10i(int e)
{
    double r = 1.0, b = 10.0;
    int a = e < 0 ? -e : e;
    while (a) {
        if (a & 1) r *= b;
        b *= b;
        a >>= 1;
    }
    return e < 0 ? 1.0 / r : r;
}
// zgexpv: p1 = 10**(NINT(LOG10(t)-SQR1)-1); t = AINT(t/p1+0.55)*p1
__host__ __device__ inline double round_step(double t)
{
    const double sqr1 = sqrt(0.1);
    double p1 = f_pow10i((int)f_nint(log10(t) - sqr1) - 1);
    return f_aint(t / p1 + 0.55) * p1;
}

// ---------------------------------------------------------------- reductions
// partial[(chunk*nblk + blk)*DOT_CHUNK*P + i*P + b] = sum over this block's rows
// of conj(basis_{i0+i}[x,b]) * y[x,b]
__global__ void __launch_bounds__(RED_THREADS)
k_dots(const zd *__restrict__ basis, size_t bstride, int nbasis, const zd *__restrict__ y,
       size_t N, int plog, zd *__restrict__ partial)
{
    const int P = 1 << plog;
    const int tid = threadIdx.x;
    const int b = tid & (P - 1);
    const int R = RED_THREADS >> plog;  // rows per block iteration
    const int chunk = blockIdx.y;
    const int i0 = chunk * DOT_CHUNK;
    const int ni = min(DOT_CHUNK, nbasis - i0);
    zd acc[DOT_CHUNK];
#pragma unroll
    for (int i = 0; i < DOT_CHUNK; ++i) acc[i] = zmake(0, 0);
    for (size_t row = (size_t)blockIdx.x * R + (tid >> plog); row < N;
         row += (size_t)gridDim.x * R) {
        const size_t e = (row << plog) | b;
        const zd yv = __ldg(&y[e]);
#pragma unroll
        for (int i = 0; i < DOT_CHUNK; ++i)
            if (i < ni) {
                const zd a = __ldg(&basis[(size_t)(i0 + i) * bstride + e]);
                acc[i].x = fma(a.x, yv.x, acc[i].x);
                acc[i].x = fma(a.y, yv.y, acc[i].x);
                acc[i].y = fma(a.x, yv.y, acc[i].y);
                acc[i].y = fma(-a.y, yv.x, acc[i].y);
            }
    }
    __shared__ zd sh[RED_THREADS];
    zd *out = partial + ((size_t)chunk * gridDim.x + blockIdx.x) * DOT_CHUNK * P;
    for (int i = 0; i < ni; ++i) {
        zd v = acc[i];
        // lanes holding the same column are P apart: shuffle within a warp,
        // then through shared memory across warps
        for (int off = 16; off >= P; off >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, off);
            v.y += __shfl_down_sync(0xffffffffu, v.y, off);
        }
        __syncthreads();
        sh[tid] = v;
        __syncthreads();
        if (P >= 32) {
            for (int s = RED_THREADS / 2; s >= P; s >>= 1) {
                if (tid < s) sh[tid] = zadd(sh[tid], sh[tid + s]);
                __syncthreads();
            }
            if (tid < P) out[i * P + tid] = sh[tid];
        } else {
            // one partial per warp (lanes 0..P-1 of each warp)
            if (tid < P) {
                zd s = zmake(0, 0);
                for (int w = 0; w < RED_THREADS / 32; ++w) s = zadd(s, sh[w * 32 + tid]);
                out[i * P + tid] = s;
            }
        }
    }
}

// out[b*ld + i0 + i] (+)= sum_blk partial
__global__ void k_dots_final(const zd *__restrict__ partial, int nblk, int nbasis, int plog,
                             int nvec, zd *__restrict__ out, int ld, int accumulate)
{
    const int P = 1 << plog;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nbasis * P) return;
    int i = q / P, b = q % P;
    if (b >= nvec) return;
    int chunk = i / DOT_CHUNK, ii = i % DOT_CHUNK;
    zd s = zmake(0, 0);
    for (int k = 0; k < nblk; ++k)
        s = zadd(s, partial[((size_t)chunk * nblk + k) * DOT_CHUNK * P + ii * P + b]);
    if (accumulate) out[b * ld + i] = zadd(out[b * ld + i], s);
    else out[b * ld + i] = s;
}

// y[x,b] -= sum_i coef[b*ld + i] * basis_i[x,b]
__global__ void __launch_bounds__(256)
k_subtract(const zd *__restrict__ basis, size_t bstride, int nbasis, const zd *__restrict__ coef,
           int ld, zd *__restrict__ y, size_t N, int plog, int nvec, const int *__restrict__ live)
{
    const size_t total = N << plog;
    const int P = 1 << plog;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e & (P - 1));
        if (b >= nvec || !live[b]) continue;
        zd v = y[e];
        for (int i = 0; i < nbasis; ++i) {
            zd c = coef[b * ld + i];
            zd a = __ldg(&basis[(size_t)i * bstride + e]);
            v.x -= c.x * a.x - c.y * a.y;
            v.y -= c.x * a.y + c.y * a.x;
        }
        y[e] = v;
    }
}

// y[x,b] *= s[b]  (only live columns)
__global__ void k_scale(zd *__restrict__ y, size_t N, int plog, int nvec,
                        const double *__restrict__ s, const int *__restrict__ live)
{
    const size_t total = N << plog;
    const int P = 1 << plog;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e & (P - 1));
        if (b >= nvec || !live[b]) continue;
        y[e] = zscale(y[e], s[b]);
    }
}

// ---------------------------------------------------------------- Lanczos
__host__ __device__ inline uint64_t mulmod48(uint64_t a, uint64_t b)
{
    return (a * b) & ((1ULL << 48) - 1);
}
__host__ __device__ inline double dlaran_draw(uint64_t n)
{
    // value of the n-th DLARAN call (1-based) from seed (0,0,0,5)
    uint64_t r = 1, base = 33952834046453ULL;
    while (n) {
        if (n & 1) r = mulmod48(r, base);
        base = mulmod48(base, base);
        n >>= 1;
    }
    return (double)mulmod48(r, 5) * 0x1p-48;
}

__global__ void k_dlaran_vec(zd *q, size_t N)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x)
        q[i] = zmake(dlaran_draw(2 * i + 1), dlaran_draw(2 * i + 2));
}

struct LState {
    double T[64 * 64];
    double bj, bjm, anorm;
    zd aj;
    double nrm2;  // reduction target
    int done, k;
};

// q *= 1/sqrt(nrm2) (first normalisation)
__global__ void k_lanczos_norm0(zd *q, size_t N, LState *ls)
{
    double inv = 1.0 / sqrt(ls->nrm2);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x)
        q[i] = zscale(q[i], inv);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ls->bj = sqrt(ls->nrm2);
        ls->bjm = 0.0;
    }
}

// w -= aj q + bjm qm
__global__ void k_lanczos_axpy(zd *w, const zd *q, const zd *qm, size_t N, const LState *ls)
{
    if (ls->done) return;
    zd aj = ls->aj;
    double bjm = ls->bjm;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
        zd v = zsub(w[i], zmul(aj, q[i]));
        w[i] = zsub(v, zscale(qm[i], bjm));
    }
}

// record T entries of step j (1-based) and decide whether to stop
__global__ void k_lanczos_post(LState *ls, int j, double tol)
{
    if (ls->done) return;
    const int k = ls->k;
    ls->T[(j - 1) * k + (j - 1)] = ls->aj.x;
    ls->bj = sqrt(ls->nrm2);
    if (j == k) { ls->done = 1; return; }
    ls->T[(j - 1) * k + j] = ls->bj;
    ls->T[j * k + (j - 1)] = ls->bj;
    if (ls->bj < tol) ls->done = 1;
}

// qm = q; q = w / bj; bjm = bj (only while running)
__global__ void k_lanczos_shift(zd *q, zd *qm, const zd *w, size_t N, LState *ls, int last)
{
    if (ls->done) return;
    double inv = 1.0 / ls->bj;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
        qm[i] = q[i];
        q[i] = zscale(w[i], inv);
    }
    (void)last;
}

__global__ void k_lanczos_bjm(LState *ls)
{
    if (!ls->done) ls->bjm = ls->bj;
}

// ---------------------------------------------------------------- step control
__global__ void k_init(VState *st, int nvec, const double *__restrict__ nrm2, int m, double tol,
                       const LState *ls, const double *__restrict__ ta, int tn,
                       int *__restrict__ act)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec) return;
    VState s;
    memset(&s, 0, sizeof(s));
    s.k1 = 2;
    s.mbrkdwn = m;
    s.beta = sqrt(nrm2[b]);
    s.vnorm = s.beta;
    s.hump = s.beta;
    s.step_min = INFINITY;
    s.xm = 1.0 / (double)m;
    const double anorm = ls->anorm;
    double p2 = tol * pow((double)(m + 1) / 2.72, (double)(m + 1)) * sqrt(2.0 * 3.14 * (double)(m + 1));
    s.t_new = round_step((1.0 / anorm) * pow(p2 / (4.0 * s.beta * anorm), s.xm));
    int tt = 0;
    while (tt < tn && s.t_now >= ta[(size_t)b * tn + tt]) ++tt;
    s.out_first = 0;
    s.out_last = tt;
    // a zero column or a zero Hamiltonian: the solution is constant
    bool trivial = !(s.beta > 0.0) || !(anorm > 0.0);
    if (trivial) {
        s.out_last = tn;
        tt = tn;
    }
    s.tt = tt;
    act[b] = tt < tn;
    st[b] = s;
}

__global__ void k_step_begin(VState *st, int nvec, const double *__restrict__ ta, int tn,
                             const int *__restrict__ act, int *__restrict__ live,
                             double *__restrict__ inv, zd *__restrict__ Hm, int mh)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec) return;
    VState &s = st[b];
    live[b] = act[b];
    s.out_first = s.out_last = 0;
    if (!act[b]) return;
    s.nstep++;
    double t_out = ta[(size_t)b * tn + s.tt];
    s.t_step = fmin(t_out - s.t_now, s.t_new);
    inv[b] = 1.0 / s.beta;
    for (int q = 0; q < mh * mh; ++q) Hm[(size_t)b * mh * mh + q] = zmake(0, 0);
}

// after orthogonalisation of column j+1 (0-based j): breakdown test, store
// H(j+1, j) and the normalisation factor
__global__ void k_arnoldi_post(VState *st, int nvec, int j, const double *__restrict__ nrm2,
                               const zd *__restrict__ h1, const zd *__restrict__ h2,
                               int *__restrict__ live,
                               double *__restrict__ inv, zd *__restrict__ Hm, int mh,
                               const double *__restrict__ ta, int tn)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec || !live[b]) return;
    VState &s = st[b];
    s.nmult++;
    zd *H = Hm + (size_t)b * mh * mh;
    for (int i = 0; i <= j; ++i)
        H[i + (size_t)j * mh] = zadd(h1[(size_t)b * mh + i], h2[(size_t)b * mh + i]);
    double hj1j = sqrt(nrm2[b]);
    if (hj1j <= BREAK_TOL) {  // happy breakdown
        s.k1 = 0;
        s.ibrkflag = 1;
        s.mbrkdwn = j + 1;
        s.tbrkdwn = s.t_now;
        s.t_step = ta[(size_t)b * tn + s.tt] - s.t_now;
        live[b] = 0;
        return;
    }
    H[(j + 1) + (size_t)j * mh] = zmake(hj1j, 0.0);
    inv[b] = 1.0 / hj1j;
}

// columns that completed m Arnoldi steps need one more matvec (avnorm)
__global__ void k_avnorm_live(const VState *st, int nvec, const int *act, int *live)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec) return;
    live[b] = act[b] && st[b].k1 != 0;
}

__global__ void k_avnorm_post(VState *st, int nvec, const double *nrm2, const int *live)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec || !live[b]) return;
    st[b].nmult++;
    st[b].avnorm = sqrt(nrm2[b]);
}

// ---------------------------------------------------------------- Pade (one CTA per column)
__device__ void cta_gemm(int n, zd alpha, const zd *A, const zd *B, zd *C)
{
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int r = e % n, c = e / n;
        zd acc = zmake(0, 0);
        for (int l = 0; l < n; ++l) zfma(acc, A[r + n * l], B[l + n * c]);
        C[e] = zmul(alpha, acc);
    }
    __syncthreads();
}

__device__ inline double cabs1(zd z) { return fabs(z.x) + fabs(z.y); }

// exp(t*H) for the n x n matrix in Hs (ld n); result pointer returned.  Uses
// the four n*n buffers starting at buf (Hs must not be one of them).
__device__ zd *cta_padm(int n, double t, const zd *Hs, zd *buf, int *ns_out, int *fail)
{
    const int ideg = 6;
    const int nn = n * n;
    zd *H2 = buf, *P = buf + nn, *Q = buf + 2 * nn, *T = buf + 3 * nn;
    __shared__ double red[256];
    __shared__ double s_hnorm;
    __shared__ int s_piv;
    // infinity norm
    double rmax = 0.0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < n; ++c) s += zabs(Hs[r + n * c]);
        rmax = fmax(rmax, s);
    }
    red[threadIdx.x] = rmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;
        for (int q = 0; q < (int)blockDim.x; ++q) m = fmax(m, red[q]);
        s_hnorm = fabs(t * m);
    }
    __syncthreads();
    double hnorm = s_hnorm;
    if (hnorm == 0.0) {
        *fail = 1;
        return nullptr;
    }
    int ns = (int)(log(hnorm) / log(2.0)) + 2;
    if (ns < 0) ns = 0;
    double scale = t / ldexp(1.0, ns);
    double c[8];
    c[0] = 1.0;
    for (int k = 1; k <= ideg; ++k)
        c[k] = c[k - 1] * (double)(ideg + 1 - k) / (double)(k * (2 * ideg + 1 - k));
    cta_gemm(n, zmake(scale * scale, 0), Hs, Hs, H2);
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        bool dg = (e % n) == (e / n);
        P[e] = zmake(dg ? c[ideg - 1] : 0.0, 0);
        Q[e] = zmake(dg ? c[ideg] : 0.0, 0);
    }
    __syncthreads();
    bool q_turn = true;
    for (int k = ideg - 1; k > 0; --k) {
        zd *X = q_turn ? Q : P;
        cta_gemm(n, zmake(1, 0), X, H2, T);
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
            zd v = T[e];
            if ((e % n) == (e / n)) v.x += c[k - 1];
            X[e] = v;
        }
        __syncthreads();
        q_turn = !q_turn;
    }
    zd *odd = q_turn ? Q : P;
    zd *even = q_turn ? P : Q;
    cta_gemm(n, zmake(scale, 0), odd, Hs, T);
    // even <- even - odd (denominator), odd <- T (numerator part)
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        odd[e] = T[e];
        even[e] = zsub(even[e], T[e]);
    }
    __syncthreads();
    // solve even * X = odd, partial pivoting on |re|+|im|
    for (int j = 0; j < n; ++j) {
        if (threadIdx.x == 0) {
            int p = j;
            double best = cabs1(even[j + n * j]);
            for (int i = j + 1; i < n; ++i) {
                double v = cabs1(even[i + n * j]);
                if (v > best) { best = v; p = i; }
            }
            s_piv = (best == 0.0) ? -1 : p;
        }
        __syncthreads();
        int p = s_piv;
        if (p < 0) {
            *fail = 2;
            return nullptr;
        }
        if (p != j)
            for (int cc = threadIdx.x; cc < 2 * n; cc += blockDim.x) {
                zd *M = cc < n ? even : odd;
                int col = cc < n ? cc : cc - n;
                zd tmp = M[j + n * col];
                M[j + n * col] = M[p + n * col];
                M[p + n * col] = tmp;
            }
        __syncthreads();
        // multipliers into column j of even (below diagonal)
        zd piv = even[j + n * j];
        double den = piv.x * piv.x + piv.y * piv.y;
        zd inv = zmake(piv.x / den, -piv.y / den);
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x)
            even[i + n * j] = zmul(even[i + n * j], inv);
        __syncthreads();
        // trailing update of even (cols > j) and of all rhs columns
        int rows = n - j - 1;
        int cols = (n - j - 1) + n;
        for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
            int i = j + 1 + e % rows;
            int cc = e / rows;
            zd l = even[i + n * j];
            if (cc < n - j - 1) {
                int col = j + 1 + cc;
                even[i + n * col] = zsub(even[i + n * col], zmul(l, even[j + n * col]));
            } else {
                int col = cc - (n - j - 1);
                odd[i + n * col] = zsub(odd[i + n * col], zmul(l, odd[j + n * col]));
            }
        }
        __syncthreads();
    }
    // back substitution, one rhs column per thread
    for (int col = threadIdx.x; col < n; col += blockDim.x) {
        zd *bcol = odd + n * col;
        for (int j = n - 1; j >= 0; --j) {
            zd u = even[j + n * j];
            double den = u.x * u.x + u.y * u.y;
            zd v = bcol[j];
            v = zmake((v.x * u.x + v.y * u.y) / den, (v.y * u.x - v.x * u.y) / den);
            bcol[j] = v;
            for (int i = 0; i < j; ++i) bcol[i] = zsub(bcol[i], zmul(even[i + n * j], v));
        }
    }
    __syncthreads();
    // r = I + 2X
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        zd v = zscale(odd[e], 2.0);
        if ((e % n) == (e / n)) v.x += 1.0;
        odd[e] = v;
    }
    __syncthreads();
    zd *cur = odd, *nxt = T;
    for (int s = 0; s < ns; ++s) {
        cta_gemm(n, zmake(1, 0), cur, cur, nxt);
        zd *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    *ns_out = ns;
    return cur;
}

__global__ void __launch_bounds__(256)
k_padm(VState *st, int nvec, const int *__restrict__ act, const zd *__restrict__ Hm, int mh, int m,
       double tol, zd *__restrict__ Ecol)
{
    const int b = blockIdx.x;
    if (b >= nvec || !act[b]) return;
    extern __shared__ zd smem[];
    VState &s = st[b];
    const int mx = s.mbrkdwn + s.k1;
    zd *Hs = smem;
    zd *buf = smem + mx * mx;
    const zd *Hg = Hm + (size_t)b * mh * mh;
    for (int e = threadIdx.x; e < mx * mx; e += blockDim.x) {
        int r = e % mx, c = e / mx;
        zd v = Hg[r + (size_t)mh * c];
        if (s.k1 != 0 && r == m + 1 && c == m) v = zmake(1.0, 0.0);  // corrected scheme
        Hs[e] = v;
    }
    __syncthreads();
    __shared__ int s_reject, s_fail;
    __shared__ double s_tstep;
    if (threadIdx.x == 0) {
        s_fail = 0;
        s_tstep = s.t_step;
    }
    __syncthreads();
    int ireject = 0;
    for (;;) {
        int ns = 0, fail = 0;
        zd *E = cta_padm(mx, s_tstep, Hs, buf, &ns, &fail);
        if (fail) {
            if (threadIdx.x == 0) {
                s.status = OOPS_ERR_NUMERIC;
                s_fail = 1;
            }
            __syncthreads();
            break;
        }
        if (threadIdx.x == 0) {
            s.nexph++;
            s.nscale += ns;
            double err;
            if (s.k1 == 0) {
                err = tol;
            } else {
                double q1 = zabs(E[m]) * s.beta;
                double q2 = zabs(E[m + 1]) * s.beta * s.avnorm;
                if (q1 > 10.0 * q2) { err = q2; s.xm = 1.0 / (double)m; }
                else if (q1 > q2) { err = (q1 * q2) / (q1 - q2); s.xm = 1.0 / (double)m; }
                else { err = q1; s.xm = 1.0 / (double)(m - 1); }
            }
            s.err_loc = err;
            s_reject = 0;
            double ts = s_tstep;
            if (s.k1 != 0 && err > DELTA * ts * tol) {
                ts = GAMMA * ts * pow(ts * tol / err, s.xm);
                ts = round_step(ts);
                s.nreject++;
                s_reject = 1;
                if (ireject + 1 > MAX_REJECT || !(ts > 0.0)) {
                    s.status = OOPS_ERR_NUMERIC;
                    s_fail = 1;
                    s_reject = 0;
                }
                s_tstep = ts;
            }
        }
        __syncthreads();
        if (s_fail) break;
        if (!s_reject) {
            for (int r = threadIdx.x; r < mx; r += blockDim.x) Ecol[(size_t)b * mh + r] = E[r];
            break;
        }
        ++ireject;
        __syncthreads();
    }
    if (threadIdx.x == 0) s.t_step = s_tstep;
}

// w[x,b] = beta_b * sum_{c<mx} V_c[x,b] E_b[c]
__global__ void __launch_bounds__(256)
k_update_w(const zd *__restrict__ basis, size_t bstride, const zd *__restrict__ Ecol, int mh,
           const VState *__restrict__ st, const int *__restrict__ act, zd *__restrict__ w,
           size_t N, int plog, int nvec)
{
    const size_t total = N << plog;
    const int P = 1 << plog;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e & (P - 1));
        if (b >= nvec || !act[b] || st[b].status) continue;
        const int mx = st[b].mbrkdwn + max(0, st[b].k1 - 1);
        zd acc = zmake(0, 0);
        for (int c = 0; c < mx; ++c) zfma(acc, __ldg(&basis[(size_t)c * bstride + e]), Ecol[(size_t)b * mh + c]);
        w[e] = zscale(acc, st[b].beta);
    }
}

__global__ void k_step_end(VState *st, int nvec, const double *__restrict__ nrm2, double tol,
                           double rndoff, const double *__restrict__ ta, int tn,
                           int *__restrict__ act, int *__restrict__ nactive)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nvec) return;
    VState &s = st[b];
    if (!act[b]) return;
    if (s.status) {
        act[b] = 0;
        return;
    }
    s.beta = sqrt(nrm2[b]);
    s.hump = fmax(s.hump, s.beta);
    double ts = s.t_step;
    double tnew = GAMMA * ts * pow(ts * tol / s.err_loc, s.xm);
    s.t_new = round_step(tnew);
    double err = fmax(s.err_loc, rndoff);
    s.t_now += ts;
    s.step_min = fmin(s.step_min, ts);
    s.step_max = fmax(s.step_max, ts);
    s.s_error += err;
    s.x_error = fmax(s.x_error, err);
    int tt = s.tt;
    s.out_first = tt;
    while (tt < tn && s.t_now >= ta[(size_t)b * tn + tt]) ++tt;
    s.out_last = tt;
    s.tt = tt;
    act[b] = tt < tn;
    if (act[b]) atomicAdd(nactive, 1);
}

// W[(tt*N + x)*nvec + b] = w[x*P + b] for tt in [out_first, out_last)
__global__ void k_write_out(const zd *__restrict__ w, const VState *__restrict__ st,
                            zd *__restrict__ W, size_t N, int plog, int nvec)
{
    const size_t total = N << plog;
    const int P = 1 << plog;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e & (P - 1));
        if (b >= nvec) continue;
        const size_t x = e >> plog;
        const zd v = w[e];
        for (int tt = st[b].out_first; tt < st[b].out_last; ++tt)
            W[((size_t)tt * N + x) * nvec + b] = v;
    }
}

__global__ void k_pad_in(const zd *__restrict__ V, zd *__restrict__ w, size_t N, int plog,
                         int nvec)
{
    const size_t total = N << plog;
    const int P = 1 << plog;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(e & (P - 1));
        w[e] = b < nvec ? V[(e >> plog) * nvec + b] : zmake(0, 0);
    }
}

__global__ void k_copy(const zd *__restrict__ a, zd *__restrict__ b, size_t n)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x)
        b[e] = a[e];
}

__global__ void k_cplx_to_norm(const zd *d, double *nrm2, int nvec)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nvec) nrm2[b] = d[b].x;
}

__global__ void k_lanczos_take_aj(const zd *d, LState *ls)
{
    ls->aj = d[0];
}
__global__ void k_lanczos_take_nrm(const zd *d, LState *ls)
{
    ls->nrm2 = d[0].x;
}

__global__ void k_collect_stats(const VState *st, oops_expv_stats *out, const LState *ls)
{
    const VState &s = st[0];
    out->nmult = s.nmult;
    out->nexph = s.nexph;
    out->nscale = s.nscale;
    out->nstep = s.nstep;
    out->nreject = s.nreject;
    out->ibrkflag = s.ibrkflag;
    out->mbrkdwn = s.mbrkdwn;
    out->anorm = ls->anorm;
    out->step_min = s.step_min;
    out->step_max = s.step_max;
    out->x_error = s.x_error;
    out->s_error = s.s_error;
    out->hump = s.vnorm > 0 ? s.hump / s.vnorm : 0.0;
}

__global__ void k_first_status(const VState *st, int nvec, int *status)
{
    for (int b = 0; b < nvec; ++b)
        if (st[b].status) { *status = st[b].status; return; }
}

inline unsigned grid_for(size_t total)
{
    size_t g = (total + 255) / 256;
    size_t cap = (size_t)oops_sm_count() * 8;
    return (unsigned)std::max<size_t>(1, std::min(g, cap));
}


// ---------------------------------------------------------------- norm estimate (host)
// The reference runs the power iteration on the k x k Lanczos matrix T on the
// host (zgexpv_cache.f:342-359), with no iteration limit.  Here the same
// iteration (same start vector, same arithmetic and exit test) runs on the
// host on a copy of T (k <= 64, at most 32 KB); if it has not met the
// reference's test after POWER_ITERS iterations -- the dominant eigenvalue is
// not unique, e.g. a spectrum symmetric about zero, where the reference's
// loop never ends -- the estimate comes from the exact dominant eigenpairs of
// T instead (cyclic Jacobi): anorm = |lambda| + |bj v_k| maximised over the
// eigenvalues of largest modulus, the value the iteration approaches.
constexpr long POWER_ITERS = 20000;

double power_anorm_host(const double *T, int k, double bj, double tol, const double *q0)
{
    std::vector<double> qr(q0, q0 + k), wr(k, 0.0);
    double cj = 0.0, cjm = 0.0;
    for (long it = 0; it < POWER_ITERS; ++it) {
        for (int r = 0; r < k; ++r) {
            double sacc = 0.0;
            for (int c = 0; c < k; ++c) sacc += T[r + c * k] * qr[c];
            wr[r] = sacc;
        }
        cj = 0.0;
        for (int r = 0; r < k; ++r) cj += qr[r] * wr[r];
        if (cj == 0.0) break;
        if (fabs(1.0 - cjm / cj) < tol) return fabs(cj) + fabs(bj * qr[k - 1]);
        cjm = cj;
        double nr = 0.0;
        for (int r = 0; r < k; ++r) nr += wr[r] * wr[r];
        nr = sqrt(nr);
        for (int r = 0; r < k; ++r) qr[r] = wr[r] / nr;
    }
    if (cj == 0.0) return fabs(bj * qr[k - 1]);
    // exact eigenpairs of the symmetric T (cyclic Jacobi, k <= 64)
    std::vector<double> A(T, T + (size_t)k * k), V((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) V[i + (size_t)i * k] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int c = 0; c < k; ++c)
            for (int r = 0; r < k; ++r) {
                const double v = A[r + (size_t)c * k] * A[r + (size_t)c * k];
                tot += v;
                if (r != c) off += v;
            }
        if (off <= 1e-32 * tot) break;
        for (int p = 0; p < k - 1; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[p + (size_t)q * k];
                if (apq == 0.0) continue;
                const double app = A[p + (size_t)p * k], aqq = A[q + (size_t)q * k];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < k; ++r) {  // A <- A J (columns p, q)
                    const double arp = A[r + (size_t)p * k], arq = A[r + (size_t)q * k];
                    A[r + (size_t)p * k] = c * arp - s * arq;
                    A[r + (size_t)q * k] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {  // A <- J^T A (rows p, q)
                    const double apr = A[p + (size_t)r * k], aqr = A[q + (size_t)r * k];
                    A[p + (size_t)r * k] = c * apr - s * aqr;
                    A[q + (size_t)r * k] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; ++r) {
                    const double vrp = V[r + (size_t)p * k], vrq = V[r + (size_t)q * k];
                    V[r + (size_t)p * k] = c * vrp - s * vrq;
                    V[r + (size_t)q * k] = s * vrp + c * vrq;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < k; ++i) lmax = std::max(lmax, fabs(A[i + (size_t)i * k]));
    double best = 0.0;
    for (int i = 0; i < k; ++i)
        if (fabs(A[i + (size_t)i * k]) >= lmax * (1.0 - 1e-12))
            best = std::max(best, lmax + fabs(bj * V[(k - 1) + (size_t)i * k]));
    return best;
}

// ---------------------------------------------------------------- workspace
}  // namespace

struct oops_expv_cache {
    // capacity of the buffers below
    size_t N = 0, tn_cap = 0;
    int plog = 0, mh = 0, nblk = 0;
    zd *basis = nullptr;   // (m+2) blocks of N*P
    zd *w = nullptr;       // N*P
    zd *partial = nullptr; // nchunk*nblk*DOT_CHUNK*P
    zd *dots = nullptr;    // P*mh   (pass 1)
    zd *dots2 = nullptr;   // P*mh   (pass 2)
    zd *Hm = nullptr;      // P*mh*mh
    zd *Ecol = nullptr;    // P*mh
    zd *red1 = nullptr;    // P (norm reduction as complex)
    double *nrm2 = nullptr, *inv = nullptr;
    int *live = nullptr, *act = nullptr, *nactive = nullptr, *status = nullptr;
    VState *st = nullptr;
    LState *ls = nullptr;
    double *ta = nullptr;
    zd *lq = nullptr, *lqm = nullptr, *lw = nullptr;
    oops_expv_stats *dstats = nullptr;
    // the norm estimate of this Hamiltonian (the Lanczos start vector is a
    // fixed sequence, so it depends only on klim and tol)
    bool anorm_valid = false;
    size_t anorm_klim = 0;
    double anorm_tol = 0.0, anorm = 0.0;
    // one integration step captured as a graph, keyed on the call's shape
    cudaGraphExec_t step_exec = nullptr;
    int g_nvec = -1, g_plog = -1, g_m = -1, g_tn = -1;
    double g_tol = 0.0, g_rndoff = 0.0;
    const zd *g_wout = nullptr;
    cudaStream_t cap_stream = nullptr;  // private stream the step is captured on
    void release_buffers()
    {
        cudaFree(basis); cudaFree(w); cudaFree(partial); cudaFree(dots); cudaFree(dots2);
        cudaFree(Hm); cudaFree(Ecol); cudaFree(red1); cudaFree(nrm2); cudaFree(inv);
        cudaFree(live); cudaFree(act); cudaFree(nactive); cudaFree(status); cudaFree(st);
        cudaFree(ta); cudaFree(lq); cudaFree(lqm); cudaFree(lw); cudaFree(dstats);
        basis = w = partial = dots = dots2 = Hm = Ecol = red1 = lq = lqm = lw = nullptr;
        nrm2 = inv = ta = nullptr;
        live = act = nactive = status = nullptr;
        st = nullptr;
        dstats = nullptr;
        N = tn_cap = 0;
        plog = mh = nblk = 0;
        drop_graph();
    }
    void drop_graph()
    {
        if (step_exec) cudaGraphExecDestroy(step_exec);
        step_exec = nullptr;
        g_nvec = g_plog = g_m = g_tn = -1;
        g_wout = nullptr;
    }
};

void oops_expv_cache_free(oops_expv_cache *c)
{
    if (!c) return;
    c->release_buffers();
    cudaFree(c->ls);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    delete c;
}

namespace {

// The view of the cached buffers one call works with (its own nvec, m).
struct Work {
    size_t N = 0;
    int plog = 0, nvec = 0, m = 0, mh = 0, nblk = 0;
    oops_expv_cache *c = nullptr;
};

int alloc(void **p, size_t bytes)
{
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return oops_set_status(OOPS_ERR_NOMEM, "cudaMalloc failed (expv workspace)");
    }
    return OOPS_OK;
}

// make the handle's buffers hold a call of this shape (grow only)
int ensure_buffers(oops_expv_cache *c, size_t N, int plog, int mh, int nblk, size_t tn_cols)
{
    const int P = 1 << plog;
    if (c->basis && c->N == N && c->plog >= plog && c->mh >= mh && c->nblk >= nblk &&
        c->tn_cap >= tn_cols)
        return OOPS_OK;
    const int Pn = 1 << std::max(plog, c->basis ? c->plog : 0);
    const int mhn = std::max(mh, c->basis ? c->mh : 0);
    const int nblkn = std::max(nblk, c->basis ? c->nblk : 0);
    const size_t tnn = std::max(tn_cols, c->basis ? c->tn_cap : (size_t)0);
    c->release_buffers();
    const size_t blk = N * Pn;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    if ((size_t)(mhn + 1) * blk * sizeof(zd) > freeb)
        return oops_set_status(OOPS_ERR_NOMEM, "Krylov basis does not fit in device memory");
    const int nchunk = (mhn + DOT_CHUNK - 1) / DOT_CHUNK;
    int rc;
    if ((rc = alloc((void **)&c->basis, (size_t)mhn * blk * sizeof(zd))) ||
        (rc = alloc((void **)&c->w, blk * sizeof(zd))) ||
        (rc = alloc((void **)&c->partial, (size_t)nchunk * nblkn * DOT_CHUNK * Pn * sizeof(zd))) ||
        (rc = alloc((void **)&c->dots, (size_t)Pn * mhn * sizeof(zd))) ||
        (rc = alloc((void **)&c->dots2, (size_t)Pn * mhn * sizeof(zd))) ||
        (rc = alloc((void **)&c->Hm, (size_t)Pn * mhn * mhn * sizeof(zd))) ||
        (rc = alloc((void **)&c->Ecol, (size_t)Pn * mhn * sizeof(zd))) ||
        (rc = alloc((void **)&c->red1, (size_t)Pn * sizeof(zd))) ||
        (rc = alloc((void **)&c->nrm2, (size_t)Pn * sizeof(double))) ||
        (rc = alloc((void **)&c->inv, (size_t)Pn * sizeof(double))) ||
        (rc = alloc((void **)&c->live, (size_t)Pn * sizeof(int))) ||
        (rc = alloc((void **)&c->act, (size_t)Pn * sizeof(int))) ||
        (rc = alloc((void **)&c->nactive, sizeof(int))) ||
        (rc = alloc((void **)&c->status, sizeof(int))) ||
        (rc = alloc((void **)&c->st, (size_t)Pn * sizeof(VState))) ||
        (rc = alloc((void **)&c->ta, tnn * sizeof(double))) ||
        (rc = alloc((void **)&c->lq, N * sizeof(zd))) || (rc = alloc((void **)&c->lqm, N * sizeof(zd))) ||
        (rc = alloc((void **)&c->lw, N * sizeof(zd))) ||
        (rc = alloc((void **)&c->dstats, sizeof(oops_expv_stats)))) {
        c->release_buffers();
        return rc;
    }
    c->N = N;
    c->plog = 0;
    while ((1 << c->plog) < Pn) ++c->plog;
    c->mh = mhn;
    c->nblk = nblkn;
    c->tn_cap = tnn;
    (void)P;
    return OOPS_OK;
}

// sum_x conj(a_i) y for i < nb, columns into out[b*ld + i] (P columns)
void dots(const Work &W, const zd *basis, size_t bstride, int nb, const zd *y, zd *out, int ld,
          int accumulate, cudaStream_t st)
{
    int nchunk = (nb + DOT_CHUNK - 1) / DOT_CHUNK;
    dim3 grid(W.nblk, nchunk);
    k_dots<<<grid, RED_THREADS, 0, st>>>(basis, bstride, nb, y, W.N, W.plog, W.c->partial);
    int P = 1 << W.plog;
    int q = nb * P;
    k_dots_final<<<(q + 127) / 128, 128, 0, st>>>(W.c->partial, W.nblk, nb, W.plog, W.nvec, out, ld,
                                                   accumulate);
}

void norms(const Work &W, const zd *y, cudaStream_t st)
{
    // ||y||^2 as the real part of <y, y>
    dots(W, y, 0, 1, y, W.c->red1, 1, 0, st);
    k_cplx_to_norm<<<(W.nvec + 127) / 128, 128, 0, st>>>(W.c->red1, W.c->nrm2, W.nvec);
}

// Lanczos (+H) on the DLARAN start vector, then the norm estimate on the host
int estimate_norm(const oops_ham *h, const Work &W, size_t klim, double tol, cudaStream_t st,
                  double *anorm_out)
{
    oops_expv_cache *c = W.c;
    const size_t N = W.N;
    LState lzero;
    memset(&lzero, 0, sizeof(lzero));
    lzero.k = (int)std::min<size_t>(klim, N);
    OOPS_CUDA_TRY(cudaMemcpyAsync(c->ls, &lzero, sizeof(LState), cudaMemcpyHostToDevice, st));
    const unsigned gN = grid_for(N);
    Work L = W;  // single-vector view for reductions
    L.plog = 0;
    L.nvec = 1;
    L.nblk = std::max(1, std::min(oops_sm_count() * 2, (int)((N + 255) / 256)));
    k_dlaran_vec<<<gN, 256, 0, st>>>(c->lq, N);
    cudaMemsetAsync(c->lqm, 0, N * sizeof(zd), st);
    dots(L, c->lq, 0, 1, c->lq, c->red1, 1, 0, st);
    k_lanczos_take_nrm<<<1, 1, 0, st>>>(c->red1, c->ls);
    k_lanczos_norm0<<<gN, 256, 0, st>>>(c->lq, N, c->ls);
    for (int j = 1; j <= lzero.k; ++j) {
        int rc = oops_ham_apply_internal(h, zmake(1, 0), c->lq, c->lw, 1, 0, nullptr, st);
        if (rc) return rc;
        dots(L, c->lq, 0, 1, c->lw, c->red1, 1, 0, st);
        k_lanczos_take_aj<<<1, 1, 0, st>>>(c->red1, c->ls);
        k_lanczos_axpy<<<gN, 256, 0, st>>>(c->lw, c->lq, c->lqm, N, c->ls);
        dots(L, c->lw, 0, 1, c->lw, c->red1, 1, 0, st);
        k_lanczos_take_nrm<<<1, 1, 0, st>>>(c->red1, c->ls);
        k_lanczos_post<<<1, 1, 0, st>>>(c->ls, j, tol);
        k_lanczos_shift<<<gN, 256, 0, st>>>(c->lq, c->lqm, c->lw, N, c->ls, j == lzero.k);
        k_lanczos_bjm<<<1, 1, 0, st>>>(c->ls);
    }
    LState hs;
    OOPS_CUDA_TRY(cudaMemcpyAsync(&hs, c->ls, sizeof(LState), cudaMemcpyDeviceToHost, st));
    OOPS_CUDA_TRY(cudaStreamSynchronize(st));
    const int k = hs.k;
    std::vector<double> q0(k);
    for (int j = 0; j < k; ++j) q0[j] = dlaran_draw(2 * N + 1 + j);
    const double anorm = k > 0 ? power_anorm_host(hs.T, k, hs.bj, tol, q0.data()) : 0.0;
    OOPS_CUDA_TRY(cudaMemcpyAsync(&c->ls->anorm, &anorm, sizeof(double), cudaMemcpyHostToDevice, st));
    OOPS_CUDA_TRY(cudaStreamSynchronize(st));
    *anorm_out = anorm;
    return OOPS_OK;
}

// one integration step for every active column (no host reads)
int enqueue_step(const oops_ham *h, const Work &W, double tol_eff, double rndoff, int tn,
                 cudaStream_t st)
{
    oops_expv_cache *c = W.c;
    const int P = 1 << W.plog;
    const size_t blk = W.N * P;
    const unsigned gB = grid_for(blk);
    const unsigned gS = (P + 127) / 128;
    const size_t smem = (size_t)5 * W.mh * W.mh * sizeof(zd);
    const zd minus_i = zmake(0, -1);
    k_step_begin<<<gS, 128, 0, st>>>(c->st, W.nvec, c->ta, tn, c->act, c->live, c->inv, c->Hm, W.mh);
    // V_0 = w / beta
    k_copy<<<gB, 256, 0, st>>>(c->w, c->basis, blk);
    k_scale<<<gB, 256, 0, st>>>(c->basis, W.N, W.plog, W.nvec, c->inv, c->live);
    for (int j = 0; j < W.m; ++j) {
        zd *vj = c->basis + (size_t)j * blk;
        zd *vn = c->basis + (size_t)(j + 1) * blk;
        int rc = oops_ham_apply_internal(h, minus_i, vj, vn, W.nvec, W.plog, c->live, st);
        if (rc) return rc;
        // CGS2: two passes of h = V^H v, v -= V h
        dots(W, c->basis, blk, j + 1, vn, c->dots, W.mh, 0, st);
        k_subtract<<<gB, 256, 0, st>>>(c->basis, blk, j + 1, c->dots, W.mh, vn, W.N, W.plog, W.nvec, c->live);
        dots(W, c->basis, blk, j + 1, vn, c->dots2, W.mh, 0, st);
        k_subtract<<<gB, 256, 0, st>>>(c->basis, blk, j + 1, c->dots2, W.mh, vn, W.N, W.plog, W.nvec, c->live);
        norms(W, vn, st);
        k_arnoldi_post<<<gS, 128, 0, st>>>(c->st, W.nvec, j, c->nrm2, c->dots, c->dots2, c->live, c->inv,
                                          c->Hm, W.mh, c->ta, tn);
        k_scale<<<gB, 256, 0, st>>>(vn, W.N, W.plog, W.nvec, c->inv, c->live);
    }
    k_avnorm_live<<<gS, 128, 0, st>>>(c->st, W.nvec, c->act, c->live);
    {
        zd *vm = c->basis + (size_t)W.m * blk;
        zd *vx = c->basis + (size_t)(W.m + 1) * blk;
        int rc = oops_ham_apply_internal(h, minus_i, vm, vx, W.nvec, W.plog, c->live, st);
        if (rc) return rc;
        norms(W, vx, st);
        k_avnorm_post<<<gS, 128, 0, st>>>(c->st, W.nvec, c->nrm2, c->live);
    }
    k_padm<<<W.nvec, 256, smem, st>>>(c->st, W.nvec, c->act, c->Hm, W.mh, W.m, tol_eff, c->Ecol);
    k_update_w<<<gB, 256, 0, st>>>(c->basis, blk, c->Ecol, W.mh, c->st, c->act, c->w, W.N, W.plog, W.nvec);
    norms(W, c->w, st);
    cudaMemsetAsync(c->nactive, 0, sizeof(int), st);
    k_step_end<<<gS, 128, 0, st>>>(c->st, W.nvec, c->nrm2, tol_eff, rndoff, c->ta, tn, c->act, c->nactive);
    return OOPS_OK;
}

}  // namespace

// Core driver: V_in is the block (N x nvec interleaved, device), ta_host per
// column (tn entries each), W_out unpadded tn x N x nvec.  Buffers, the norm
// estimate and the captured integration step live on the Hamiltonian handle
// and are reused by its later calls.  The integration runs in chunks of steps
// (1, 2, 4, ... up to 64) between which the host reads one counter: columns
// that finish inside a chunk make the remaining steps of the chunk no-ops.
int oops_expv_run(const oops_ham *h, const zd *V_in, size_t nvec, size_t tn,
                  const double *ta_host, size_t m, double tol, size_t klim, zd *W_out,
                  oops_expv_stats *stats, cudaStream_t st)
{
    const size_t N = oops_ham_dim(h);
    if (nvec == 0 || nvec > 256) return oops_set_status(OOPS_ERR_SIZE, "nvec must be 1..256");
    if (m == 0 || m >= N) return oops_set_status(OOPS_ERR_SIZE, "bad sizes (m must satisfy 1 <= m < n)");
    if (m > 50) return oops_set_status(OOPS_ERR_SIZE, "m > 50 (mmax of the reference driver)");
    if (klim == 0 || klim > 64) return oops_set_status(OOPS_ERR_SIZE, "Lanczos length k must be 1..64");
    if (tn == 0) return OOPS_OK;
    oops_expv_cache *&cache = oops_ham_expv_cache(h);
    if (!cache) {
        cache = new oops_expv_cache();
        int rc = alloc((void **)&cache->ls, sizeof(LState));
        if (rc) {
            delete cache;
            cache = nullptr;
            return rc;
        }
    }
    oops_expv_cache *c = cache;
    Work W;
    W.c = c;
    W.N = N;
    W.nvec = (int)nvec;
    while ((1u << W.plog) < nvec) ++W.plog;
    const int P = 1 << W.plog;
    W.m = (int)m;
    W.mh = (int)m + 2;
    W.nblk = std::max(1, std::min(oops_sm_count() * 2, (int)((N * P + 255) / 256)));
    int rc = ensure_buffers(c, N, W.plog, W.mh, W.nblk, tn * nvec);
    if (rc) return rc;
    const size_t blk = N * P;
    OOPS_CUDA_TRY(cudaMemcpyAsync(c->ta, ta_host, tn * nvec * sizeof(double), cudaMemcpyHostToDevice, st));
    OOPS_CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int), st));
    // ---- norm estimate, once per Hamiltonian (and klim, tol)
    if (!c->anorm_valid || c->anorm_klim != klim || c->anorm_tol != tol) {
        if ((rc = estimate_norm(h, W, klim, tol, st, &c->anorm))) return rc;
        c->anorm_valid = true;
        c->anorm_klim = klim;
        c->anorm_tol = tol;
        c->drop_graph();  // the graph bakes in rndoff
    } else {
        OOPS_CUDA_TRY(cudaMemcpyAsync(&c->ls->anorm, &c->anorm, sizeof(double), cudaMemcpyHostToDevice, st));
    }
    const double tol_eff = tol <= 0x1p-52 ? sqrt(0x1p-52) : tol;
    const double rndoff = 0x1p-52 * c->anorm;
    // ---- state and initial outputs
    const unsigned gB = grid_for(blk);
    k_pad_in<<<gB, 256, 0, st>>>(V_in, c->w, N, W.plog, W.nvec);
    norms(W, c->w, st);
    k_init<<<(P + 127) / 128, 128, 0, st>>>(c->st, W.nvec, c->nrm2, W.m, tol_eff, c->ls, c->ta, (int)tn, c->act);
    k_write_out<<<gB, 256, 0, st>>>(c->w, c->st, W_out, N, W.plog, W.nvec);
    const size_t smem = (size_t)5 * W.mh * W.mh * sizeof(zd);
    cudaFuncSetAttribute(k_padm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nact = 0;
    {
        std::vector<int> a(P);
        OOPS_CUDA_TRY(cudaMemcpyAsync(a.data(), c->act, P * sizeof(int), cudaMemcpyDeviceToHost, st));
        OOPS_CUDA_TRY(cudaStreamSynchronize(st));
        for (int b = 0; b < W.nvec; ++b) nact += a[b];
    }
    long steps = 0;
    int chunk = 1;
    while (nact > 0) {
        if (steps > 20000000L) return oops_set_status(OOPS_ERR_NUMERIC, "step limit exceeded");
        if (steps == 0) {
            // the first step with plain launches (many calls need one step)
            if ((rc = enqueue_step(h, W, tol_eff, rndoff, (int)tn, st))) return rc;
            k_write_out<<<gB, 256, 0, st>>>(c->w, c->st, W_out, N, W.plog, W.nvec);
        } else {
            // later steps: one captured graph of a step, replayed `chunk` times
            const bool same = c->step_exec && c->g_nvec == W.nvec && c->g_plog == W.plog &&
                              c->g_m == W.m && c->g_tn == (int)tn && c->g_tol == tol_eff &&
                              c->g_rndoff == rndoff && c->g_wout == W_out;
            if (!same) {
                c->drop_graph();
                // captured on a private stream (the caller's may be the legacy
                // default stream, which cannot be captured), launched on st
                if (!c->cap_stream)
                    OOPS_CUDA_TRY(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
                cudaStream_t cs = c->cap_stream;
                cudaGraph_t g = nullptr;
                OOPS_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                rc = enqueue_step(h, W, tol_eff, rndoff, (int)tn, cs);
                k_write_out<<<gB, 256, 0, cs>>>(c->w, c->st, W_out, N, W.plog, W.nvec);
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
                e = cudaGraphInstantiate(&c->step_exec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    c->step_exec = nullptr;
                    return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
                }
                c->g_nvec = W.nvec;
                c->g_plog = W.plog;
                c->g_m = W.m;
                c->g_tn = (int)tn;
                c->g_tol = tol_eff;
                c->g_rndoff = rndoff;
                c->g_wout = W_out;
            }
            for (int s = 0; s < chunk; ++s) OOPS_CUDA_TRY(cudaGraphLaunch(c->step_exec, st));
        }
        steps += steps == 0 ? 1 : chunk;
        if (steps > 1) chunk = std::min(chunk * 2, 64);
        OOPS_CUDA_TRY(cudaMemcpyAsync(&nact, c->nactive, sizeof(int), cudaMemcpyDeviceToHost, st));
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    }
    // status of the columns
    k_first_status<<<1, 1, 0, st>>>(c->st, W.nvec, c->status);
    int sc = 0;
    OOPS_CUDA_TRY(cudaMemcpyAsync(&sc, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (stats) {
        k_collect_stats<<<1, 1, 0, st>>>(c->st, c->dstats, c->ls);
        OOPS_CUDA_TRY(cudaMemcpyAsync(stats, c->dstats, sizeof(oops_expv_stats), cudaMemcpyDeviceToHost, st));
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(e));
    if (sc) return oops_set_status(sc, "Pade failure or step-rejection cap in a column");
    return OOPS_OK;
}
