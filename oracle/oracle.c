/*
 * oracle.c -- CPU restatement of the nzhao/oops CCE hot path (TEST
 * INFRASTRUCTURE ONLY; see oracle.h for the parity status and the rule that
 * only tests/, smoke() and bench.py's baseline legs may use it).
 *
 * Written from the published algorithms (Sidje, "Expokit", ACM TOMS 24(1),
 * 1998, for the Krylov/Pade parts; LAPACK DLARAN for the generator) and from
 * the behaviour of the reference files cited at each function.  No reference
 * source is copied.  Plain C11, no BLAS: every loop is written out.
 */
#include "oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846
/* armadillo datum:: constants of the reference's era (CODATA 2014);
 * the armadillo version the reference linked is not pinned. */
#define ORC_HBAR 1.054571800e-34
#define ORC_MU0 1.2566370614e-06

/* ------------------------------------------------------------------------ */
/* DLARAN (expokit/DLARAN.f:3-92)                                            */
/* ------------------------------------------------------------------------ */
double orc_dlaran(int iseed[4])
{
    /* seed as one 48-bit integer, 12 bits per element, element 1 highest */
    uint64_t s = ((uint64_t)iseed[0] << 36) | ((uint64_t)iseed[1] << 24) |
                 ((uint64_t)iseed[2] << 12) | (uint64_t)iseed[3];
    const uint64_t mult = 33952834046453ULL;
    s = (s * mult) & ((1ULL << 48) - 1);
    iseed[0] = (int)((s >> 36) & 4095);
    iseed[1] = (int)((s >> 24) & 4095);
    iseed[2] = (int)((s >> 12) & 4095);
    iseed[3] = (int)(s & 4095);
    /* exact: 48 bits fit the 53-bit mantissa */
    return (double)s * 0x1p-48;
}

/* ------------------------------------------------------------------------ */
/* small dense helpers                                                       */
/* ------------------------------------------------------------------------ */
static double znrm2(size_t n, const orc_z *x)
{
    /* scaled sum of squares, as a reference BLAS dznrm2 does */
    double scale = 0.0, ssq = 1.0;
    for (size_t i = 0; i < n; ++i) {
        double p[2] = {creal(x[i]), cimag(x[i])};
        for (int c = 0; c < 2; ++c) {
            if (p[c] != 0.0) {
                double a = fabs(p[c]);
                if (scale < a) {
                    ssq = 1.0 + ssq * (scale / a) * (scale / a);
                    scale = a;
                } else {
                    ssq += (a / scale) * (a / scale);
                }
            }
        }
    }
    return scale * sqrt(ssq);
}

static orc_z zdotc(size_t n, const orc_z *x, const orc_z *y)
{
    orc_z s = 0;
    for (size_t i = 0; i < n; ++i) s += conj(x[i]) * y[i];
    return s;
}

/* C = alpha*A*B + beta*C, column-major, A m x k, B k x n */
static void zgemm_nn(int m, int n, int k, orc_z alpha, const orc_z *A,
                     int lda, const orc_z *B, int ldb, orc_z beta, orc_z *C,
                     int ldc)
{
    for (int j = 0; j < n; ++j) {
        orc_z *c = C + (size_t)j * ldc;
        if (beta == 0)
            for (int i = 0; i < m; ++i) c[i] = 0;
        else if (beta != 1)
            for (int i = 0; i < m; ++i) c[i] *= beta;
        for (int l = 0; l < k; ++l) {
            orc_z b = alpha * B[l + (size_t)j * ldb];
            if (b == 0) continue;
            const orc_z *a = A + (size_t)l * lda;
            for (int i = 0; i < m; ++i) c[i] += a[i] * b;
        }
    }
}

static double cabs1(orc_z z) { return fabs(creal(z)) + fabs(cimag(z)); }

/* Solve A X = B in place (A n x n overwritten by LU, B n x nrhs), partial
 * pivoting on |re|+|im| as LAPACK's ZGETRF/IZAMAX.  Returns 0 or -1. */
static int zgesv(int n, int nrhs, orc_z *A, int lda, orc_z *B, int ldb)
{
    int *piv = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int j = 0; j < n; ++j) {
        int p = j;
        double best = cabs1(A[j + (size_t)j * lda]);
        for (int i = j + 1; i < n; ++i) {
            double v = cabs1(A[i + (size_t)j * lda]);
            if (v > best) { best = v; p = i; }
        }
        piv[j] = p;
        if (best == 0.0) { free(piv); return -1; }
        if (p != j)
            for (int c = 0; c < n; ++c) {
                orc_z t = A[j + (size_t)c * lda];
                A[j + (size_t)c * lda] = A[p + (size_t)c * lda];
                A[p + (size_t)c * lda] = t;
            }
        orc_z inv = 1.0 / A[j + (size_t)j * lda];
        for (int i = j + 1; i < n; ++i) A[i + (size_t)j * lda] *= inv;
        for (int c = j + 1; c < n; ++c) {
            orc_z f = A[j + (size_t)c * lda];
            if (f == 0) continue;
            for (int i = j + 1; i < n; ++i)
                A[i + (size_t)c * lda] -= A[i + (size_t)j * lda] * f;
        }
    }
    for (int r = 0; r < nrhs; ++r) {
        orc_z *b = B + (size_t)r * ldb;
        for (int j = 0; j < n; ++j)
            if (piv[j] != j) { orc_z t = b[j]; b[j] = b[piv[j]]; b[piv[j]] = t; }
        for (int j = 0; j < n; ++j) /* L y = b, unit diagonal */
            for (int i = j + 1; i < n; ++i) b[i] -= A[i + (size_t)j * lda] * b[j];
        for (int j = n - 1; j >= 0; --j) { /* U x = y */
            b[j] /= A[j + (size_t)j * lda];
            for (int i = 0; i < j; ++i) b[i] -= A[i + (size_t)j * lda] * b[j];
        }
    }
    free(piv);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Kronecker matvec (hamvec_func3.cpp:73-100, 307-389)                       */
/* ------------------------------------------------------------------------ */
void orc_kron_mode(size_t m, size_t s, size_t n, const orc_z *A, orc_z *x)
{
    orc_z tmp[64];
    for (size_t k = 0; k < m * n; ++k) {
        /* element k of the m*n groups: high index k/n, low index k%n */
        size_t base = (k / n) * s * n + (k % n);
        for (size_t q = 0; q < s; ++q) tmp[q] = x[base + n * q];
        for (size_t p = 0; p < s; ++p) {
            orc_z acc = 0;
            for (size_t q = 0; q < s; ++q) acc += tmp[q] * A[p + s * q];
            x[base + n * p] = acc;
        }
    }
}

void orc_hamvec(size_t nspin, size_t nterm, const orc_z *coeff,
                const size_t *nbody_lst, const size_t *pos_i_idx,
                const size_t *pos_i_lst, const size_t *dim_i_lst,
                const size_t *mat_i_idx, const orc_z *mat_i_lst, size_t vlen,
                const size_t *nspin_dim, const orc_z *v, orc_z *w, orc_z *w_med)
{
    size_t *mlst = (size_t *)malloc(sizeof(size_t) * nspin);
    size_t *nlst = (size_t *)malloc(sizeof(size_t) * nspin);
    for (size_t i = 0; i < nspin; ++i) {
        size_t a = 1, b = 1;
        for (size_t j = 0; j < i; ++j) a *= nspin_dim[j];
        for (size_t j = i + 1; j < nspin; ++j) b *= nspin_dim[j];
        mlst[i] = a;
        nlst[i] = b;
    }
    for (size_t i = 0; i < vlen; ++i) w[i] = 0;
    for (size_t t = 0; t < nterm; ++t) {
        size_t nb = nbody_lst[t];
        memcpy(w_med, v, sizeof(orc_z) * vlen);
        for (size_t b = 0; b < nb; ++b) {
            size_t idx = pos_i_idx[t] + nb - 1 - b; /* last body first */
            size_t pos = pos_i_lst[idx];
            orc_kron_mode(mlst[pos], dim_i_lst[idx], nlst[pos],
                          mat_i_lst + mat_i_idx[idx], w_med);
        }
        orc_z c = coeff[t];
        for (size_t i = 0; i < vlen; ++i) w[i] += c * w_med[i];
    }
    free(mlst);
    free(nlst);
}

/* ------------------------------------------------------------------------ */
/* Pade exponential (expokit.f:762-933)                                      */
/* ------------------------------------------------------------------------ */
int orc_padm(int ideg, int m, double t, const orc_z *H, int ldh, orc_z *E,
             int *ns_out)
{
    size_t mm = (size_t)m * m;
    /* infinity norm (max row sum of |h_ij|) */
    double hnorm = 0.0;
    for (int i = 0; i < m; ++i) {
        double r = 0.0;
        for (int j = 0; j < m; ++j) r += cabs(H[i + (size_t)j * ldh]);
        if (r > hnorm) hnorm = r;
    }
    hnorm = fabs(t * hnorm);
    if (hnorm == 0.0) return -1;
    int ns = (int)(log(hnorm) / log(2.0)) + 2; /* C cast truncates, as INT */
    if (ns < 0) ns = 0;
    double scale = t / ldexp(1.0, ns);
    double scale2 = scale * scale;

    /* diagonal Pade coefficients c_k = c_{k-1} (p+1-k) / (k (2p+1-k)) */
    double c[32];
    c[0] = 1.0;
    for (int k = 1; k <= ideg; ++k)
        c[k] = c[k - 1] * (double)(ideg + 1 - k) / (double)(k * (2 * ideg + 1 - k));

    orc_z *H2 = (orc_z *)calloc(mm, sizeof(orc_z));
    orc_z *P = (orc_z *)calloc(mm, sizeof(orc_z));
    orc_z *Q = (orc_z *)calloc(mm, sizeof(orc_z));
    orc_z *T = (orc_z *)calloc(mm, sizeof(orc_z));
    /* H2 = scale^2 * H * H (copy H to a packed buffer first) */
    orc_z *Hp = (orc_z *)calloc(mm, sizeof(orc_z));
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) Hp[i + (size_t)j * m] = H[i + (size_t)j * ldh];
    zgemm_nn(m, m, m, scale2, Hp, m, Hp, m, 0, H2, m);

    /* Horner on the even (q) and odd (p) parts, starting with q */
    for (int i = 0; i < m; ++i) {
        P[i + (size_t)i * m] = c[ideg - 1];
        Q[i + (size_t)i * m] = c[ideg];
    }
    int q_turn = 1;
    for (int k = ideg - 1; k > 0; --k) {
        orc_z *X = q_turn ? Q : P;
        zgemm_nn(m, m, m, 1.0, X, m, H2, m, 0, T, m);
        for (int i = 0; i < m; ++i) T[i + (size_t)i * m] += c[k - 1];
        memcpy(X, T, mm * sizeof(orc_z));
        q_turn = !q_turn;
    }
    /* the part updated last pairs with the even powers; multiply the other
     * by scale*H to form the odd part */
    orc_z *odd = q_turn ? Q : P;   /* q_turn now names the one NOT updated last */
    orc_z *even = q_turn ? P : Q;
    zgemm_nn(m, m, m, scale, odd, m, Hp, m, 0, T, m);
    memcpy(odd, T, mm * sizeof(orc_z));
    /* denominator = even - odd, solve (even - odd) X = odd */
    for (size_t i = 0; i < mm; ++i) even[i] -= odd[i];
    if (zgesv(m, m, even, m, odd, m) != 0) {
        free(H2); free(P); free(Q); free(T); free(Hp);
        return -2;
    }
    /* (even - odd)^-1 odd  ->  I + 2X = (even + odd)/(even - odd) for either
     * parity of ideg (the Fortran reaches the same value through a sign flip
     * for odd ideg) */
    for (size_t i = 0; i < mm; ++i) odd[i] *= 2.0;
    for (int i = 0; i < m; ++i) odd[i + (size_t)i * m] += 1.0;
    orc_z *cur = odd, *nxt = T;
    for (int s = 0; s < ns; ++s) {
        zgemm_nn(m, m, m, 1.0, cur, m, cur, m, 0, nxt, m);
        orc_z *sw = cur; cur = nxt; nxt = sw;
    }
    memcpy(E, cur, mm * sizeof(orc_z));
    if (ns_out) *ns_out = ns;
    free(H2); free(P); free(Q); free(T); free(Hp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Krylov expv (hamvec_zgexpv_w_mkl_profile.f:186-538, main_mkl.f:1-130)     */
/* ------------------------------------------------------------------------ */
typedef struct {
    size_t nspin, nterm;
    const size_t *nbody, *pidx, *plst, *dlst, *midx, *sdim;
    const orc_z *mats;
    orc_z *coeffz;
    size_t n;
    orc_z *wmed;
} orc_op;

static void op_apply(orc_op *op, const orc_z *x, orc_z *y)
{
    orc_hamvec(op->nspin, op->nterm, op->coeffz, op->nbody, op->pidx, op->plst,
               op->dlst, op->midx, op->mats, op->n, op->sdim, x, y, op->wmed);
}

/* Fortran NINT (round half away from zero) and AINT (truncate) */
static double f_nint(double x) { return x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5); }
static double f_aint(double x) { return x >= 0 ? floor(x) : -floor(-x); }
static double f_pow10i(int e)
{
    double r = 1.0, b = 10.0;
    int a = e < 0 ? -e : e;
    while (a) { if (a & 1) r *= b; b *= b; a >>= 1; }
    return e < 0 ? 1.0 / r : r;
}
static double round_step(double t)
{
    const double sqr1 = sqrt(0.1);
    double p1 = f_pow10i((int)f_nint(log10(t) - sqr1) - 1);
    return f_aint(t / p1 + 0.55) * p1;
}

/* Lanczos (k steps, no re-orthogonalisation) + power iteration on T_k:
 * zgexpv lines 258-341 of the MKL variant. Coefficients real (+H). */
static double estimate_anorm(orc_op *op, size_t klim, double tol)
{
    size_t n = op->n;
    size_t k = klim;
    if (k > n) k = n;
    if (k == 0) return 0.0;
    for (size_t t = 0; t < op->nterm; ++t) op->coeffz[t] = creal(op->coeffz[t]);
    int iseed[4] = {0, 0, 0, 5};
    orc_z *qj = (orc_z *)malloc(sizeof(orc_z) * n);
    orc_z *qjm = (orc_z *)calloc(n, sizeof(orc_z));
    orc_z *w = (orc_z *)malloc(sizeof(orc_z) * n);
    double *tk = (double *)calloc(k * k, sizeof(double));
    for (size_t i = 0; i < n; ++i) {
        double re = orc_dlaran(iseed); /* real part drawn first */
        double im = orc_dlaran(iseed);
        qj[i] = re + I * im;
    }
    double bj = znrm2(n, qj);
    for (size_t i = 0; i < n; ++i) qj[i] *= 1.0 / bj;
    double bjm = 0.0;
    for (size_t j = 1; j <= k; ++j) {
        op_apply(op, qj, w);
        orc_z aj = zdotc(n, qj, w);
        tk[(j - 1) * k + (j - 1)] = creal(aj);
        for (size_t i = 0; i < n; ++i) w[i] -= aj * qj[i];
        for (size_t i = 0; i < n; ++i) w[i] -= bjm * qjm[i];
        bj = znrm2(n, w);
        if (j == k) break;
        tk[(j - 1) * k + j] = bj;
        tk[j * k + (j - 1)] = bj;
        if (bj < tol) break;
        memcpy(qjm, qj, sizeof(orc_z) * n);
        for (size_t i = 0; i < n; ++i) qj[i] = w[i] * (1.0 / bj);
        bjm = bj;
    }
    double *qr = (double *)malloc(sizeof(double) * k);
    double *wr = (double *)malloc(sizeof(double) * k);
    for (size_t j = 0; j < k; ++j) qr[j] = orc_dlaran(iseed);
    double cj = 0.0, cjm = 0.0;
    for (long it = 0; it < 1000000; ++it) {
        for (size_t r = 0; r < k; ++r) {
            double s = 0.0;
            for (size_t c = 0; c < k; ++c) s += tk[r + c * k] * qr[c];
            wr[r] = s;
        }
        cj = 0.0;
        for (size_t r = 0; r < k; ++r) cj += qr[r] * wr[r];
        if (cj == 0.0) break; /* the Fortran would divide by zero here */
        if (fabs(1.0 - cjm / cj) < tol) break;
        cjm = cj;
        double nr = 0.0;
        for (size_t r = 0; r < k; ++r) nr += wr[r] * wr[r];
        nr = sqrt(nr);
        for (size_t r = 0; r < k; ++r) qr[r] = wr[r] / nr;
    }
    double anorm = fabs(cj) + fabs(bj * qr[k - 1]);
    free(qj); free(qjm); free(w); free(tk); free(qr); free(wr);
    return anorm;
}

typedef struct {
    double t_now, t_new, beta, vnorm, hump, xm, s_error, x_error, step_min,
        step_max, tbrkdwn;
    long k1, mbrkdwn, nmult, nexph, nscale, nstep, nreject, ibrkflag;
} krylov_state;

/* integrate one column from its current t_now up to t_out (zgexpv 100-500) */
static int integrate_to(orc_op *op, krylov_state *s, orc_z *w, double t_out,
                        size_t m, double tol, double anorm, orc_z *V, orc_z *Hm,
                        orc_z *E)
{
    const size_t n = op->n;
    const size_t mh = m + 2;
    const double delta = 1.2, gamma = 0.9, break_tol = 1.0e-7;
    const double rndoff = 0x1p-52 * anorm;
    double avnorm = 0.0;
    while (s->t_now < t_out) {
        s->nstep++;
        double t_step = fmin(t_out - s->t_now, s->t_new);
        double p1 = 1.0 / s->beta;
        for (size_t i = 0; i < n; ++i) V[i] = p1 * w[i];
        memset(Hm, 0, sizeof(orc_z) * mh * mh);
        int broke = 0;
        for (size_t j = 1; j <= m; ++j) {
            s->nmult++;
            orc_z *vj = V + (j - 1) * n, *vn = V + j * n;
            op_apply(op, vj, vn);
            for (size_t i = 1; i <= j; ++i) { /* modified Gram-Schmidt */
                orc_z hij = zdotc(n, V + (i - 1) * n, vn);
                for (size_t r = 0; r < n; ++r) vn[r] -= hij * V[(i - 1) * n + r];
                Hm[(i - 1) + (j - 1) * mh] = hij;
            }
            double hj1j = znrm2(n, vn);
            if (hj1j <= break_tol) { /* happy breakdown */
                s->k1 = 0;
                s->ibrkflag = 1;
                s->mbrkdwn = (long)j;
                s->tbrkdwn = s->t_now;
                t_step = t_out - s->t_now;
                broke = 1;
                break;
            }
            Hm[j + (j - 1) * mh] = hj1j;
            for (size_t r = 0; r < n; ++r) vn[r] *= 1.0 / hj1j;
        }
        if (!broke) {
            s->nmult++;
            op_apply(op, V + m * n, V + (m + 1) * n);
            avnorm = znrm2(n, V + (m + 1) * n);
        }
        Hm[(m + 1) + m * mh] = 1.0; /* corrected scheme */
        double err_loc;
        long ireject = 0;
        for (;;) {
            s->nexph++;
            int mx = (int)(s->mbrkdwn + s->k1);
            int ns = 0;
            if (orc_padm(6, mx, t_step, Hm, (int)mh, E, &ns) != 0) return -4;
            s->nscale += ns;
            if (s->k1 == 0) {
                err_loc = tol;
            } else {
                double q1 = cabs(E[m]) * s->beta;
                double q2 = cabs(E[m + 1]) * s->beta * avnorm;
                if (q1 > 10.0 * q2) { err_loc = q2; s->xm = 1.0 / (double)m; }
                else if (q1 > q2) { err_loc = (q1 * q2) / (q1 - q2); s->xm = 1.0 / (double)m; }
                else { err_loc = q1; s->xm = 1.0 / (double)(m - 1); }
            }
            if (s->k1 != 0 && err_loc > delta * t_step * tol) {
                t_step = gamma * t_step * pow(t_step * tol / err_loc, s->xm);
                t_step = round_step(t_step);
                ireject++;
                s->nreject++;
                if (ireject > 10000 || !(t_step > 0.0)) return 3;
                continue;
            }
            break;
        }
        int mx = (int)(s->mbrkdwn + (s->k1 - 1 > 0 ? s->k1 - 1 : 0));
        /* w = beta * V(:,1:mx) * E(1:mx,1) */
        for (size_t r = 0; r < n; ++r) {
            orc_z acc = 0;
            for (int c = 0; c < mx; ++c) acc += V[(size_t)c * n + r] * E[c];
            w[r] = s->beta * acc;
        }
        s->beta = znrm2(n, w);
        if (s->beta > s->hump) s->hump = s->beta;
        s->t_new = gamma * t_step * pow(t_step * tol / err_loc, s->xm);
        s->t_new = round_step(s->t_new);
        if (err_loc < rndoff) err_loc = rndoff;
        s->t_now += t_step;
        if (t_step < s->step_min) s->step_min = t_step;
        if (t_step > s->step_max) s->step_max = t_step;
        s->s_error += err_loc;
        if (err_loc > s->x_error) s->x_error = err_loc;
    }
    return 0;
}

static void state_init(krylov_state *s, const orc_z *w, size_t n, size_t m,
                       double tol, double anorm)
{
    memset(s, 0, sizeof(*s));
    s->k1 = 2;
    s->mbrkdwn = (long)m;
    s->beta = znrm2(n, w);
    s->vnorm = s->beta;
    s->hump = s->beta;
    s->step_min = INFINITY;
    s->xm = 1.0 / (double)m;
    /* first step size (zgexpv lines 415-420) */
    double p2 = tol * pow((double)(m + 1) / 2.72, (double)(m + 1)) *
                sqrt(2.0 * 3.14 * (double)(m + 1));
    double t_new = (1.0 / anorm) * pow(p2 / (4.0 * s->beta * anorm), s->xm);
    s->t_new = round_step(t_new);
}

static int expv_core(size_t nspin, size_t nterm, const double *coeff_lst,
                     const size_t *nbody_lst, const size_t *pos_i_idx,
                     const size_t *pos_i_lst, const size_t *dim_i_lst,
                     const size_t *mat_i_idx, const orc_z *mat_i_lst,
                     size_t n, const size_t *nspin_dim, const orc_z *Vin,
                     size_t nvec, size_t klim, size_t tn, const double *ta,
                     int per_column_times, size_t m, double tol, orc_z *W,
                     orc_expv_stats *stats)
{
    if (m == 0 || m >= n) return -3; /* 'bad sizes' */
    if (klim == 0) return -5;
    orc_op op = {nspin, nterm, nbody_lst, pos_i_idx, pos_i_lst, dim_i_lst,
                 mat_i_idx, nspin_dim, mat_i_lst, NULL, n, NULL};
    op.coeffz = (orc_z *)malloc(sizeof(orc_z) * (nterm ? nterm : 1));
    op.wmed = (orc_z *)malloc(sizeof(orc_z) * n);
    for (size_t t = 0; t < nterm; ++t) op.coeffz[t] = coeff_lst[t];
    double anorm = estimate_anorm(&op, klim, tol);
    double eps = 0x1p-52; /* the Fortran adjusts tol after the estimate */
    if (tol <= eps) tol = sqrt(eps);
    for (size_t t = 0; t < nterm; ++t) op.coeffz[t] = -I * coeff_lst[t];
    size_t mh = m + 2;
    orc_z *V = (orc_z *)malloc(sizeof(orc_z) * n * (m + 2));
    orc_z *Hm = (orc_z *)malloc(sizeof(orc_z) * mh * mh);
    orc_z *E = (orc_z *)malloc(sizeof(orc_z) * mh * mh);
    orc_z *w = (orc_z *)malloc(sizeof(orc_z) * n);
    int rc = 0;
    for (size_t c = 0; c < nvec && rc == 0; ++c) {
        memcpy(w, Vin + c * n, sizeof(orc_z) * n);
        krylov_state s;
        state_init(&s, w, n, m, tol, anorm);
        const double *tcol = ta + (per_column_times ? c * tn : 0);
        for (size_t tt = 0; tt < tn; ++tt) {
            rc = integrate_to(&op, &s, w, tcol[tt], m, tol, anorm, V, Hm, E);
            if (rc) break;
            memcpy(W + (c * tn + tt) * n, w, sizeof(orc_z) * n);
        }
        if (stats && c == 0) {
            stats->anorm = anorm;
            stats->nmult = s.nmult; stats->nexph = s.nexph;
            stats->nscale = s.nscale; stats->nstep = s.nstep;
            stats->nreject = s.nreject; stats->ibrkflag = s.ibrkflag;
            stats->mbrkdwn = s.mbrkdwn; stats->step_min = s.step_min;
            stats->step_max = s.step_max; stats->x_error = s.x_error;
            stats->s_error = s.s_error; stats->hump = s.hump / s.vnorm;
            stats->tbrkdwn = s.tbrkdwn; stats->t_now = s.t_now;
            stats->iflag = rc;
        }
    }
    free(op.coeffz); free(op.wmed); free(V); free(Hm); free(E); free(w);
    return rc;
}

int orc_expv(size_t nspin, size_t nterm, const double *coeff_lst,
             const size_t *nbody_lst, const size_t *pos_i_idx,
             const size_t *pos_i_lst, const size_t *dim_i_lst,
             const size_t *mat_i_idx, const orc_z *mat_i_lst, size_t ham_dim,
             const size_t *nspin_dim, const orc_z *v, size_t klim, size_t tn,
             const double *ta, size_t m, double tol, orc_z *w_seq,
             orc_expv_stats *stats)
{
    return expv_core(nspin, nterm, coeff_lst, nbody_lst, pos_i_idx, pos_i_lst,
                     dim_i_lst, mat_i_idx, mat_i_lst, ham_dim, nspin_dim, v, 1,
                     klim, tn, ta, 0, m, tol, w_seq, stats);
}

int orc_expv_block(size_t nspin, size_t nterm, const double *coeff_lst,
                   const size_t *nbody_lst, const size_t *pos_i_idx,
                   const size_t *pos_i_lst, const size_t *dim_i_lst,
                   const size_t *mat_i_idx, const orc_z *mat_i_lst,
                   size_t ham_dim, const size_t *nspin_dim, const orc_z *V,
                   size_t nvec, size_t klim, size_t tn, const double *ta,
                   size_t m, double tol, orc_z *W_seq)
{
    return expv_core(nspin, nterm, coeff_lst, nbody_lst, pos_i_idx, pos_i_lst,
                     dim_i_lst, mat_i_idx, mat_i_lst, ham_dim, nspin_dim, V,
                     nvec, klim, tn, ta, 1, m, tol, W_seq, NULL);
}

/* ------------------------------------------------------------------------ */
/* spin physics (misc.cpp, DefectCenter.cpp, SpinInteraction*.cpp)           */
/* ------------------------------------------------------------------------ */
void orc_dipole(const double c1[3], const double c2[3], double g1, double g2,
                double out[9])
{
    double r[3] = {c1[0] - c2[0], c1[1] - c2[1], c1[2] - c2[2]};
    double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (d <= 1e-10) { memset(out, 0, 9 * sizeof(double)); return; }
    double nv[3] = {r[0] / d, r[1] / d, r[2] / d};
    double d0 = d * 1e-10;
    double pre = ORC_HBAR * ORC_MU0 / (4.0 * ORC_PI) * (g1 * g2) / (d0 * d0 * d0);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            out[3 * a + b] = pre * ((a == b ? 1.0 : 0.0) - 3.0 * nv[a] * nv[b]);
}

/* spin-1 operators, Spin.cpp:28-95 (column-major 3x3) */
static void spin1_ops(orc_z sx[9], orc_z sy[9], orc_z sz[9])
{
    double r2 = 1.0 / sqrt(2.0);
    memset(sx, 0, 9 * sizeof(orc_z)); memset(sy, 0, 9 * sizeof(orc_z));
    memset(sz, 0, 9 * sizeof(orc_z));
    /* (row, col) -> row + 3*col */
    sx[0 + 3 * 1] = r2; sx[1 + 3 * 0] = r2; sx[1 + 3 * 2] = r2; sx[2 + 3 * 1] = r2;
    sy[0 + 3 * 1] = -I * r2; sy[1 + 3 * 0] = I * r2;
    sy[1 + 3 * 2] = -I * r2; sy[2 + 3 * 1] = I * r2;
    sz[0] = 1.0; sz[8] = -1.0;
}

/* cyclic complex Jacobi for a 3x3 Hermitian matrix; eigenvalues ascending */
static void herm3_eig(const orc_z A[9], double ev[3], orc_z Vout[9])
{
    orc_z a[9], v[9];
    memcpy(a, A, sizeof(a));
    memset(v, 0, sizeof(v));
    v[0] = v[4] = v[8] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) off += cabs(a[p + 3 * q]);
        if (off < 1e-300) break;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) {
                orc_z apq = a[p + 3 * q];
                double mag = cabs(apq);
                if (mag == 0) continue;
                double app = creal(a[p + 3 * p]), aqq = creal(a[q + 3 * q]);
                double theta = 0.5 * atan2(2.0 * mag, aqq - app);
                double c = cos(theta), s = sin(theta);
                orc_z ph = apq / mag; /* e^{i phi} */
                /* rotation G: columns p,q: [c, -s*ph; s*conj(ph), c] applied
                 * so that (G^H A G)_pq = 0 */
                orc_z gpp = c, gpq = s * ph, gqp = -s * conj(ph), gqq = c;
                for (int k = 0; k < 3; ++k) { /* A <- A G */
                    orc_z akp = a[k + 3 * p], akq = a[k + 3 * q];
                    a[k + 3 * p] = akp * gpp + akq * gqp;
                    a[k + 3 * q] = akp * gpq + akq * gqq;
                    orc_z vkp = v[k + 3 * p], vkq = v[k + 3 * q];
                    v[k + 3 * p] = vkp * gpp + vkq * gqp;
                    v[k + 3 * q] = vkp * gpq + vkq * gqq;
                }
                for (int k = 0; k < 3; ++k) { /* A <- G^H A */
                    orc_z apk = a[p + 3 * k], aqk = a[q + 3 * k];
                    a[p + 3 * k] = conj(gpp) * apk + conj(gqp) * aqk;
                    a[q + 3 * k] = conj(gpq) * apk + conj(gqq) * aqk;
                }
            }
    }
    int idx[3] = {0, 1, 2};
    double d[3] = {creal(a[0]), creal(a[4]), creal(a[8])};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[idx[j]] < d[idx[i]]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
    for (int i = 0; i < 3; ++i) {
        ev[i] = d[idx[i]];
        for (int k = 0; k < 3; ++k) Vout[k + 3 * i] = v[k + 3 * idx[i]];
    }
}

void orc_nv_states(const double B[3], double eval[3], double svec[9])
{
    /* NVe: multiplicity 3, gamma -1.760859708e11, omegaQ 2.87e3 MHz
     * (SpinData.cpp:8) */
    const double gamma = -1.760859708e11;
    const double D = 2.87e3 * 2.0 * ORC_PI * 1e6;
    orc_z sx[9], sy[9], sz[9], s111[9], H[9];
    spin1_ops(sx, sy, sz);
    for (int i = 0; i < 9; ++i) s111[i] = (sx[i] + sy[i] + sz[i]) / sqrt(3.0);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            orc_z acc = 0;
            for (int k = 0; k < 3; ++k) acc += s111[r + 3 * k] * s111[k + 3 * c];
            H[r + 3 * c] = D * acc + gamma * (B[0] * sx[r + 3 * c] +
                                              B[1] * sy[r + 3 * c] +
                                              B[2] * sz[r + 3 * c]);
        }
    orc_z V[9];
    herm3_eig(H, eval, V);
    const orc_z *ops[3] = {sx, sy, sz};
    for (int st = 0; st < 3; ++st)
        for (int a = 0; a < 3; ++a) {
            orc_z acc = 0;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    acc += conj(V[r + 3 * st]) * ops[a][r + 3 * c] * V[c + 3 * st];
            svec[3 * st + a] = creal(acc);
        }
}

/* spin-1/2 operators (Spin.cpp:28-70), column-major 2x2 */
static void half_ops(int a, orc_z out[4])
{
    memset(out, 0, 4 * sizeof(orc_z));
    if (a == 0) { out[1] = 0.5; out[2] = 0.5; }
    else if (a == 1) { out[1] = 0.5 * I; out[2] = -0.5 * I; }
    else { out[0] = 0.5; out[3] = -0.5; }
}

size_t orc_cluster_hamiltonian(size_t k, const double *coords, double g,
                               const double B[3], const double cc[3], double gc,
                               const double sv[3], double *coeff,
                               size_t *nbody, size_t *pos_i_idx,
                               size_t *pos_list, size_t *dim_list,
                               size_t *mat_offset, orc_z *matC)
{
    size_t nt = 0, nb = 0;
#define ADD_TERM(cf, n, p0, a0, p1, a1)                                      \
    do {                                                                       \
        coeff[nt] = (cf); nbody[nt] = (n); pos_i_idx[nt] = nb;                 \
        pos_list[nb] = (p0); dim_list[nb] = 2; mat_offset[nb] = 4 * nb;        \
        half_ops((a0), matC + 4 * nb); nb++;                                   \
        if ((n) == 2) {                                                        \
            pos_list[nb] = (p1); dim_list[nb] = 2; mat_offset[nb] = 4 * nb;    \
            half_ops((a1), matC + 4 * nb); nb++;                               \
        }                                                                      \
        nt++;                                                                  \
    } while (0)
    /* SpinDipolarInteraction: pairs i<j, components xx,xy,...,zz */
    for (size_t i = 0; i < k; ++i)
        for (size_t j = i + 1; j < k; ++j) {
            double d9[9];
            orc_dipole(coords + 3 * i, coords + 3 * j, g, g, d9);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    if (d9[3 * a + b] != 0.0) ADD_TERM(d9[3 * a + b], 2, i, a, j, b);
        }
    /* SpinZeemanInteraction: -g B_a (quadrupole terms are zero for 13C) */
    for (size_t i = 0; i < k; ++i)
        for (int a = 0; a < 3; ++a) {
            double c = -g * B[a];
            if (c != 0.0) ADD_TERM(c, 1, i, a, 0, 0);
        }
    /* DipolarField: (D . <S>)_a */
    for (size_t i = 0; i < k; ++i) {
        double d9[9];
        orc_dipole(coords + 3 * i, cc, g, gc, d9);
        for (int a = 0; a < 3; ++a) {
            /* reshape(dip,3,3) is column-major; the tensor is symmetric */
            double f = d9[a] * sv[0] + d9[3 + a] * sv[1] + d9[6 + a] * sv[2];
            if (f != 0.0) ADD_TERM(f, 1, i, a, 0, 0);
        }
    }
#undef ADD_TERM
    pos_i_idx[nt] = nb;
    mat_offset[nb] = 4 * nb;
    return nt;
}

void orc_dense_hamiltonian(size_t nspin, size_t nterm, const double *coeff,
                           const size_t *nbody, const size_t *pos_i_idx,
                           const size_t *pos_list, const size_t *dim_list,
                           const size_t *mat_offset, const orc_z *matC,
                           const size_t *spin_dim, orc_z *Hout)
{
    size_t D = 1;
    for (size_t i = 0; i < nspin; ++i) D *= spin_dim[i];
    orc_z *cz = (orc_z *)malloc(sizeof(orc_z) * (nterm ? nterm : 1));
    for (size_t t = 0; t < nterm; ++t) cz[t] = coeff[t];
    orc_z *e = (orc_z *)calloc(D, sizeof(orc_z));
    orc_z *wm = (orc_z *)malloc(sizeof(orc_z) * D);
    for (size_t c = 0; c < D; ++c) {
        memset(e, 0, sizeof(orc_z) * D);
        e[c] = 1.0;
        orc_hamvec(nspin, nterm, cz, nbody, pos_i_idx, pos_list, dim_list,
                   mat_offset, matC, D, spin_dim, e, Hout + c * D, wm);
    }
    free(cz); free(e); free(wm);
}

void orc_cpmg_intervals(int n, double *frac)
{
    double prev = 0.0;
    for (int i = 0; i < n; ++i) {
        double t = (2.0 * i + 1.0) / (2.0 * n);
        frac[i] = t - prev;
        prev = t;
    }
    frac[n] = 1.0 - prev;
}

/* ------------------------------------------------------------------------ */
/* dense cluster propagation                                                  */
/* ------------------------------------------------------------------------ */
static void expm_scaled(size_t D, const orc_z *M, orc_z pref, orc_z *out)
{
    /* MatExp::pade_exp_mat (MatExp.cpp:29-77): res = pref*M, zgpadm(t=1) */
    size_t DD = D * D;
    orc_z *S = (orc_z *)malloc(sizeof(orc_z) * DD);
    for (size_t i = 0; i < DD; ++i) S[i] = pref * M[i];
    if (orc_padm(6, (int)D, 1.0, S, (int)D, out, NULL) != 0) {
        memset(out, 0, sizeof(orc_z) * DD); /* the reference returns zeros */
    }
    free(S);
}

void orc_coherence_hilbert(size_t D, const orc_z *H0, const orc_z *H1,
                           int pulse_num, size_t nT, double dt, double *L)
{
    int nseg = pulse_num + 1;
    double frac[64];
    orc_cpmg_intervals(pulse_num, frac);
    size_t DD = D * D;
    /* E[b][j]: branch b segment j propagator, P[b][j]: its running power */
    orc_z **E = (orc_z **)malloc(sizeof(orc_z *) * 2 * nseg);
    orc_z **P = (orc_z **)malloc(sizeof(orc_z *) * 2 * nseg);
    for (int b = 0; b < 2; ++b)
        for (int j = 0; j < nseg; ++j) {
            const orc_z *H = ((j + b) % 2 == 0) ? H0 : H1;
            E[b * nseg + j] = (orc_z *)malloc(sizeof(orc_z) * DD);
            P[b * nseg + j] = (orc_z *)malloc(sizeof(orc_z) * DD);
            expm_scaled(D, H, -I * frac[j] * dt, E[b * nseg + j]);
            memcpy(P[b * nseg + j], E[b * nseg + j], sizeof(orc_z) * DD);
        }
    orc_z *B[2], *T = (orc_z *)malloc(sizeof(orc_z) * DD);
    B[0] = (orc_z *)malloc(sizeof(orc_z) * DD);
    B[1] = (orc_z *)malloc(sizeof(orc_z) * DD);
    L[0] = 1.0;
    for (size_t i = 1; i < nT; ++i) {
        for (int b = 0; b < 2; ++b) {
            /* B = P_0 P_1 ... P_n (segment 0 leftmost) */
            memcpy(B[b], P[b * nseg + 0], sizeof(orc_z) * DD);
            for (int j = 1; j < nseg; ++j) {
                zgemm_nn((int)D, (int)D, (int)D, 1.0, B[b], (int)D,
                         P[b * nseg + j], (int)D, 0, T, (int)D);
                memcpy(B[b], T, sizeof(orc_z) * DD);
            }
            for (int j = 0; j < nseg; ++j) { /* P <- E P */
                zgemm_nn((int)D, (int)D, (int)D, 1.0, E[b * nseg + j], (int)D,
                         P[b * nseg + j], (int)D, 0, T, (int)D);
                memcpy(P[b * nseg + j], T, sizeof(orc_z) * DD);
            }
        }
        orc_z tr = 0;
        for (size_t q = 0; q < DD; ++q) tr += conj(B[1][q]) * B[0][q];
        L[i] = creal(tr) / (double)D;
    }
    for (int q = 0; q < 2 * nseg; ++q) { free(E[q]); free(P[q]); }
    free(E); free(P); free(B[0]); free(B[1]); free(T);
}

void orc_coherence_state(size_t D, const orc_z *H0, const orc_z *H1, int pulse_num,
                         size_t nT, double dt, size_t b, double *L)
{
    /* SingleSampleCCE::cluster_evolution (single_sample_cce.cpp:48-72): two
     * PiecewiseFullMatrixVectorEvolution runs (QuantumEvolutionAlgorithm.cpp:
     * 60-83) of the basis state e_b, through riffle(H0, H1) and riffle(H1, H0);
     * calc_observables (:118-127): L_i = Re <state1_i, state2_i>. */
    int nseg = pulse_num + 1;
    double frac[64];
    orc_cpmg_intervals(pulse_num, frac);
    size_t DD = D * D;
    orc_z **E = (orc_z **)malloc(sizeof(orc_z *) * 2 * nseg);
    orc_z **P = (orc_z **)malloc(sizeof(orc_z *) * 2 * nseg);
    for (int a = 0; a < 2; ++a)
        for (int j = 0; j < nseg; ++j) {
            const orc_z *H = ((j + a) % 2 == 0) ? H0 : H1;
            E[a * nseg + j] = (orc_z *)malloc(sizeof(orc_z) * DD);
            P[a * nseg + j] = (orc_z *)malloc(sizeof(orc_z) * DD);
            expm_scaled(D, H, -I * frac[j] * dt, E[a * nseg + j]);
            memcpy(P[a * nseg + j], E[a * nseg + j], sizeof(orc_z) * DD);
        }
    orc_z *v[2], *T = (orc_z *)malloc(sizeof(orc_z) * DD), *u = (orc_z *)malloc(sizeof(orc_z) * D);
    v[0] = (orc_z *)malloc(sizeof(orc_z) * D);
    v[1] = (orc_z *)malloc(sizeof(orc_z) * D);
    L[0] = 1.0;
    for (size_t i = 1; i < nT; ++i) {
        for (int a = 0; a < 2; ++a) {
            memset(v[a], 0, sizeof(orc_z) * D);
            v[a][b] = 1.0;
            for (int j = 0; j < nseg; ++j) { /* state = P_j state; P_j <- E_j P_j */
                zgemm_nn((int)D, 1, (int)D, 1.0, P[a * nseg + j], (int)D, v[a], (int)D, 0, u, (int)D);
                memcpy(v[a], u, sizeof(orc_z) * D);
                zgemm_nn((int)D, (int)D, (int)D, 1.0, E[a * nseg + j], (int)D, P[a * nseg + j],
                         (int)D, 0, T, (int)D);
                memcpy(P[a * nseg + j], T, sizeof(orc_z) * DD);
            }
        }
        orc_z acc = 0;
        for (size_t q = 0; q < D; ++q) acc += conj(v[0][q]) * v[1][q];
        L[i] = creal(acc);
    }
    for (int q = 0; q < 2 * nseg; ++q) { free(E[q]); free(P[q]); }
    free(E); free(P); free(v[0]); free(v[1]); free(T); free(u);
}

void orc_coherence_liouville(size_t k, const orc_z *H0, const orc_z *H1,
                             int pulse_num, size_t nT, double dt,
                             double dephase_rate, const double axis[3],
                             const double pol[3], double *L)
{
    size_t D = (size_t)1 << k, D2 = D * D, DD2 = D2 * D2;
    int nseg = pulse_num + 1;
    double frac[64];
    orc_cpmg_intervals(pulse_num, frac);
    /* superoperators in vec (column-major) ordering:
     * Sharp(H) <-> rho H = (H^T (x) I), Flat(H) <-> H rho = (I (x) H) */
    orc_z *LA = (orc_z *)calloc(DD2, sizeof(orc_z));
    orc_z *LB = (orc_z *)calloc(DD2, sizeof(orc_z));
    for (size_t c1 = 0; c1 < D; ++c1)        /* column of rho (input)  */
        for (size_t r1 = 0; r1 < D; ++r1) {  /* row of rho (input)     */
            size_t in = r1 + D * c1;
            for (size_t c0 = 0; c0 < D; ++c0) { /* (rho H)_{r1,c0} += rho_{r1,c1} H_{c1,c0} */
                size_t out = r1 + D * c0;
                LA[out + D2 * in] += H0[c1 + D * c0];
                LB[out + D2 * in] += H1[c1 + D * c0];
            }
            for (size_t r0 = 0; r0 < D; ++r0) { /* (H rho)_{r0,c1} */
                size_t out = r0 + D * c1;
                LA[out + D2 * in] -= H1[r0 + D * r1];
                LB[out + D2 * in] -= H0[r0 + D * r1];
            }
        }
    if (dephase_rate != 0.0) {
        /* i*rate*(sigma_n rho sigma_n - rho) per spin,
         * SpinInteractionComponent.cpp:285-304 */
        double nn = sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
        double nx = axis[0] / nn, ny = axis[1] / nn, nz = axis[2] / nn;
        orc_z sg[4] = {nz, nx + I * ny, nx - I * ny, -nz}; /* column-major */
        for (size_t s = 0; s < k; ++s) {
            size_t stride = (size_t)1 << (k - 1 - s); /* spin 0 most significant */
            for (size_t c1 = 0; c1 < D; ++c1)
                for (size_t r1 = 0; r1 < D; ++r1) {
                    size_t in = r1 + D * c1;
                    int br = (int)((r1 / stride) & 1), bc = (int)((c1 / stride) & 1);
                    for (int ar = 0; ar < 2; ++ar)
                        for (int ac = 0; ac < 2; ++ac) {
                            size_t r0 = (size_t)((long)r1 + (long)(ar - br) * (long)stride);
                            size_t c0 = (size_t)((long)c1 + (long)(ac - bc) * (long)stride);
                            /* (s rho s)_{r0,c0} = s_{r0 r1} rho_{r1 c1} s_{c1 c0} */
                            orc_z val = sg[ar + 2 * br] * sg[bc + 2 * ac];
                            orc_z cf = I * dephase_rate * val;
                            LA[(r0 + D * c0) + D2 * in] += cf;
                            LB[(r0 + D * c0) + D2 * in] += cf;
                        }
                    LA[in + D2 * in] -= I * dephase_rate;
                    LB[in + D2 * in] -= I * dephase_rate;
                }
        }
    }
    /* rho0 = I/D + sum_i p.S_i (vectorised) */
    orc_z *rho0 = (orc_z *)calloc(D2, sizeof(orc_z));
    for (size_t d = 0; d < D; ++d) rho0[d + D * d] = 1.0 / (double)D;
    for (size_t s = 0; s < k; ++s) {
        size_t stride = (size_t)1 << (k - 1 - s);
        for (int a = 0; a < 3; ++a) {
            if (pol[a] == 0.0) continue;
            orc_z op[4];
            half_ops(a, op);
            for (size_t c = 0; c < D; ++c)
                for (size_t r = 0; r < D; ++r) {
                    if ((r & ~stride) != (c & ~stride)) continue;
                    int br = (int)((r / stride) & 1), bc = (int)((c / stride) & 1);
                    rho0[r + D * c] += pol[a] * op[br + 2 * bc];
                }
        }
    }
    orc_z **E = (orc_z **)malloc(sizeof(orc_z *) * nseg);
    orc_z **P = (orc_z **)malloc(sizeof(orc_z *) * nseg);
    for (int j = 0; j < nseg; ++j) {
        E[j] = (orc_z *)malloc(sizeof(orc_z) * DD2);
        P[j] = (orc_z *)malloc(sizeof(orc_z) * DD2);
        expm_scaled(D2, (j % 2 == 0) ? LA : LB, -I * frac[j] * dt, E[j]);
        memcpy(P[j], E[j], sizeof(orc_z) * DD2);
    }
    orc_z *st = (orc_z *)malloc(sizeof(orc_z) * D2);
    orc_z *st2 = (orc_z *)malloc(sizeof(orc_z) * D2);
    orc_z *T = (orc_z *)malloc(sizeof(orc_z) * DD2);
    for (size_t i = 0; i < nT; ++i) {
        memcpy(st, rho0, sizeof(orc_z) * D2);
        if (i > 0)
            for (int j = 0; j < nseg; ++j) {
                zgemm_nn((int)D2, 1, (int)D2, 1.0, P[j], (int)D2, st, (int)D2, 0,
                         st2, (int)D2);
                memcpy(st, st2, sizeof(orc_z) * D2);
                zgemm_nn((int)D2, (int)D2, (int)D2, 1.0, E[j], (int)D2, P[j],
                         (int)D2, 0, T, (int)D2);
                memcpy(P[j], T, sizeof(orc_z) * DD2);
            }
        orc_z acc = 0;
        for (size_t q = 0; q < D2; ++q) acc += conj((double)D * rho0[q]) * st[q];
        L[i] = creal(acc);
    }
    for (int j = 0; j < nseg; ++j) { free(E[j]); free(P[j]); }
    free(E); free(P); free(st); free(st2); free(T); free(rho0); free(LA); free(LB);
}

/* ------------------------------------------------------------------------ */
/* cluster enumeration (SpinCollection.cpp, SpinClusterAlgorithm.cpp,        */
/* SpinClusterIndex.cpp, SpinCluster.cpp)                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    size_t count;
    size_t *idx;      /* count x (order+1) sorted spin indices */
    size_t *par_off;  /* count+1 offsets into par */
    size_t *par;      /* direct parent positions (sorted, unique) */
} orc_order;

struct orc_enum {
    int max_order;
    orc_order *ord;
    size_t **sub_off; /* per order: closure offsets */
    size_t **sub;     /* per order: closure (order,pos) pairs */
};

typedef struct {
    size_t off; /* offset of the w sorted spin indices in the row store */
    size_t parent;
} gen_row;

static size_t g_cmp_width;
static const size_t *g_cmp_store;
static int cmp_gen(const void *a, const void *b)
{
    const gen_row *x = (const gen_row *)a, *y = (const gen_row *)b;
    const size_t *xs = g_cmp_store + x->off, *ys = g_cmp_store + y->off;
    for (size_t i = 0; i < g_cmp_width; ++i)
        if (xs[i] != ys[i]) return xs[i] < ys[i] ? -1 : 1;
    if (x->parent != y->parent) return x->parent < y->parent ? -1 : 1;
    return 0;
}

orc_enum *orc_enumerate(size_t nspin, const double *coords, double cutoff,
                        int max_order)
{
    orc_enum *e = (orc_enum *)calloc(1, sizeof(orc_enum));
    e->max_order = max_order;
    e->ord = (orc_order *)calloc((size_t)max_order, sizeof(orc_order));
    e->sub_off = (size_t **)calloc((size_t)max_order, sizeof(size_t *));
    e->sub = (size_t **)calloc((size_t)max_order, sizeof(size_t *));
    /* connection matrix: dist <= cutoff, diagonal zeroed */
    unsigned char *C = (unsigned char *)calloc(nspin * nspin, 1);
    for (size_t i = 0; i < nspin; ++i)
        for (size_t j = i + 1; j < nspin; ++j) {
            double dx = coords[3 * i] - coords[3 * j];
            double dy = coords[3 * i + 1] - coords[3 * j + 1];
            double dz = coords[3 * i + 2] - coords[3 * j + 2];
            double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (d <= cutoff) C[i * nspin + j] = C[j * nspin + i] = 1;
        }
    if (max_order < 1) { free(C); return e; }
    /* order 0: identity rows */
    orc_order *o0 = &e->ord[0];
    o0->count = nspin;
    o0->idx = (size_t *)malloc(sizeof(size_t) * (nspin ? nspin : 1));
    o0->par_off = (size_t *)calloc(nspin + 1, sizeof(size_t));
    o0->par = NULL;
    for (size_t i = 0; i < nspin; ++i) o0->idx[i] = i;
    unsigned char *mark = (unsigned char *)malloc(nspin ? nspin : 1);
    for (int o = 1; o < max_order; ++o) {
        orc_order *pv = &e->ord[o - 1], *cu = &e->ord[o];
        size_t w = (size_t)o + 1, pw = (size_t)o;
        size_t cap = 1024, ng = 0;
        gen_row *rows = (gen_row *)malloc(sizeof(gen_row) * cap);
        size_t *store = NULL;
        size_t scap = 0, sused = 0;
        for (size_t p = 0; p < pv->count; ++p) {
            const size_t *ps = pv->idx + p * pw;
            memset(mark, 0, nspin);
            for (size_t a = 0; a < pw; ++a)
                for (size_t j = 0; j < nspin; ++j)
                    if (C[ps[a] * nspin + j]) mark[j] = 1;
            for (size_t j = 0; j < nspin; ++j) {
                if (!mark[j]) continue;
                int inpar = 0;
                for (size_t a = 0; a < pw; ++a) if (ps[a] == j) inpar = 1;
                if (inpar) continue;
                if (ng == cap) { cap *= 2; rows = (gen_row *)realloc(rows, sizeof(gen_row) * cap); }
                if (sused + w > scap) {
                    scap = scap ? scap * 2 : 4096;
                    while (scap < sused + w) scap *= 2;
                    store = (size_t *)realloc(store, sizeof(size_t) * scap);
                }
                size_t *dst = store + sused;
                size_t q = 0, a = 0;
                int put = 0;
                while (q < w) { /* sorted merge of parent + j */
                    if (!put && (a == pw || j < ps[a])) { dst[q++] = j; put = 1; }
                    else dst[q++] = ps[a++];
                }
                rows[ng].off = sused;
                rows[ng].parent = p;
                ng++;
                sused += w;
            }
        }
        g_cmp_width = w;
        g_cmp_store = store;
        qsort(rows, ng, sizeof(gen_row), cmp_gen);
        /* unique clusters, parent lists */
        size_t nu = 0;
#define ROWS(r) (store + rows[(r)].off)
        for (size_t r = 0; r < ng; ++r)
            if (r == 0 || memcmp(ROWS(r), ROWS(r - 1), sizeof(size_t) * w)) nu++;
        cu->count = nu;
        cu->idx = (size_t *)malloc(sizeof(size_t) * (nu > 0 ? nu * w : 1));
        cu->par_off = (size_t *)calloc(nu + 1, sizeof(size_t));
        cu->par = (size_t *)malloc(sizeof(size_t) * (ng ? ng : 1));
        size_t u = (size_t)-1, np = 0;
        for (size_t r = 0; r < ng; ++r) {
            if (r == 0 || memcmp(ROWS(r), ROWS(r - 1), sizeof(size_t) * w)) {
                u++;
                memcpy(cu->idx + u * w, ROWS(r), sizeof(size_t) * w);
                cu->par_off[u] = np;
            }
            if (np == cu->par_off[u] || cu->par[np - 1] != rows[r].parent)
                cu->par[np++] = rows[r].parent;
        }
#undef ROWS
        if (nu) cu->par_off[nu] = np;
        free(rows);
        free(store);
        if (nu == 0) { /* nothing grows further */
            for (int q = o + 1; q < max_order; ++q) {
                e->ord[q].count = 0;
                e->ord[q].par_off = (size_t *)calloc(1, sizeof(size_t));
            }
            break;
        }
    }
    free(mark);
    free(C);
    /* transitive closures (getSubClusters), bottom-up; pairs (order,pos) */
    for (int o = 0; o < max_order; ++o) {
        orc_order *cu = &e->ord[o];
        e->sub_off[o] = (size_t *)calloc(cu->count + 1, sizeof(size_t));
        size_t cap = 256, used = 0;
        size_t *buf = (size_t *)malloc(sizeof(size_t) * cap);
        size_t tmpcap = 256;
        size_t *tmp = (size_t *)malloc(sizeof(size_t) * tmpcap);
        for (size_t c = 0; c < cu->count; ++c) {
            size_t nt = 0;
            if (o > 0) {
                for (size_t q = cu->par_off[c]; q < cu->par_off[c + 1]; ++q) {
                    size_t p = cu->par[q];
                    size_t need = 2 + (e->sub_off[o - 1][p + 1] - e->sub_off[o - 1][p]) * 2;
                    while (nt * 2 + need > tmpcap) { tmpcap *= 2; tmp = (size_t *)realloc(tmp, sizeof(size_t) * tmpcap); }
                    tmp[2 * nt] = (size_t)(o - 1); tmp[2 * nt + 1] = p; nt++;
                    for (size_t s = e->sub_off[o - 1][p]; s < e->sub_off[o - 1][p + 1]; ++s) {
                        tmp[2 * nt] = e->sub[o - 1][2 * s];
                        tmp[2 * nt + 1] = e->sub[o - 1][2 * s + 1];
                        nt++;
                    }
                }
                /* sort pairs + unique */
                for (size_t a = 1; a < nt; ++a) {
                    size_t k0 = tmp[2 * a], k1 = tmp[2 * a + 1];
                    size_t b = a;
                    while (b > 0 && (tmp[2 * (b - 1)] > k0 ||
                                     (tmp[2 * (b - 1)] == k0 && tmp[2 * (b - 1) + 1] > k1))) {
                        tmp[2 * b] = tmp[2 * (b - 1)]; tmp[2 * b + 1] = tmp[2 * (b - 1) + 1]; b--;
                    }
                    tmp[2 * b] = k0; tmp[2 * b + 1] = k1;
                }
                size_t nu = 0;
                for (size_t a = 0; a < nt; ++a)
                    if (nu == 0 || tmp[2 * (nu - 1)] != tmp[2 * a] || tmp[2 * (nu - 1) + 1] != tmp[2 * a + 1]) {
                        tmp[2 * nu] = tmp[2 * a]; tmp[2 * nu + 1] = tmp[2 * a + 1]; nu++;
                    }
                nt = nu;
            }
            while (used + 2 * nt > cap) { cap *= 2; buf = (size_t *)realloc(buf, sizeof(size_t) * cap); }
            memcpy(buf + used, tmp, sizeof(size_t) * 2 * nt);
            e->sub_off[o][c] = used / 2;
            used += 2 * nt;
        }
        e->sub_off[o][cu->count] = used / 2;
        e->sub[o] = buf;
        free(tmp);
    }
    return e;
}

size_t orc_enum_count(const orc_enum *e, int order)
{
    if (order < 0 || order >= e->max_order) return 0;
    return e->ord[order].count;
}

void orc_enum_cluster(const orc_enum *e, int order, size_t idx, size_t *out)
{
    memcpy(out, e->ord[order].idx + idx * (size_t)(order + 1),
           sizeof(size_t) * (size_t)(order + 1));
}

size_t orc_enum_parents(const orc_enum *e, int order, size_t idx, size_t *out,
                        size_t cap)
{
    const orc_order *o = &e->ord[order];
    if (order == 0) return 0;
    size_t n = o->par_off[idx + 1] - o->par_off[idx];
    for (size_t i = 0; i < n && i < cap; ++i) out[i] = o->par[o->par_off[idx] + i];
    return n;
}

size_t orc_enum_subclusters(const orc_enum *e, int order, size_t idx,
                            size_t *out, size_t cap)
{
    size_t a = e->sub_off[order][idx], b = e->sub_off[order][idx + 1];
    for (size_t i = a; i < b && (i - a) < cap; ++i) {
        out[2 * (i - a)] = e->sub[order][2 * i];
        out[2 * (i - a) + 1] = e->sub[order][2 * i + 1];
    }
    return b - a;
}

void orc_enum_free(orc_enum *e)
{
    if (!e) return;
    for (int o = 0; o < e->max_order; ++o) {
        free(e->ord[o].idx); free(e->ord[o].par_off); free(e->ord[o].par);
        free(e->sub_off[o]); free(e->sub[o]);
    }
    free(e->ord); free(e->sub_off); free(e->sub); free(e);
}

void orc_cce_reduce(const orc_enum *e, int max_order, size_t nT,
                    double *const *Lraw, double *const *Ltilde,
                    double *final_each, double *final_cum)
{
    double *cum = (double *)malloc(sizeof(double) * nT);
    double *acc = (double *)malloc(sizeof(double) * nT);
    for (size_t t = 0; t < nT; ++t) cum[t] = 1.0;
    for (int o = 0; o < max_order; ++o) {
        size_t cnt = orc_enum_count(e, o);
        for (size_t j = 0; j < cnt; ++j) {
            double *res = Ltilde[o] + j * nT;
            memcpy(res, Lraw[o] + j * nT, sizeof(double) * nT);
            for (size_t s = e->sub_off[o][j]; s < e->sub_off[o][j + 1]; ++s) {
                const double *sub = Ltilde[e->sub[o][2 * s]] + e->sub[o][2 * s + 1] * nT;
                for (size_t t = 0; t < nT; ++t) res[t] = res[t] / sub[t];
            }
        }
        for (size_t t = 0; t < nT; ++t) acc[t] = 1.0;
        for (size_t j = 0; j < cnt; ++j)
            for (size_t t = 0; t < nT; ++t) acc[t] = acc[t] * Ltilde[o][j * nT + t];
        for (size_t t = 0; t < nT; ++t) {
            final_each[o * nT + t] = acc[t];
            cum[t] = cum[t] * acc[t];
            final_cum[o * nT + t] = cum[t];
        }
    }
    free(cum); free(acc);
}
