/*
 * CPU oracle for the Parament equiprop path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C99 double-precision complex arithmetic, the
 * algorithm that the reference library runs on the GPU with cuBLAS.  It is
 * the checker for the CUDA library: only the test-suite, the smoke check and
 * the CPU-baseline leg of the benchmark load it.  The product never calls it.
 *
 * Reference anchors (paths inside the parament project):
 *   - norm bound          src/cuda/mathhelper.cpp:82-114, used at src/cuda/parament.cpp:279-287
 *   - order tables        src/cuda/parament.cpp:723-766
 *   - Bessel coefficients src/cuda/mathhelper.cpp:35-80, src/cuda/parament.cpp:373-409
 *   - quadrature weights  src/cuda/control_expansion.cu:27-170
 *   - commutator stack    src/cuda/parament.cpp:289-359 (pair slots re-indexed, see below)
 *   - expansion           src/cuda/parament.cpp:486-563
 *   - Clenshaw recurrence src/cuda/parament.cpp:569-652
 *   - tree product        src/cuda/parament.cpp:657-718
 *   - driver              src/cuda/parament.cpp:791-851
 *
 * Matrices are row-major (C order), complex numbers interleaved (re, im), as
 * at the reference API.  cuBLAS sees these buffers as column-major, so the
 * reference's GEMM "D1 <- s*X*D0 + beta*D1" means D1 = s*D0*X + beta*D1 in
 * row-major terms, and its tree level W_i = R_2i * R_2i+1 means
 * W_i = U_(2i+1) * U_(2i): the later step stands on the left.
 *
 * Deliberate deviation: the reference stores the Magnus pair commutator of
 * controls (j, i), j < i, in slot 2K+(i-1)+j, which collides for K >= 4
 * (src/cuda/parament.cpp:330, src/cuda/control_expansion.cu:53).  This oracle
 * uses the collision-free triangular slot 2K + i(i-1)/2 + j.  For K <= 3 the
 * two indexings coincide.
 */
#define _DEFAULT_SOURCE 1 /* jn() is an XSI extension of libm */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* Rounds the real and imaginary parts to float: the complex64 context keeps
 * its Bessel coefficients, scale factor and step weights in float
 * (src/cuda/mathhelper.cpp:19-32, src/cuda/parament.cpp:583-584,
 * src/cuda/control_expansion.cu:27-60).  Those roundings repeat identically at
 * every step, so they shift the result coherently; the oracle reproduces them
 * and keeps everything else in FP64. */
static cplx round_c64(cplx z) { return (double)(float)creal(z) + I * (double)(float)cimag(z); }

enum { PR_NONE = 0, PR_MIDPOINT = 0x01000000, PR_SIMPSON = 0x02000000 };

/* Order tables: thresholds on Hnorm*dt and the odd orders they select.
 * src/cuda/parament.cpp:723-766.  Returns -1 when Hnorm*dt is too large. */
static const double fp32_limits[14] = {
    0.032516793, 0.219062571, 0.619625593, 1.218059203, 1.979888284, 2.873301187, 3.872963682,
    4.959398466, 6.117657121, 7.336154907, 8.605792444, 9.919320831, 11.27088616, 12.65570085};
static const double fp64_limits[20] = {
    0.000213616, 0.00768149, 0.0501474, 0.162592, 0.368382, 0.676861, 1.08784,
    1.59605,     2.19402,    2.87366,   3.62716,  4.44725,  5.3274,   6.26179,
    7.2453,      8.27338,    9.34206,   10.4478,  11.5875,  12.7584};

int pr_select_cycles(int fp64, double hnorm, double dt) {
    const double *lim = fp64 ? fp64_limits : fp32_limits;
    int n = fp64 ? 20 : 14;
    double v = hnorm * dt;
    for (int i = 0; i < n; ++i)
        if (v <= lim[i]) return 3 + 2 * i;
    return -1;
}

/* Maximum absolute row sum, accumulated in double.  For a single-precision
 * context the element modulus is formed in float, as the reference does with
 * its float complex type (src/cuda/mathhelper.cpp:82-98). */
double pr_onenorm(const cplx *m, unsigned d, int single) {
    double best = 0.0;
    for (unsigned i = 0; i < d; ++i) {
        double sum = 0.0;
        for (unsigned j = 0; j < d; ++j) {
            cplx z = m[(size_t)i * d + j];
            if (single)
                sum += (double)hypotf((float)creal(z), (float)cimag(z));
            else
                sum += hypot(creal(z), cimag(z));
        }
        if (sum > best) best = sum;
    }
    return best;
}

/* J[k] = (-i)^k * J_k(x), k = 0..M  (src/cuda/mathhelper.cpp:35-80). */
void pr_bessel_coeffs(int M, double x, cplx *J) {
    static const cplx ipow[4] = {1.0, -I, -1.0, I};
    for (int k = 0; k <= M; ++k) J[k] = ipow[k % 4] * jn(k, x);
}

/* Number of exponentiated steps after quadrature (src/cuda/parament.cpp:820-831). */
long pr_num_steps(int mode, int magnus, unsigned pts) {
    if (magnus || mode == PR_SIMPSON) return pts >= 1 ? (long)((pts - 1) / 2) : 0;
    if (mode == PR_MIDPOINT) return pts >= 1 ? (long)pts - 1 : 0;
    return pts;
}

/* Number of expansion matrices beside H0 (src/cuda/parament.cpp:535). */
unsigned pr_expansion_count(unsigned K, int magnus) {
    return magnus ? 2 * K + K * (K - 1) / 2 : K;
}

static void matmul(const cplx *A, const cplx *B, cplx *C, unsigned d) {
    /* C = A * B, row-major. */
    memset(C, 0, sizeof(cplx) * d * d);
    for (unsigned i = 0; i < d; ++i)
        for (unsigned k = 0; k < d; ++k) {
            cplx a = A[(size_t)i * d + k];
            const cplx *b = B + (size_t)k * d;
            cplx *c = C + (size_t)i * d;
            for (unsigned j = 0; j < d; ++j) c[j] += a * b[j];
        }
}

/* Expansion stack: slot 0 = H0, slots 1..K = H_k, then (Magnus) K commutators
 * [H0, H_k] and the pair commutators [H_j, H_i] for j < i at triangular slots.
 * src/cuda/parament.cpp:289-359 (orientation worked out for row-major data). */
void pr_build_stack(const cplx *H0, const cplx *H1, unsigned d, unsigned K, int magnus, cplx *stack) {
    size_t dd = (size_t)d * d;
    memcpy(stack, H0, sizeof(cplx) * dd);
    memcpy(stack + dd, H1, sizeof(cplx) * dd * K);
    if (!magnus) return;
    cplx *t1 = malloc(sizeof(cplx) * dd), *t2 = malloc(sizeof(cplx) * dd);
    for (unsigned k = 0; k < K; ++k) {
        const cplx *Hk = H1 + k * dd;
        cplx *dst = stack + (1 + K + k) * dd;
        matmul(H0, Hk, t1, d);
        matmul(Hk, H0, t2, d);
        for (size_t e = 0; e < dd; ++e) dst[e] = t1[e] - t2[e];
    }
    for (unsigned i = 1; i < K; ++i)
        for (unsigned j = 0; j < i; ++j) {
            const cplx *Hi = H1 + i * dd, *Hj = H1 + j * dd;
            cplx *dst = stack + (1 + 2 * K + i * (i - 1) / 2 + j) * dd;
            matmul(Hj, Hi, t1, d);
            matmul(Hi, Hj, t2, d);
            for (size_t e = 0; e < dd; ++e) dst[e] = t1[e] - t2[e];
        }
    free(t1);
    free(t2);
}

/* Weights of step s for the expansion matrices 1..Ke (slot 0, H0, has weight 1).
 * carr holds `amps` arrays of `pts` samples; controls amps..K-1 have zero
 * amplitude.  h is the effective step (2*dt for Simpson and Magnus).
 * src/cuda/control_expansion.cu:27-170. */
void pr_step_weights(const cplx *carr, unsigned pts, unsigned amps, unsigned K, int mode, int magnus,
                     double h, long s, cplx *w) {
    unsigned Ke = pr_expansion_count(K, magnus);
    for (unsigned m = 0; m < Ke; ++m) w[m] = 0.0;
    for (unsigned k = 0; k < K && k < amps; ++k) {
        const cplx *u = carr + (size_t)k * pts;
        if (magnus || mode == PR_SIMPSON)
            w[k] = (u[2 * s] + 4.0 * u[2 * s + 1] + u[2 * s + 2]) / 6.0;
        else if (mode == PR_MIDPOINT)
            w[k] = 0.5 * (u[s] + u[s + 1]);
        else
            w[k] = u[s];
    }
    if (!magnus) return;
    cplx f = I * (h / 12.0);
    for (unsigned k = 0; k < K && k < amps; ++k) {
        const cplx *u = carr + (size_t)k * pts;
        w[K + k] = f * (u[2 * s + 2] - u[2 * s]);
    }
    for (unsigned i = 1; i < K && i < amps; ++i)
        for (unsigned j = 0; j < i; ++j) {
            const cplx *ui = carr + (size_t)i * pts, *uj = carr + (size_t)j * pts;
            w[2 * K + i * (i - 1) / 2 + j] = f * (uj[2 * s] * ui[2 * s + 2] - uj[2 * s + 2] * ui[2 * s]);
        }
}

void pr_assemble(const cplx *stack, unsigned d, unsigned Ke, const cplx *w, cplx *X) {
    size_t dd = (size_t)d * d;
    memcpy(X, stack, sizeof(cplx) * dd);
    for (unsigned m = 0; m < Ke; ++m) {
        const cplx *Hm = stack + (1 + m) * dd;
        for (size_t e = 0; e < dd; ++e) X[e] += w[m] * Hm[e];
    }
}

/* Clenshaw evaluation of J0 + 2 sum_k J[k] T_k(X/Hnorm) with the reference's
 * sequence (src/cuda/parament.cpp:588-648):
 *   b_M = J[M] I;  b_k = s b_(k+1) X - b_(k+2) + J[k] I;  U = s b_1 X - 2 b_2 + J[0] I,
 * s = 2/Hnorm.  work holds 3*d*d entries.  M must be >= 1 and odd. */
void pr_clenshaw(const cplx *X, unsigned d, int M, const cplx *J, double s, cplx *U, cplx *work) {
    size_t dd = (size_t)d * d;
    cplx *b1 = work, *b2 = work + dd, *t = work + 2 * dd;
    memset(b1, 0, sizeof(cplx) * dd);
    memset(b2, 0, sizeof(cplx) * dd);
    for (unsigned i = 0; i < d; ++i) b1[(size_t)i * d + i] = J[M];
    for (int k = M - 1; k >= 0; --k) {
        matmul(b1, X, t, d);
        double beta = (k == 0) ? -2.0 : -1.0;
        for (size_t e = 0; e < dd; ++e) t[e] = s * t[e] + beta * b2[e];
        for (unsigned i = 0; i < d; ++i) t[(size_t)i * d + i] += J[k];
        cplx *old2 = b2;
        b2 = b1;
        b1 = t;
        t = old2;
    }
    memcpy(U, b1, sizeof(cplx) * dd);
}

/* Reference tree over P matrices in place (src/cuda/parament.cpp:677-714):
 * out_i = U_(2i+1) U_(2i); an odd leftover moves up unchanged. */
static void tree_reduce(cplx *mats, long P, unsigned d, int nthreads);

typedef struct {
    const cplx *stack;
    const cplx *carr;
    const cplx *J;
    cplx *U;
    unsigned d, pts, amps, K, Ke;
    int mode, magnus, M, single;
    double h, s;
    long s0, s1;
} step_job;

static void *step_worker(void *arg) {
    step_job *jb = arg;
    size_t dd = (size_t)jb->d * jb->d;
    cplx *w = malloc(sizeof(cplx) * (jb->Ke + 1));
    cplx *X = malloc(sizeof(cplx) * dd);
    cplx *work = malloc(sizeof(cplx) * dd * 3);
    for (long s = jb->s0; s < jb->s1; ++s) {
        pr_step_weights(jb->carr, jb->pts, jb->amps, jb->K, jb->mode, jb->magnus,
                        jb->single ? (double)(float)jb->h : jb->h, s, w);
        if (jb->single)
            for (unsigned m = 0; m < jb->Ke; ++m) w[m] = round_c64(w[m]);
        pr_assemble(jb->stack, jb->d, jb->Ke, w, X);
        pr_clenshaw(X, jb->d, jb->M, jb->J, jb->s, jb->U + s * dd, work);
    }
    free(w);
    free(X);
    free(work);
    return NULL;
}

typedef struct {
    cplx *src, *dst;
    unsigned d;
    long i0, i1;
} pair_job;

static void *pair_worker(void *arg) {
    pair_job *jb = arg;
    size_t dd = (size_t)jb->d * jb->d;
    for (long i = jb->i0; i < jb->i1; ++i)
        matmul(jb->src + (2 * i + 1) * dd, jb->src + (2 * i) * dd, jb->dst + i * dd, jb->d);
    return NULL;
}

static void tree_reduce(cplx *mats, long P, unsigned d, int nthreads) {
    size_t dd = (size_t)d * d;
    if (P <= 1) return;
    cplx *tmp = malloc(sizeof(cplx) * dd * ((P + 1) / 2));
    cplx *rd = mats, *wr = tmp;
    long remain = P;
    pthread_t th[256];
    pair_job jobs[256];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    while (remain > 1) {
        long pairs = remain / 2;
        int nt = nthreads < pairs ? nthreads : (int)pairs;
        for (int t = 0; t < nt; ++t) {
            jobs[t] = (pair_job){rd, wr, d, pairs * t / nt, pairs * (t + 1) / nt};
            if (nt > 1)
                pthread_create(&th[t], NULL, pair_worker, &jobs[t]);
            else
                pair_worker(&jobs[t]);
        }
        if (nt > 1)
            for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
        if (remain % 2) memcpy(wr + pairs * dd, rd + 2 * pairs * dd, sizeof(cplx) * dd);
        remain = pairs + remain % 2;
        cplx *t = rd;
        rd = wr;
        wr = t;
    }
    if (rd != mats) memcpy(mats, rd, sizeof(cplx) * dd);
    free(tmp);
}


/* Full equiprop restatement (src/cuda/parament.cpp:791-851).
 *   single   : 1 = the reference's complex64 context: single-precision order
 *              table, float moduli in the norm, and the float roundings of the
 *              Bessel coefficients, the scale 2/Hnorm and the step weights;
 *              0 = the complex128 context.
 *   M_manual : > 0 forces the Chebyshev order (setIterationCyclesManually).
 *   nthreads : host threads for the step exponentials and each tree level.
 * Returns 0 on success, 70 when the order table overflows, 50 when the
 * quadrature leaves no step, 10 on host allocation failure; *M_used and
 * *hnorm_out report the chosen order and the norm bound. */
int pr_equiprop(const cplx *H0, const cplx *H1, unsigned d, unsigned K, int magnus, int mode, const cplx *carr,
                double dt, unsigned pts, unsigned amps, int single, int M_manual, int nthreads, cplx *out,
                int *M_used, double *hnorm_out) {
    size_t dd = (size_t)d * d;
    double hnorm = pr_onenorm(H0, d, single);
    for (unsigned k = 0; k < K; ++k) hnorm += pr_onenorm(H1 + k * dd, d, single);
    if (hnorm_out) *hnorm_out = hnorm;
    double h = (magnus || mode == PR_SIMPSON) ? 2.0 * dt : dt;
    int M = M_manual > 0 ? M_manual : pr_select_cycles(!single, hnorm, h);
    if (M_used) *M_used = M;
    if (M < 3 && M_manual <= 0) return 70;
    long P = pr_num_steps(mode, magnus, pts);
    if (P <= 0) return 50;
    unsigned Ke = pr_expansion_count(K, magnus);
    cplx *stack = malloc(sizeof(cplx) * dd * (1 + Ke));
    cplx *J = malloc(sizeof(cplx) * (M + 1));
    cplx *U = malloc(sizeof(cplx) * dd * P);
    if (!stack || !J || !U) {
        free(stack);
        free(J);
        free(U);
        return 10;
    }
    pr_build_stack(H0, H1, d, K, magnus, stack);
    pr_bessel_coeffs(M, h * hnorm, J);
    double s = 2.0 / hnorm;
    if (single) {
        for (int k = 0; k <= M; ++k) J[k] = round_c64(J[k]);
        s = (double)(float)s;
    }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    int nt = nthreads < P ? nthreads : (int)P;
    pthread_t th[256];
    step_job jobs[256];
    for (int t = 0; t < nt; ++t) {
        jobs[t] = (step_job){stack, carr, J, U, d, pts, amps, K, Ke, mode, magnus, M, single, h, s, P * t / nt,
                             P * (t + 1) / nt};
        if (nt > 1)
            pthread_create(&th[t], NULL, step_worker, &jobs[t]);
        else
            step_worker(&jobs[t]);
    }
    if (nt > 1)
        for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    tree_reduce(U, P, d, nthreads);
    memcpy(out, U, sizeof(cplx) * dd);
    free(stack);
    free(J);
    free(U);
    return 0;
}

/* Exponentials of the steps [s0, s1) only, written to U (used by tests that
 * compare single steps and by the host-core throughput sample). */
int pr_step_exponentials(const cplx *H0, const cplx *H1, unsigned d, unsigned K, int magnus, int mode,
                         const cplx *carr, double dt, unsigned pts, unsigned amps, int M, double hnorm, long s0,
                         long s1, int nthreads, cplx *U) {
    size_t dd = (size_t)d * d;
    double h = (magnus || mode == PR_SIMPSON) ? 2.0 * dt : dt;
    unsigned Ke = pr_expansion_count(K, magnus);
    cplx *stack = malloc(sizeof(cplx) * dd * (1 + Ke));
    cplx *J = malloc(sizeof(cplx) * (M + 1));
    if (!stack || !J) {
        free(stack);
        free(J);
        return 10;
    }
    pr_build_stack(H0, H1, d, K, magnus, stack);
    pr_bessel_coeffs(M, h * hnorm, J);
    long P = s1 - s0;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    int nt = nthreads < P ? nthreads : (int)P;
    pthread_t th[256];
    step_job jobs[256];
    for (int t = 0; t < nt; ++t) {
        jobs[t] = (step_job){stack, carr, J, U - s0 * dd, d, pts, amps, K, Ke, mode, magnus, M, 0, h, 2.0 / hnorm,
                             s0 + P * t / nt, s0 + P * (t + 1) / nt};
        if (nt > 1)
            pthread_create(&th[t], NULL, step_worker, &jobs[t]);
        else
            step_worker(&jobs[t]);
    }
    if (nt > 1)
        for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    free(stack);
    free(J);
    return 0;
}

/* Ordered product of P matrices with the reference's tree (in place; result in mats[0]). */
void pr_tree_product(cplx *mats, long P, unsigned d, int nthreads) { tree_reduce(mats, P, d, nthreads); }
