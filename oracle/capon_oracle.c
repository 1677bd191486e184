/*
 * FP64 CPU restatement of the reference's Capon/MVDR per-pixel path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA path is checked
 * against (tests, smoke check) and the "port" CPU baseline of the benchmark.
 * The product never links or calls it.
 *
 * Element space follows framework/beamformer/capon/getCaponC.pyx:
 *   snapshot gather            :203-205
 *   band covariance R_full     :207-223
 *   spatial smoothing + conj   :226-242   (R[j,k] = sum_s R_full[s+j,s+k], k>=j)
 *   subarray sums g            :246-255
 *   diagonal loading           :257-262   (R += regCoef*trace(R)/L * I)
 *   solve (Cholesky)           :274       -> framework/linalg/linearSolvec.pyx:259-282
 *   weights / amplitude        :276-283
 *   power (upper-triangle sum) :285-289   (the reference's "zPow", see below)
 * Cholesky / triangular solves follow framework/linalg/matrixDecompc.pyx:19-50
 * and framework/linalg/linearSolvec.pyx:312-346.
 *
 * The reference declares regCoef, K_inv and norm_inv as C float
 * (getCaponC.pyx:79,129-132).  `fp32_scalars=1` reproduces that rounding,
 * `fp32_scalars=0` gives the pure-FP64 definition.
 *
 * Output power.  The reference's zPow sums only the upper triangle of the
 * loaded covariance, because its R has an empty lower triangle
 * (getCaponC.pyx:180, 231-242, 285-289).  Both are returned:
 *   zpow_ref = sum_{i} sum_{j>=i} conj(w_j) R[i,j] w_i        (complex)
 *   P        = w^H R w = 1 / Re(a^H R^-1 a)                    (real, true MVDR power)
 *
 * Beamspace follows the reference GPU default route,
 * framework/beamformer/capon/RealTimeCapon/Capon.cpp:285-410:
 * Butler matrix B (Nb x L) per capon_kernel.cu:47-77 (beam b <= Nb/2 -> DFT bin b,
 * otherwise bin b + L - 2*(Nb/2) - 1; B[b,l] = exp(-j 2 pi bin l / L)/sqrt(L)),
 * element-space loading (buildR_kernel.cu:153-154), R_bs = B R_d B^H,
 * a_bs = B 1, Ria = B^H R_bs^-1 a_bs, then the element-space output step
 * (w = Ria / sum(Ria), z = sum conj(w) g; capon_kernel.cu:338-427).
 * `bs_loading = 1` instead loads after the transform with trace(R_bs)/Nb, the
 * convention of framework/beamformer/capon/getCaponAllC.pyx:376-385.
 * `bs_loading = 2` adds an absolute loading regCoef*I to the normalised R (no
 * reference counterpart: the form with a learnable loading scalar).
 *
 * Forward-backward averaging (`fb = 1`) replaces the element-space covariance
 * by R = (R + J R^T J) / 2 before the loading and any beamspace transform
 * (getCaponAllC.pyx:346-347; getCaponPy_ref.py:103-104;
 * getCaponMatlab_ref.m:90-92 as R = (R + rot90(conj(R), 2)) / 2).
 */
#define _GNU_SOURCE
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

static const double kPi = 3.14159265358979323846;

/* ---- small dense kernels (matrixDecompc.pyx / linearSolvec.pyx) ---------- */

/* Upper Cholesky factor U (row-major n x n) with U^H U = A; reads A's upper
 * triangle only.  matrixDecompc.pyx:19-50 (complex square root of the pivot). */
void oracle_cholesky(const cplx *A, int n, cplx *U)
{
    memset(U, 0, sizeof(cplx) * (size_t)n * n);
    for (int i = 0; i < n; ++i) {
        cplx s = 0;
        for (int k = 0; k < i; ++k) s += U[k * n + i] * conj(U[k * n + i]);
        U[i * n + i] = csqrt(A[i * n + i] - s);
        for (int j = i + 1; j < n; ++j) {
            cplx t = 0;
            for (int k = 0; k < i; ++k) t += conj(U[k * n + i]) * U[k * n + j];
            U[i * n + j] = (A[i * n + j] - t) / U[i * n + i];
        }
    }
}

/* Lower-triangular solve A x = b (linearSolvec.pyx:312-327). */
void oracle_forward_solve(const cplx *A, const cplx *b, int n, cplx *x)
{
    for (int i = 0; i < n; ++i) {
        cplx v = b[i];
        for (int k = 0; k < i; ++k) v -= A[i * n + k] * x[k];
        x[i] = v / A[i * n + i];
    }
}

/* Upper-triangular solve A x = b (linearSolvec.pyx:330-346). */
void oracle_back_solve(const cplx *A, const cplx *b, int n, cplx *x)
{
    for (int i = n - 1; i >= 0; --i) {
        cplx v = b[i];
        for (int k = n - 1; k > i; --k) v -= A[i * n + k] * x[k];
        x[i] = v / A[i * n + i];
    }
}

/* solveCholesky: U = chol(A); y = (U^H)^-1 b; x = U^-1 y (linearSolvec.pyx:259-282).
 * `work` holds 2*n*n + n elements. */
void oracle_solve_cholesky(const cplx *A, const cplx *b, int n, cplx *x, cplx *work)
{
    cplx *U = work, *UT = work + (size_t)n * n, *y = work + 2 * (size_t)n * n;
    oracle_cholesky(A, n, U);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) UT[j * n + i] = conj(U[i * n + j]);
    oracle_forward_solve(UT, b, n, y);
    oracle_back_solve(U, y, n, x);
}

/* DFT bin of beam b (capon_kernel.cu:53-59; the even-Nb branch there is dead code). */
static int butler_bin(int b, int Nb, int L)
{
    return (b > Nb / 2) ? b + (L - 2 * (Nb / 2) - 1) : b;
}

/* Butler matrix, row-major Nb x L.  symmetric=1: the GPU beam layout of
 * capon_kernel.cu:47-77; symmetric=0: the first Nb DFT bins, as
 * framework/linalg/beamspace.py:18-34 (butlerMatrix) lays them out. */
void oracle_butler_layout(int Nb, int L, cplx *B, int symmetric)
{
    for (int b = 0; b < Nb; ++b) {
        int bin = symmetric ? butler_bin(b, Nb, L) : b;
        for (int l = 0; l < L; ++l)
            B[b * L + l] = cexp(-I * 2.0 * kPi * (double)bin * (double)l / (double)L) / sqrt((double)L);
    }
}

/* Butler matrix in the GPU beam layout (capon_kernel.cu:47-77). */
void oracle_butler(int Nb, int L, cplx *B)
{
    for (int b = 0; b < Nb; ++b) {
        int bin = butler_bin(b, Nb, L);
        for (int l = 0; l < L; ++l)
            B[b * L + l] = cexp(-I * 2.0 * kPi * (double)bin * (double)l / (double)L) / sqrt((double)L);
    }
}

/* ---- the per-pixel path -------------------------------------------------- */

typedef struct {
    const float *Xd;   /* interleaved complex64 [Nx][Ny][M] */
    int Nx, Ny, M, L, Navg, Nb, fp32_scalars, bs_loading, fb;
    double regCoef;
    const cplx *V;     /* Nb x L subspace matrix (row-major) or NULL for the Butler matrix */
    /* outputs (any may be NULL except z): [Nx][Ny-2Navg](...) */
    cplx *z, *zpow, *w, *R;
    double *P;
    int x0, x1;        /* beam range for this worker */
} job_t;

static void pixel_run(const job_t *jb, int x, int y, cplx *scratch)
{
    const int M = jb->M, L = jb->L, Navg = jb->Navg, Ny = jb->Ny, Nb = jb->Nb;
    const int T = 2 * Navg + 1, Ns = M - L + 1;
    const int Npy = Ny - 2 * Navg;
    const size_t pix = (size_t)x * Npy + (size_t)(y - Navg);

    double regCoef = jb->regCoef, K_inv = 1.0 / Ns, norm_inv = 1.0 / ((double)Ns * T);
    if (jb->fp32_scalars) {
        regCoef = (float)regCoef;
        K_inv = (float)(1.0f / (float)Ns);
        norm_inv = (float)(1.0f / ((float)Ns * (float)T));
    }

    cplx *ar = scratch;                       /* T x M   */
    cplx *Rf = ar + (size_t)T * M;            /* M x M   */
    cplx *R = Rf + (size_t)M * M;             /* L x L   */
    cplx *g = R + (size_t)L * L;              /* L       */
    cplx *a = g + L;                          /* L       */
    cplx *Ria = a + L;                        /* L       */
    cplx *wk = Ria + L;                       /* 2 L L + L */
    cplx *wv = wk + 2 * (size_t)L * L + L;    /* L       */

    /* :203-205 snapshot gather */
    for (int t = 0; t < T; ++t)
        for (int m = 0; m < M; ++m) {
            const float *p = jb->Xd + 2 * (((size_t)x * Ny + (y - Navg + t)) * M + m);
            ar[t * M + m] = (double)p[0] + I * (double)p[1];
        }
    /* :207-223 band of R_full = ar^H ar, R_full[i, i+j] for 0 <= j < L */
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < L && i + j < M; ++j) {
            cplx s = 0;
            for (int t = 0; t < T; ++t) s += conj(ar[t * M + i]) * ar[t * M + i + j];
            Rf[i * M + i + j] = s;
        }
    /* :226-242 smoothing over subarrays (upper triangle), then conj / norm */
    for (int j = 0; j < L; ++j)
        for (int k = 0; k < L; ++k) R[j * L + k] = 0;
    for (int s = 0; s < Ns; ++s)
        for (int j = 0; j < L; ++j)
            for (int k = j; k < L; ++k) R[j * L + k] += Rf[(s + j) * M + s + k];
    for (int j = 0; j < L; ++j)
        for (int k = j; k < L; ++k) R[j * L + k] = conj(R[j * L + k]) * norm_inv;

    /* :246-255 subarray sums of the centre snapshot */
    {
        cplx s0 = 0;
        const cplx *xc = ar + (size_t)Navg * M;
        for (int i = 0; i < Ns; ++i) s0 += xc[i];
        g[0] = s0;
        for (int i = 1; i < L; ++i) g[i] = g[i - 1] - xc[i - 1] + xc[M - L + i];
        for (int i = 0; i < L; ++i) g[i] *= K_inv;
    }

    /* full Hermitian R (lower from upper) for the solve and the outputs */
    for (int j = 0; j < L; ++j)
        for (int k = 0; k < j; ++k) R[j * L + k] = conj(R[k * L + j]);

    if (jb->fb) {   /* R = (R + J R^T J) / 2: (J R^T J)[j][k] = R[L-1-k][L-1-j] */
        cplx *Rt = wk;
        for (int i = 0; i < L * L; ++i) Rt[i] = R[i];
        for (int j = 0; j < L; ++j)
            for (int k = 0; k < L; ++k) R[j * L + k] = 0.5 * (Rt[j * L + k] + Rt[(L - 1 - k) * L + (L - 1 - j)]);
    }

    cplx zz = 0, zp = 0;
    double Pv;
    if (Nb <= 0) {
        /* :257-262 diagonal loading */
        cplx tr = 0;
        for (int i = 0; i < L; ++i) tr += R[i * L + i];
        cplx dl = jb->bs_loading == 2 ? (cplx)regCoef : tr * regCoef / L;
        for (int i = 0; i < L; ++i) R[i * L + i] += dl;
        for (int i = 0; i < L; ++i) a[i] = 1.0;
        /* :274 */
        oracle_solve_cholesky(R, a, L, Ria, wk);
        /* :276-283 */
        cplx aRia = 0;
        for (int i = 0; i < L; ++i) aRia += conj(a[i]) * Ria[i];
        for (int i = 0; i < L; ++i) wv[i] = Ria[i] / aRia;
        for (int i = 0; i < L; ++i) zz += conj(wv[i]) * g[i];
        /* :285-289 upper-triangle quirk */
        for (int i = 0; i < L; ++i) {
            cplx idot = 0;
            for (int j = i; j < L; ++j) idot += conj(wv[j]) * R[i * L + j];
            zp += idot * wv[i];
        }
        Pv = 1.0 / creal(aRia);
    } else {
        /* beamspace: R_bs = B R_d B^H (Capon.cpp:311-319) */
        cplx *B = wk;                                  /* Nb x L */
        cplx *Rb = B + (size_t)Nb * L;                 /* Nb x Nb */
        cplx *tmp = Rb + (size_t)Nb * Nb;              /* Nb x L */
        cplx *ab = tmp + (size_t)Nb * L;               /* Nb */
        cplx *xb = ab + Nb;                            /* Nb */
        cplx *wb = xb + Nb;                            /* 2 Nb Nb + Nb */
        if (jb->V) /* a given subspace (getCaponAllC.pyx:226-231, 365-370) */
            for (int i = 0; i < Nb * L; ++i) B[i] = jb->V[i];
        else
            oracle_butler(Nb, L, B);
        if (jb->bs_loading != 1) {
            cplx tr = 0;
            for (int i = 0; i < L; ++i) tr += R[i * L + i];
            cplx dl = jb->bs_loading == 2 ? (cplx)regCoef : tr * regCoef / L;
            for (int i = 0; i < L; ++i) R[i * L + i] += dl;
        }
        for (int b = 0; b < Nb; ++b)
            for (int l = 0; l < L; ++l) {
                cplx s = 0;
                for (int k = 0; k < L; ++k) s += B[b * L + k] * R[k * L + l];
                tmp[b * L + l] = s;
            }
        for (int b = 0; b < Nb; ++b)
            for (int c = 0; c < Nb; ++c) {
                cplx s = 0;
                for (int l = 0; l < L; ++l) s += tmp[b * L + l] * conj(B[c * L + l]);
                Rb[b * Nb + c] = s;
            }
        if (jb->bs_loading == 1) {   /* getCaponAllC.pyx:376-385 */
            cplx tr = 0;
            for (int i = 0; i < Nb; ++i) tr += Rb[i * Nb + i];
            cplx dl = tr * regCoef / Nb;
            for (int i = 0; i < Nb; ++i) Rb[i * Nb + i] += dl;
        }
        for (int b = 0; b < Nb; ++b) {               /* a_bs = B 1 (Capon.cpp:329-333) */
            cplx s = 0;
            for (int l = 0; l < L; ++l) s += B[b * L + l];
            ab[b] = s;
        }
        oracle_solve_cholesky(Rb, ab, Nb, xb, wb);
        for (int l = 0; l < L; ++l) {                 /* Ria = B^H Ria_bs (Capon.cpp:366-369) */
            cplx s = 0;
            for (int b = 0; b < Nb; ++b) s += conj(B[b * L + l]) * xb[b];
            Ria[l] = s;
        }
        cplx sum = 0;                                 /* capon_kernel.cu:373-379 */
        for (int l = 0; l < L; ++l) sum += Ria[l];
        for (int l = 0; l < L; ++l) wv[l] = Ria[l] / sum;
        for (int l = 0; l < L; ++l) zz += conj(wv[l]) * g[l];
        cplx aRia = 0;
        for (int b = 0; b < Nb; ++b) aRia += conj(ab[b]) * xb[b];
        Pv = 1.0 / creal(aRia);
        /* zpow analogue in beamspace: upper-triangle sum with w_bs */
        for (int i = 0; i < Nb; ++i) {
            cplx idot = 0;
            for (int j = i; j < Nb; ++j) idot += conj(xb[j] / aRia) * Rb[i * Nb + j];
            zp += idot * (xb[i] / aRia);
        }
    }

    jb->z[pix] = zz;
    if (jb->zpow) jb->zpow[pix] = zp;
    if (jb->P) jb->P[pix] = Pv;
    if (jb->w)
        for (int i = 0; i < L; ++i) jb->w[pix * L + i] = wv[i];
    if (jb->R)   /* loaded, normalised, full Hermitian, row-major per pixel */
        for (int i = 0; i < L * L; ++i) jb->R[pix * L * L + i] = R[i];
}

static size_t scratch_elems(int M, int L, int Navg, int Nb)
{
    int T = 2 * Navg + 1;
    size_t n = (size_t)T * M + (size_t)M * M + (size_t)L * L + 4 * (size_t)L + 2 * (size_t)L * L + L;
    n += (size_t)Nb * L * 2 + (size_t)Nb * Nb * 3 + 4 * (size_t)Nb + 16;
    return n;
}

static void *worker(void *arg)
{
    const job_t *jb = (const job_t *)arg;
    cplx *scratch = (cplx *)malloc(sizeof(cplx) * scratch_elems(jb->M, jb->L, jb->Navg, jb->Nb));
    if (!scratch) return (void *)1;
    for (int x = jb->x0; x < jb->x1; ++x)
        for (int y = jb->Navg; y < jb->Ny - jb->Navg; ++y) pixel_run(jb, x, y, scratch);
    free(scratch);
    return NULL;
}

/*
 * Capon over a cube Xd[Nx][Ny][M] (interleaved complex64 input, as the GPU
 * path receives it).  Outputs are complex128 / float64 arrays indexed
 * [Nx][Ny-2*Navg](...).  `nthreads` splits the beams into contiguous slabs.
 * Returns 0 on success, 1 on invalid arguments, 2 on allocation failure.
 */
int oracle_capon_v(const float *Xd, int Nx, int Ny, int M, double regCoef, int L, int Navg,
                   int Nb, int bs_loading, int fp32_scalars, int fb, const cplx *V,
                   cplx *z, cplx *zpow, cplx *w, double *P, cplx *R, int nthreads);

int oracle_capon_ex(const float *Xd, int Nx, int Ny, int M, double regCoef, int L, int Navg,
                    int Nb, int bs_loading, int fp32_scalars, int fb,
                    cplx *z, cplx *zpow, cplx *w, double *P, cplx *R, int nthreads)
{
    return oracle_capon_v(Xd, Nx, Ny, M, regCoef, L, Navg, Nb, bs_loading, fp32_scalars, fb, NULL, z, zpow, w, P,
                          R, nthreads);
}

int oracle_capon(const float *Xd, int Nx, int Ny, int M, double regCoef, int L, int Navg,
                 int Nb, int bs_loading, int fp32_scalars,
                 cplx *z, cplx *zpow, cplx *w, double *P, cplx *R, int nthreads)
{
    return oracle_capon_ex(Xd, Nx, Ny, M, regCoef, L, Navg, Nb, bs_loading, fp32_scalars, 0, z, zpow, w, P, R,
                           nthreads);
}

/* Nb > 0 with V != NULL: beamspace over the given subspace (V B^H-style
 * transform of the loaded element-space R; a_bs = V 1; w = V^H x_bs / a_bs^H x_bs) */
int oracle_capon_v(const float *Xd, int Nx, int Ny, int M, double regCoef, int L, int Navg,
                   int Nb, int bs_loading, int fp32_scalars, int fb, const cplx *V,
                   cplx *z, cplx *zpow, cplx *w, double *P, cplx *R, int nthreads)
{
    if (Nx < 1 || Ny < 1 || L < 1 || M < 1 || Navg < 0 || Nb < 0 || L > M || Nb > L ||
        2 * Navg >= Ny || !Xd || !z)
        return 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > Nx) nthreads = Nx;
    job_t base = {Xd, Nx, Ny, M, L, Navg, Nb, fp32_scalars, bs_loading, fb ? 1 : 0, regCoef, V,
                  z, zpow, w, R, P, 0, Nx};
    if (nthreads == 1) return worker(&base) ? 2 : 0;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    job_t *jobs = (job_t *)malloc(sizeof(job_t) * nthreads);
    if (!th || !jobs) { free(th); free(jobs); return 2; }
    int rc = 0;
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = base;
        jobs[i].x0 = (int)((long)Nx * i / nthreads);
        jobs[i].x1 = (int)((long)Nx * (i + 1) / nthreads);
        pthread_create(&th[i], NULL, worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) {
        void *ret = NULL;
        pthread_join(th[i], &ret);
        if (ret) rc = 2;
    }
    free(th);
    free(jobs);
    return rc;
}

/* ---- sliding-window inverse (Sherman-Morrison along range) --------------- */

/*
 * Rank-1 change of an inverse, framework/linalg/woodburyc.pyx:73-100:
 * for A <- A + sign x x^H and B = A^-1,
 *     B <- B - sign (B x)(x^H B) / (1 + sign x^H B x).
 * The reference forms B x and x^H B separately (:88-90); both are formed
 * here too.  `u` holds 2n elements.  Returns 1 + sign x^H B x (the
 * reference raises when it is 0, :95-96; the caller checks it).
 */
double oracle_sm_update(cplx *B, const cplx *x, int n, int sign, cplx *u)
{
    cplx *Bx = u, *xB = u + n;
    for (int i = 0; i < n; ++i) {
        cplx s = 0, t = 0;
        for (int j = 0; j < n; ++j) {
            s += B[i * n + j] * x[j];
            t += conj(x[j]) * B[j * n + i];
        }
        Bx[i] = s;
        xB[i] = t;
    }
    cplx xBx = 0;
    for (int i = 0; i < n; ++i) xBx += conj(x[i]) * Bx[i];
    const cplx den = 1.0 + (double)sign * xBx;
    const cplx f = (double)sign / den;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) B[i * n + j] -= f * Bx[i] * xB[j];
    return creal(den);
}

/* iterativeBuildUpRinv / iterativeBuildDownRinv (woodburyc.pyx:15-42): one
 * rank-1 change per subarray l = 0..M-L of the row X[0..M-1], in that order. */
double oracle_sm_row(cplx *B, const cplx *X, int M, int L, int sign, cplx *u)
{
    double dmin = INFINITY;
    for (int l = 0; l + L <= M; ++l) {
        double den = oracle_sm_update(B, X + l, L, sign, u);
        if (den < dmin) dmin = den;
    }
    return dmin;
}

typedef struct {
    const float *Xd;
    int Nx, Ny, M, L, Navg, segment;
    double d;
    cplx *z, *w;
    double *P, *den_min;
    int x0, x1;
} slide_job_t;

static void slide_row(const float *src, int M, cplx *dst)
{
    for (int m = 0; m < M; ++m) dst[m] = src[2 * m] + I * src[2 * m + 1];
}

static void *slide_worker(void *arg)
{
    const slide_job_t *jb = (const slide_job_t *)arg;
    const int M = jb->M, L = jb->L, T = 2 * jb->Navg + 1, Ns = M - L + 1, Npy = jb->Ny - 2 * jb->Navg;
    const double nt = (double)Ns * T;
    cplx *B = (cplx *)malloc(sizeof(cplx) * ((size_t)L * L + 2 * (size_t)L + 2 * (size_t)M + L));
    if (!B) return (void *)1;
    cplx *u = B + (size_t)L * L, *row = u + 2 * L, *xc = row + M, *ria = xc + M;
    double dmin = INFINITY;
    for (int bx = jb->x0; bx < jb->x1; ++bx) {
        const float *xb = jb->Xd + (size_t)bx * jb->Ny * M * 2;
        for (int p0 = 0; p0 < Npy; p0 += jb->segment) {
            const int p1 = p0 + jb->segment < Npy ? p0 + jb->segment : Npy;
            /* fresh build-up of the window of pixel p0 (woodburyc.pyx:46-70):
             * B = I / (Ns T d), then rows p0 .. p0+2K */
            memset(B, 0, sizeof(cplx) * (size_t)L * L);
            for (int i = 0; i < L; ++i) B[i * L + i] = 1.0 / (nt * jb->d);
            for (int t = p0; t < p0 + T; ++t) {
                slide_row(xb + (size_t)t * M * 2, M, row);
                double dm = oracle_sm_row(B, row, M, L, +1, u);
                if (dm < dmin) dmin = dm;
            }
            for (int p = p0; p < p1; ++p) {
                if (p > p0) {
                    /* the window moves one row: row p+2K enters, row p-1 leaves
                     * (getCaponAllC.pyx:240-252 with the rows in this order) */
                    slide_row(xb + (size_t)(p + T - 1) * M * 2, M, row);
                    double dm = oracle_sm_row(B, row, M, L, +1, u);
                    if (dm < dmin) dmin = dm;
                    slide_row(xb + (size_t)(p - 1) * M * 2, M, row);
                    dm = oracle_sm_row(B, row, M, L, -1, u);
                    if (dm < dmin) dmin = dm;
                }
                /* R_d^-1 a = Ns T B 1 (the normalisation of woodburyc.pyx:68) */
                cplx aRia = 0;
                for (int i = 0; i < L; ++i) {
                    cplx s = 0;
                    for (int j = 0; j < L; ++j) s += B[i * L + j];
                    ria[i] = nt * s;
                    aRia += ria[i];
                }
                /* subarray sums of the centre row (getCaponC.pyx:246-255) */
                slide_row(xb + (size_t)(p + jb->Navg) * M * 2, M, xc);
                cplx zz = 0;
                for (int i = 0; i < L; ++i) {
                    cplx g = 0;
                    for (int s = 0; s < Ns; ++s) g += xc[i + s];
                    g /= (double)Ns;
                    const cplx wi = ria[i] / aRia;
                    zz += conj(wi) * g;
                    if (jb->w) jb->w[((size_t)bx * Npy + p) * L + i] = wi;
                }
                jb->z[(size_t)bx * Npy + p] = zz;
                if (jb->P) jb->P[(size_t)bx * Npy + p] = 1.0 / creal(aRia);
            }
        }
    }
    if (jb->den_min) *jb->den_min = dmin;
    free(B);
    return NULL;
}

/*
 * Capon with R_d^-1 tracked along range by rank-1 changes instead of a
 * factorisation per pixel: the SOLVE_WOOD branch of
 * framework/beamformer/capon/getCaponAllC.pyx:240-252 with the updates of
 * framework/linalg/woodburyc.pyx:15-107.
 *   * Loading is absolute on the normalised covariance, R_d = R + d I, so that
 *     A = sum x x^H + Ns T d I and R_d^-1 = Ns T A^-1 (the build-up starts
 *     from (1/loading) I and scales by Ns T at the end, woodburyc.pyx:57-68).
 *   * Every `segment` pixels along range start from a fresh build-up; between
 *     two pixels row p+2K enters and row p-1 leaves.  (The reference branch
 *     builds only at y == 0, which its range loop never reaches for Navg > 0,
 *     and applies the entering row as a downdate; both are corrected here.)
 *   * Outputs as the element-space path: w = R_d^-1 a / a^H R_d^-1 a,
 *     z = sum conj(w) g, P = 1 / Re(a^H R_d^-1 a).
 * den_min (optional, one per thread) receives the smallest Sherman-Morrison
 * denominator seen.  Returns 0, 1 (invalid arguments) or 2 (allocation).
 */
int oracle_capon_sliding(const float *Xd, int Nx, int Ny, int M, double d, int L, int Navg, int segment,
                         cplx *z, cplx *w, double *P, double *den_min, int nthreads)
{
    if (Nx < 1 || Ny < 1 || L < 1 || M < 1 || Navg < 0 || L > M || 2 * Navg >= Ny || segment < 1 || !(d > 0) ||
        !Xd || !z)
        return 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > Nx) nthreads = Nx;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    slide_job_t *jobs = (slide_job_t *)malloc(sizeof(slide_job_t) * nthreads);
    double *dm = (double *)malloc(sizeof(double) * nthreads);
    if (!th || !jobs || !dm) { free(th); free(jobs); free(dm); return 2; }
    int rc = 0;
    for (int i = 0; i < nthreads; ++i) {
        slide_job_t j = {Xd, Nx, Ny, M, L, Navg, segment, d, z, w, P, &dm[i],
                         (int)((long)Nx * i / nthreads), (int)((long)Nx * (i + 1) / nthreads)};
        jobs[i] = j;
        pthread_create(&th[i], NULL, slide_worker, &jobs[i]);
    }
    double dmin = INFINITY;
    for (int i = 0; i < nthreads; ++i) {
        void *ret = NULL;
        pthread_join(th[i], &ret);
        if (ret) rc = 2;
        else if (dm[i] < dmin) dmin = dm[i];
    }
    if (den_min) *den_min = dmin;
    free(th);
    free(jobs);
    free(dm);
    return rc;
}
