/*
 * ORACLE — test infrastructure only. Not part of the shipped product.
 *
 * Double-precision complex FFT used by the CPU restatement of SPECTER's
 * transforms.  The reference calls FFTW 3.x (dfftw_plan_many_dft /
 * dfftw_plan_many_dft_r2c / _c2r, src/fftp/fftp.fpp:96-142, executed at
 * fftp.fpp:469,780,913,1089).  FFTW is not vendored in the reference and
 * is not installed here, so this file restates the published algorithms it
 * computes: the unnormalised DFT
 *     X_j = sum_k x_k exp(sign * 2*pi*i*j*k/n),  sign = -1 forward, +1 backward
 * evaluated by an iterative Stockham autosort mixed-radix FFT (radices 4, 2,
 * 3, 5 specialised, any other prime <= 13 by a direct radix-p DFT) and, for
 * lengths with a larger prime factor, by Bluestein's chirp-z algorithm
 * (L. Bluestein, IEEE Trans. Audio Electroacoust. 18 (1970) 451) over a
 * {2,3,5}-smooth padded length.  Accuracy is checked against numpy.fft
 * (pocketfft) in tests/test_oracle_fft.py.
 */
#include "orc_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int smooth235(int m) {
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    return m == 1;
}

/* exp(-2*pi*i*t/n) evaluated with long double argument reduction. */
static cplx unit_root(long t, long n) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)(t % n) / (long double)n;
    return (double)cosl(a) + I * (double)sinl(a);
}

static int factorize(int n, int *radix) {
    int nf = 0;
    while (n % 4 == 0) { radix[nf++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[nf++] = 2; n /= 2; }
    static const int odd[] = {3, 5, 7, 11, 13};
    for (int i = 0; i < 5; i++)
        while (n % odd[i] == 0) { radix[nf++] = odd[i]; n /= odd[i]; }
    if (n != 1) return -1; /* prime factor > 13 left */
    return nf;
}

orc_fftplan *orc_fft_plan(int n) {
    orc_fftplan *p = (orc_fftplan *)calloc(1, sizeof(orc_fftplan));
    p->n = n;
    p->nf = factorize(n, p->radix);
    if (p->nf >= 0) {
        p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
        for (int t = 0; t < n; t++) p->tw[t] = unit_root(t, n);
        return p;
    }
    /* Bluestein: X_j = c_j * sum_k (x_k c_k) conj(c_{j-k}), c_k = exp(sign*pi*i*k^2/n) */
    int m = 2 * n - 1;
    while (!smooth235(m)) m++;
    p->m = m;
    p->sub = orc_fft_plan(m);
    p->chirp = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (long k = 0; k < n; k++) {
        long k2 = (k * k) % (2L * n);
        long double a = -3.14159265358979323846264338327950288L * (long double)k2 / (long double)n;
        p->chirp[k] = (double)cosl(a) + I * (double)sinl(a); /* forward-sign chirp */
    }
    p->bf = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    p->bb = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    cplx *work = (cplx *)malloc(sizeof(cplx) * (size_t)orc_fft_work(p->sub));
    /* filter for the forward sign: conj(c_fwd(m)) = c_bwd, placed circularly */
    memset(p->bf, 0, sizeof(cplx) * (size_t)m);
    memset(p->bb, 0, sizeof(cplx) * (size_t)m);
    for (int k = 0; k < n; k++) {
        cplx cf = p->chirp[k];
        p->bf[k] = conj(cf);
        p->bb[k] = cf;
        if (k) { p->bf[m - k] = conj(cf); p->bb[m - k] = cf; }
    }
    orc_fft_exec(p->sub, p->bf, -1, work);
    orc_fft_exec(p->sub, p->bb, -1, work);
    free(work);
    return p;
}

void orc_fft_free(orc_fftplan *p) {
    if (!p) return;
    free(p->tw); free(p->chirp); free(p->bf); free(p->bb);
    orc_fft_free(p->sub);
    free(p);
}

size_t orc_fft_work(const orc_fftplan *p) {
    if (p->nf >= 0) return (size_t)p->n;
    return (size_t)p->m + orc_fft_work(p->sub);
}

static inline cplx twid(const orc_fftplan *p, int t, int sign) {
    cplx w = p->tw[t];
    return sign < 0 ? w : conj(w);
}

/* One Stockham stage: radix R, Ns = product of earlier radices. */
static void stockham_stage(const orc_fftplan *p, int R, int Ns, const cplx *X, cplx *Y, int sign) {
    const int n = p->n, nR = n / R, step = n / (Ns * R);
    const double s = (double)sign;
    for (int j = 0; j < nR; j++) {
        const int k = j % Ns;
        cplx a[13];
        for (int q = 0; q < R; q++) {
            a[q] = X[j + q * nR];
            if (k) a[q] *= twid(p, q * k * step, sign);
        }
        cplx b[13];
        switch (R) {
        case 2:
            b[0] = a[0] + a[1];
            b[1] = a[0] - a[1];
            break;
        case 4: {
            cplx t0 = a[0] + a[2], t1 = a[0] - a[2];
            cplx t2 = a[1] + a[3], t3 = (a[1] - a[3]) * (s * I);
            b[0] = t0 + t2; b[2] = t0 - t2;
            b[1] = t1 + t3; b[3] = t1 - t3;
            break;
        }
        case 3: {
            const double c3 = -0.5, s3 = s * 0.86602540378443864676372317075294;
            cplx t1 = a[1] + a[2], t2 = (a[1] - a[2]) * (s3 * I);
            cplx m1 = a[0] + c3 * t1;
            b[0] = a[0] + t1; b[1] = m1 + t2; b[2] = m1 - t2;
            break;
        }
        default: {
            /* direct radix-R DFT: exp(s*2*pi*i*q*r/R) = tw[(q*r mod R)*(n/R)] */
            for (int r = 0; r < R; r++) {
                cplx acc = a[0];
                for (int q = 1; q < R; q++) acc += a[q] * twid(p, ((q * r) % R) * nR, sign);
                b[r] = acc;
            }
        }
        }
        const int base = (j / Ns) * Ns * R + k;
        for (int q = 0; q < R; q++) Y[base + q * Ns] = b[q];
    }
}

void orc_fft_exec(const orc_fftplan *p, cplx *x, int sign, cplx *work) {
    const int n = p->n;
    if (p->nf >= 0) {
        cplx *X = x, *Y = work;
        int Ns = 1;
        for (int f = 0; f < p->nf; f++) {
            stockham_stage(p, p->radix[f], Ns, X, Y, sign);
            Ns *= p->radix[f];
            cplx *t = X; X = Y; Y = t;
        }
        if (X != x) memcpy(x, X, sizeof(cplx) * (size_t)n);
        return;
    }
    const int m = p->m;
    cplx *a = work, *subw = work + m;
    const cplx *filt = sign < 0 ? p->bf : p->bb;
    for (int k = 0; k < n; k++) a[k] = x[k] * (sign < 0 ? p->chirp[k] : conj(p->chirp[k]));
    for (int k = n; k < m; k++) a[k] = 0;
    orc_fft_exec(p->sub, a, -1, subw);
    for (int k = 0; k < m; k++) a[k] *= filt[k];
    orc_fft_exec(p->sub, a, +1, subw);
    const double inv = 1.0 / (double)m;
    for (int k = 0; k < n; k++) x[k] = a[k] * inv * (sign < 0 ? p->chirp[k] : conj(p->chirp[k]));
}
