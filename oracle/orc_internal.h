/*
 * ORACLE — test infrastructure only (CPU restatement of SPECTER's per-RK-stage
 * hot path, FP64).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The shipped product never links it.
 */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

#include <complex.h>
#include <stddef.h>

typedef double _Complex cplx;

typedef struct orc_fftplan {
    int n;
    int nf;          /* number of Stockham stages, -1 when Bluestein is used */
    int radix[40];
    cplx *tw;        /* tw[t] = exp(-2*pi*i*t/n) */
    int m;           /* Bluestein padded length */
    struct orc_fftplan *sub;
    cplx *chirp;     /* exp(-i*pi*k^2/n) */
    cplx *bf, *bb;   /* FFT_m of the circular chirp filter, forward / backward sign */
} orc_fftplan;

orc_fftplan *orc_fft_plan(int n);
void orc_fft_free(orc_fftplan *p);
size_t orc_fft_work(const orc_fftplan *p);
/* in-place unnormalised DFT of x[0..n), sign -1 forward, +1 backward */
void orc_fft_exec(const orc_fftplan *p, cplx *x, int sign, cplx *work);

#endif
