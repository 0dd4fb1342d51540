/*
 * ORACLE — test infrastructure only (see oracle.h for the parity status and
 * who may load it).
 *
 * FP64 CPU restatement of SPECTER's per-RK-stage hot path.  Every function
 * names the reference routine (file:line) it restates; expression order
 * follows the Fortran source so that FP64 results agree to rounding.
 * Compiled with -fcx-fortran-rules so complex products follow Fortran rules.
 */
#include "oracle.h"
#include "orc_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_grid {
    int nx, ny, nz, cz, oz, nxh, pkend;
    double Lx, Ly, Lz, Dkx, Dky, Dkz;
    double *kx, *ky, *kz, *khom, *z;
    double *dir; /* dir(i,j) = dir[i + cz*j], C x d, Fortran order */
    orc_fftplan *px, *py, *pz;
};

#define PI_GP 3.14159265358979323846

static inline size_t SIDX(const orc_grid *g, int z, int ky, int kx) {
    return ((size_t)kx * g->ny + ky) * g->nz + z;
}
static inline size_t RIDX(const orc_grid *g, int x, int y, int z) {
    return ((size_t)z * g->ny + y) * g->nx + x;
}
static inline size_t NS(const orc_grid *g) { return (size_t)g->nxh * g->ny * g->nz; }
static inline size_t NR(const orc_grid *g) { return (size_t)g->nx * g->ny * g->nz; }
/* im*k*a with Fortran complex-product arithmetic: (0,k)*(ar,ai) */
static inline cplx imk(double k, cplx a) { return (0.0 * creal(a) - k * cimag(a)) + I * (0.0 * cimag(a) + k * creal(a)); }
static inline double kk2(const orc_grid *g, int z, int ky, int kx) {
    return g->kx[kx] * g->kx[kx] + g->ky[ky] * g->ky[ky] + g->kz[z] * g->kz[z];
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* load_dirichlet_tables, src/fftp/fcgram_mod.f90:180-257: A(C,d) and Q(d,d) are raw
 * float64 streams in Fortran order; Q = TRANSPOSE(Q); dir = MATMUL(A,Q). */
static int load_dirichlet(orc_grid *g, const char *tdir) {
    const int C = g->cz, d = g->oz;
    char path[4096];
    double *A = malloc(sizeof(double) * C * d), *Q = malloc(sizeof(double) * d * d);
    snprintf(path, sizeof path, "%s/A%d-%d.dat", tdir, C, d);
    FILE *f = fopen(path, "rb");
    if (!f || fread(A, sizeof(double), (size_t)C * d, f) != (size_t)C * d) { if (f) fclose(f); free(A); free(Q); return 2; }
    fclose(f);
    snprintf(path, sizeof path, "%s/Q%d.dat", tdir, d);
    f = fopen(path, "rb");
    if (!f || fread(Q, sizeof(double), (size_t)d * d, f) != (size_t)d * d) { if (f) fclose(f); free(A); free(Q); return 2; }
    fclose(f);
    g->dir = malloc(sizeof(double) * C * d);
    for (int i = 0; i < C; i++)
        for (int j = 0; j < d; j++) {
            double s = 0.0; /* (A * Q^T)(i,j) = sum_l A(i,l) * Q(j,l) */
            for (int l = 0; l < d; l++) s += A[i + C * l] * Q[j + d * l];
            g->dir[i + C * j] = s;
        }
    free(A); free(Q);
    return 0;
}

/* grids and wavenumbers: src/specter.fpp:683-800 (periodic x,y; FC-Gram z) */
orc_grid *orc_create(int nx, int ny, int nz, int cz, int oz, double Lx, double Ly, double Lz,
                     const char *tdir, int *err) {
    *err = 0;
    if (nx < 2 || ny < 2 || nz < 2 || (nx % 2) || (ny % 2) || (nz % 2) || cz <= 0 || oz <= 0 ||
        nz - cz < 2 * oz || nz - cz < 2) { *err = 1; return NULL; }
    orc_grid *g = calloc(1, sizeof(orc_grid));
    g->nx = nx; g->ny = ny; g->nz = nz; g->cz = cz; g->oz = oz;
    g->nxh = nx / 2 + 1; g->pkend = nz - cz;
    g->Lx = Lx; g->Ly = Ly; g->Lz = Lz;
    if ((*err = load_dirichlet(g, tdir))) { free(g); return NULL; }
    g->Dkx = 1.0 / Lx;
    g->Dky = 1.0 / Ly;
    const double dz = Lz / (nz - cz - 1);
    g->Dkz = 2.0 * PI_GP / (dz * nz);
    g->z = malloc(sizeof(double) * nz);
    for (int k = 0; k < nz; k++) g->z[k] = dz * k;
    g->kx = malloc(sizeof(double) * nx);
    g->ky = malloc(sizeof(double) * ny);
    g->kz = malloc(sizeof(double) * nz);
    for (int i = 0; i < nx / 2; i++) { g->kx[i] = i; g->kx[i + nx / 2] = i - nx / 2; }
    for (int j = 0; j < ny / 2; j++) { g->ky[j] = j; g->ky[j + ny / 2] = j - ny / 2; }
    for (int k = 0; k < nz / 2; k++) { g->kz[k] = k; g->kz[k + nz / 2] = k - nz / 2; }
    for (int i = 0; i < nx; i++) g->kx[i] *= g->Dkx;
    for (int j = 0; j < ny; j++) g->ky[j] *= g->Dky;
    for (int k = 0; k < nz; k++) g->kz[k] *= g->Dkz;
    g->khom = malloc(sizeof(double) * g->nxh * ny);
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < ny; j++) g->khom[i * ny + j] = sqrt(kk2(g, 0, j, i));
    g->px = orc_fft_plan(nx);
    g->py = orc_fft_plan(ny);
    g->pz = orc_fft_plan(nz);
    return g;
}

void orc_destroy(orc_grid *g) {
    if (!g) return;
    free(g->kx); free(g->ky); free(g->kz); free(g->khom); free(g->z); free(g->dir);
    orc_fft_free(g->px); orc_fft_free(g->py); orc_fft_free(g->pz);
    free(g);
}

void orc_grid_info(const orc_grid *g, double *kx, double *ky, double *kz, double *z, double *dir) {
    if (kx) memcpy(kx, g->kx, sizeof(double) * g->nxh);
    if (ky) memcpy(ky, g->ky, sizeof(double) * g->ny);
    if (kz) memcpy(kz, g->kz, sizeof(double) * g->nz);
    if (z) memcpy(z, g->z, sizeof(double) * g->nz);
    if (dir) memcpy(dir, g->dir, sizeof(double) * g->cz * g->oz);
}

/* ------------------------------------------------------------------------- */
/* fftp                                                                      */
/* ------------------------------------------------------------------------- */

/* FC-Gram continuation of one column, src/fftp/fftp.fpp:755-773 */
static void continuation(const orc_grid *g, cplx *f) {
    const int n = g->nz, C = g->cz, d = g->oz;
    const double *dir = g->dir;
    for (int ii = 0; ii < C; ii++) {
        cplx acc = dir[ii] * f[n - C - d] + dir[C - 1 - ii] * f[d - 1];
        for (int jj = 1; jj < d; jj++)
            acc = acc + dir[ii + C * jj] * f[n - C - d + jj] + dir[(C - 1 - ii) + C * jj] * f[d - 1 - jj];
        f[n - C + ii] = acc;
    }
}

/* fftp1d_real_to_complex_z, src/fftp/fftp.fpp:720-786: continuation, then forward C2C in z */
void orc_fftp1d_real_to_complex_z(const orc_grid *g, double *inout_) {
    cplx *a = (cplx *)inout_;
    const int ncol = g->nxh * g->ny;
#pragma omp parallel
    {
        cplx *w = malloc(sizeof(cplx) * orc_fft_work(g->pz));
#pragma omp for schedule(static)
        for (int c = 0; c < ncol; c++) {
            cplx *f = a + (size_t)c * g->nz;
            continuation(g, f);
            orc_fft_exec(g->pz, f, -1, w);
        }
        free(w);
    }
}

/* fftp1d_complex_to_real_z, src/fftp/fftp.fpp:1060-1094: backward C2C in z, in place */
void orc_fftp1d_complex_to_real_z(const orc_grid *g, double *inout_) {
    cplx *a = (cplx *)inout_;
    const int ncol = g->nxh * g->ny;
#pragma omp parallel
    {
        cplx *w = malloc(sizeof(cplx) * orc_fft_work(g->pz));
#pragma omp for schedule(static)
        for (int c = 0; c < ncol; c++) orc_fft_exec(g->pz, a + (size_t)c * g->nz, +1, w);
        free(w);
    }
}

/* fftp2d_real_to_complex_xy, src/fftp/fftp.fpp:428-524: per z-plane R2C over (x,y)
 * (FFTW r2c, :469), then the transpose c1(i,j,k) -> out(k,j,i) (:506-519). */
void orc_fftp2d_real_to_complex_xy(const orc_grid *g, const double *in, double *out_) {
    cplx *out = (cplx *)out_;
    const int nx = g->nx, ny = g->ny, nxh = g->nxh;
#pragma omp parallel
    {
        cplx *row = malloc(sizeof(cplx) * (nx > ny ? nx : ny));
        cplx *plane = malloc(sizeof(cplx) * (size_t)nxh * ny);
        size_t wl = orc_fft_work(g->px) > orc_fft_work(g->py) ? orc_fft_work(g->px) : orc_fft_work(g->py);
        cplx *w = malloc(sizeof(cplx) * wl);
#pragma omp for schedule(static)
        for (int z = 0; z < g->nz; z++) {
            for (int y = 0; y < ny; y++) {
                for (int x = 0; x < nx; x++) row[x] = in[RIDX(g, x, y, z)];
                orc_fft_exec(g->px, row, -1, w);
                for (int kx = 0; kx < nxh; kx++) plane[(size_t)y * nxh + kx] = row[kx];
            }
            for (int kx = 0; kx < nxh; kx++) {
                for (int y = 0; y < ny; y++) row[y] = plane[(size_t)y * nxh + kx];
                orc_fft_exec(g->py, row, -1, w);
                for (int ky = 0; ky < ny; ky++) out[SIDX(g, z, ky, kx)] = row[ky];
            }
        }
        free(row); free(plane); free(w);
    }
}

/* fftp2d_complex_to_real_xy, src/fftp/fftp.fpp:824-919: transpose (:866-880), then
 * per z-plane C2R over (x,y) (:913).  The C2R treats the half spectrum as the
 * Hermitian half of a real signal: the imaginary parts of the kx=0 and kx=nx/2
 * entries do not contribute (real part of the full Hermitian-extended sum). */
void orc_fftp2d_complex_to_real_xy(const orc_grid *g, const double *in_, double *out) {
    const cplx *in = (const cplx *)in_;
    const int nx = g->nx, ny = g->ny, nxh = g->nxh;
#pragma omp parallel
    {
        cplx *row = malloc(sizeof(cplx) * (nx > ny ? nx : ny));
        cplx *plane = malloc(sizeof(cplx) * (size_t)nxh * ny);
        size_t wl = orc_fft_work(g->px) > orc_fft_work(g->py) ? orc_fft_work(g->px) : orc_fft_work(g->py);
        cplx *w = malloc(sizeof(cplx) * wl);
#pragma omp for schedule(static)
        for (int z = 0; z < g->nz; z++) {
            for (int kx = 0; kx < nxh; kx++) {
                for (int ky = 0; ky < ny; ky++) row[ky] = in[SIDX(g, z, ky, kx)];
                orc_fft_exec(g->py, row, +1, w);
                for (int y = 0; y < ny; y++) plane[(size_t)y * nxh + kx] = row[y];
            }
            for (int y = 0; y < ny; y++) {
                for (int k = 0; k < nxh; k++) row[k] = plane[(size_t)y * nxh + k];
                for (int k = 1; k < nx / 2; k++) row[nx - k] = conj(plane[(size_t)y * nxh + k]);
                orc_fft_exec(g->px, row, +1, w);
                for (int x = 0; x < nx; x++) out[RIDX(g, x, y, z)] = creal(row[x]);
            }
        }
        free(row); free(plane); free(w);
    }
}

/* fftp3d_real_to_complex, src/fftp/fftp.fpp:388-425 (x,y periodic branch) */
void orc_fftp3d_real_to_complex(const orc_grid *g, const double *in, double *out) {
    orc_fftp2d_real_to_complex_xy(g, in, out);
    orc_fftp1d_real_to_complex_z(g, out);
}

/* fftp3d_complex_to_real, src/fftp/fftp.fpp:789-821; the input is destroyed (:812) */
void orc_fftp3d_complex_to_real(const orc_grid *g, double *in, double *out) {
    orc_fftp1d_complex_to_real_z(g, in);
    orc_fftp2d_complex_to_real_xy(g, in, out);
}

/* ------------------------------------------------------------------------- */
/* pseudo                                                                    */
/* ------------------------------------------------------------------------- */

/* derivk, src/pseudo/pseudospec_hd.f90:28-94: b = im*k_dir*a */
void orc_derivk(const orc_grid *g, const double *a_, double *b_, int dir) {
    const cplx *a = (const cplx *)a_;
    cplx *b = (cplx *)b_;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                double kk = dir == 1 ? g->kx[i] : dir == 2 ? g->ky[j] : g->kz[k];
                b[q] = imk(kk, a[q]);
            }
}

/* laplak, src/pseudo/pseudospec_hd.f90:97-127: b = -kk2*a */
void orc_laplak(const orc_grid *g, const double *a_, double *b_) {
    const cplx *a = (const cplx *)a_;
    cplx *b = (cplx *)b_;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                b[q] = -kk2(g, k, j, i) * a[q];
            }
}

/* curlk, src/pseudo/pseudospec_hd.f90:130-206 */
void orc_curlk(const orc_grid *g, const double *a, const double *b, double *c_, int dir) {
    const size_t ns = NS(g);
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns);
    if (dir == 1) { orc_derivk(g, a, c1, 3); orc_derivk(g, b, c2, 2); }
    else if (dir == 2) { orc_derivk(g, a, c1, 3); orc_derivk(g, b, c2, 1); }
    else { orc_derivk(g, a, c1, 2); orc_derivk(g, b, c2, 1); }
    cplx *c = (cplx *)c_, *C1 = (cplx *)c1, *C2 = (cplx *)c2;
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < ns; q++) c[q] = dir == 2 ? C1[q] - C2[q] : C2[q] - C1[q];
    free(c1); free(c2);
}

static double inv_n2(const orc_grid *g) {
    double t = (double)g->nx * (double)g->ny * (double)g->nz;
    return 1.0 / (t * t);
}

/* gradre, src/pseudo/pseudospec_hd.f90:209-319: (A.grad)A via 12 c2r + 3 r2c,
 * products only on the physical z rows k <= pkend, scaled 1/(nx*ny*nz)^2.
 * Rows above pkend of rx,ry,rz are never read back: the r2c continuation
 * overwrites them. */
void orc_gradre(const orc_grid *g, const double *a, const double *b, const double *c,
                double *d, double *e, double *f) {
    const size_t ns = NS(g), nr = NR(g), plane = (size_t)g->nx * g->ny;
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns);
    double *c3 = malloc(sizeof(cplx) * ns), *c4 = malloc(sizeof(cplx) * ns);
    double *r1 = malloc(sizeof(double) * nr), *r2 = malloc(sizeof(double) * nr);
    double *r3 = malloc(sizeof(double) * nr), *r4 = malloc(sizeof(double) * nr);
    double *rx = calloc(nr, sizeof(double)), *ry = calloc(nr, sizeof(double)), *rz = calloc(nr, sizeof(double));
    const double *comp[3] = {a, b, c};
    const size_t nphys = (size_t)g->pkend * plane;
    const double tmp = inv_n2(g);
    for (int dir = 1; dir <= 3; dir++) {
        memcpy(c1, comp[dir - 1], sizeof(cplx) * ns);
        orc_derivk(g, a, c2, dir);
        orc_derivk(g, b, c3, dir);
        orc_derivk(g, c, c4, dir);
        orc_fftp3d_complex_to_real(g, c1, r1);
        orc_fftp3d_complex_to_real(g, c2, r2);
        orc_fftp3d_complex_to_real(g, c3, r3);
        orc_fftp3d_complex_to_real(g, c4, r4);
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < nphys; q++) {
            if (dir == 1) {
                rx[q] = r1[q] * r2[q]; ry[q] = r1[q] * r3[q]; rz[q] = r1[q] * r4[q];
            } else if (dir == 2) {
                rx[q] = rx[q] + r1[q] * r2[q]; ry[q] = ry[q] + r1[q] * r3[q]; rz[q] = rz[q] + r1[q] * r4[q];
            } else {
                rx[q] = (rx[q] + r1[q] * r2[q]) * tmp;
                ry[q] = (ry[q] + r1[q] * r3[q]) * tmp;
                rz[q] = (rz[q] + r1[q] * r4[q]) * tmp;
            }
        }
    }
    orc_fftp3d_real_to_complex(g, rx, d);
    orc_fftp3d_real_to_complex(g, ry, e);
    orc_fftp3d_real_to_complex(g, rz, f);
    free(c1); free(c2); free(c3); free(c4); free(r1); free(r2); free(r3); free(r4);
    free(rx); free(ry); free(rz);
}

/* advect, src/pseudo/pseudospec_phd.f90:23-113: (A.grad)B for a scalar B */
void orc_advect(const orc_grid *g, const double *a, const double *b, const double *c,
                const double *d, double *e) {
    const size_t ns = NS(g), nr = NR(g), plane = (size_t)g->nx * g->ny;
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns);
    double *r1 = malloc(sizeof(double) * nr), *r2 = malloc(sizeof(double) * nr);
    double *r3 = calloc(nr, sizeof(double));
    const double *comp[3] = {a, b, c};
    const size_t nphys = (size_t)g->pkend * plane;
    const double tmp = inv_n2(g);
    for (int dir = 1; dir <= 3; dir++) {
        memcpy(c1, comp[dir - 1], sizeof(cplx) * ns);
        orc_derivk(g, d, c2, dir);
        orc_fftp3d_complex_to_real(g, c1, r1);
        orc_fftp3d_complex_to_real(g, c2, r2);
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < nphys; q++) {
            if (dir == 1) r3[q] = r1[q] * r2[q];
            else if (dir == 2) r3[q] = r3[q] + r1[q] * r2[q];
            else r3[q] = (r3[q] + r1[q] * r2[q]) * tmp;
        }
    }
    orc_fftp3d_real_to_complex(g, r3, e);
    free(c1); free(c2); free(r1); free(r2); free(r3);
}

/* fc_filter, src/pseudo/pseudospec_hd.f90:1082-1115: a *= exp(-alpha(2k_i/N_i/Dk_i)^(2p)), alpha=16 ln 10, p=50 */
void orc_fc_filter(const orc_grid *g, double *a_) {
    cplx *a = (cplx *)a_;
    const double alpha = 16.0 * log(10.0), p2 = 100.0;
    double *fx = malloc(sizeof(double) * g->nxh), *fy = malloc(sizeof(double) * g->ny),
           *fz = malloc(sizeof(double) * g->nz);
    for (int i = 0; i < g->nxh; i++) fx[i] = exp(-alpha * pow(2 * g->kx[i] / g->nx / g->Dkx, p2));
    for (int j = 0; j < g->ny; j++) fy[j] = exp(-alpha * pow(2 * g->ky[j] / g->ny / g->Dky, p2));
    for (int k = 0; k < g->nz; k++) fz[k] = exp(-alpha * pow(2 * g->kz[k] / g->nz / g->Dkz, p2));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                a[q] = a[q] * fx[i] * fy[j] * fz[k];
            }
    free(fx); free(fy); free(fz);
}

/* mean over the physical z rows with weight 1 for kx=0 and 2 otherwise; the shared tail of
 * energy/helicity/cross/divergence (e.g. pseudospec_hd.f90:604-628) */
static double mean_sum(const orc_grid *g, const double *r, double tmp) {
    double dloc = 0.0;
    for (int j = 0; j < g->ny; j++)
        for (int k = 0; k < g->nz - g->cz; k++) dloc = dloc + r[SIDX(g, k, j, 0)] * tmp;
#pragma omp parallel for schedule(static) reduction(+ : dloc)
    for (int i = 1; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz - g->cz; k++) dloc = dloc + 2 * r[SIDX(g, k, j, i)] * tmp;
    return dloc;
}

static double diag_tmp(const orc_grid *g) { return inv_n2(g) / (double)(g->nz - g->cz); }

static void add_abs2(const orc_grid *g, double *R1, const cplx *C1, int first) {
    const size_t ns = NS(g);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < ns; q++) {
        double re = creal(C1[q]), im = cimag(C1[q]);
        R1[q] = first ? re * re + im * im : R1[q] + re * re + im * im;
    }
}

/* energy, src/pseudo/pseudospec_hd.f90:405-635 (kin=0 reproduces the reference:
 * the y-curl is accumulated twice and the z-curl never, :527-551) */
double orc_energy(const orc_grid *g, const double *a, const double *b, const double *c, int kin) {
    const size_t ns = NS(g);
    double *c1 = malloc(sizeof(cplx) * ns), *R1 = malloc(sizeof(double) * ns);
    if (kin == 1) {
        const double *comp[3] = {a, b, c};
        for (int m = 0; m < 3; m++) {
            memcpy(c1, comp[m], sizeof(cplx) * ns);
            orc_fftp1d_complex_to_real_z(g, c1);
            add_abs2(g, R1, (cplx *)c1, m == 0);
        }
    } else if (kin == 0) {
        orc_curlk(g, b, c, c1, 1); orc_fftp1d_complex_to_real_z(g, c1); add_abs2(g, R1, (cplx *)c1, 1);
        orc_curlk(g, a, c, c1, 2); orc_fftp1d_complex_to_real_z(g, c1); add_abs2(g, R1, (cplx *)c1, 0);
        orc_curlk(g, a, c, c1, 2); orc_fftp1d_complex_to_real_z(g, c1); add_abs2(g, R1, (cplx *)c1, 0);
    } else {
        double *c2 = malloc(sizeof(cplx) * ns), *c3 = malloc(sizeof(cplx) * ns), *c4 = malloc(sizeof(cplx) * ns);
        orc_curlk(g, b, c, c1, 1); orc_curlk(g, a, c, c2, 2); orc_curlk(g, a, b, c3, 3);
        orc_curlk(g, c2, c3, c4, 1); orc_curlk(g, c1, c3, c3, 2); orc_curlk(g, c1, c2, c1, 3);
        orc_fftp1d_complex_to_real_z(g, c4); add_abs2(g, R1, (cplx *)c4, 1);
        orc_fftp1d_complex_to_real_z(g, c3); add_abs2(g, R1, (cplx *)c3, 0);
        orc_fftp1d_complex_to_real_z(g, c1); add_abs2(g, R1, (cplx *)c1, 0);
        free(c2); free(c3); free(c4);
    }
    double d = mean_sum(g, R1, diag_tmp(g));
    free(c1); free(R1);
    return d;
}

static void add_redot(const orc_grid *g, double *r1, const cplx *x, const cplx *y, int first) {
    const size_t ns = NS(g);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < ns; q++) {
        double v = creal(x[q] * conj(y[q]));
        r1[q] = first ? v : r1[q] + v;
    }
}

/* helicity, src/pseudo/pseudospec_hd.f90:638-775 */
double orc_helicity(const orc_grid *g, const double *a, const double *b, const double *c) {
    const size_t ns = NS(g);
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns), *r1 = malloc(sizeof(double) * ns);
    const double *comp[3] = {a, b, c};
    for (int m = 0; m < 3; m++) {
        memcpy(c1, comp[m], sizeof(cplx) * ns);
        if (m == 0) orc_curlk(g, b, c, c2, 1);
        else if (m == 1) orc_curlk(g, a, c, c2, 2);
        else orc_curlk(g, a, b, c2, 3);
        orc_fftp1d_complex_to_real_z(g, c1);
        orc_fftp1d_complex_to_real_z(g, c2);
        add_redot(g, r1, (cplx *)c1, (cplx *)c2, m == 0);
    }
    double d = mean_sum(g, r1, diag_tmp(g));
    free(c1); free(c2); free(r1);
    return d;
}

/* cross, src/pseudo/pseudospec_hd.f90:778-940 */
double orc_cross(const orc_grid *g, const double *a, const double *b, const double *c,
                 const double *d, const double *e, const double *f, int kin) {
    const size_t ns = NS(g);
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns), *r1 = malloc(sizeof(double) * ns);
    const double *A[3] = {a, b, c}, *B[3] = {d, e, f};
    for (int m = 0; m < 3; m++) {
        if (kin == 1) {
            memcpy(c1, A[m], sizeof(cplx) * ns);
            memcpy(c2, B[m], sizeof(cplx) * ns);
        } else if (m == 0) { orc_curlk(g, b, c, c1, 1); orc_curlk(g, e, f, c2, 1); }
        else if (m == 1) { orc_curlk(g, a, c, c1, 2); orc_curlk(g, d, f, c2, 2); }
        else { orc_curlk(g, a, b, c1, 3); orc_curlk(g, d, e, c2, 3); }
        orc_fftp1d_complex_to_real_z(g, c1);
        orc_fftp1d_complex_to_real_z(g, c2);
        add_redot(g, r1, (cplx *)c1, (cplx *)c2, m == 0);
    }
    double gsum = mean_sum(g, r1, diag_tmp(g));
    free(c1); free(c2); free(r1);
    return gsum;
}

/* divergence, src/pseudo/pseudospec_hd.f90:1118-1235 */
double orc_divergence(const orc_grid *g, const double *a, const double *b, const double *c) {
    const size_t ns = NS(g);
    double *c1 = malloc(sizeof(cplx) * ns), *c2 = malloc(sizeof(cplx) * ns), *R1 = malloc(sizeof(double) * ns);
    cplx *C1 = (cplx *)c1, *C2 = (cplx *)c2;
    orc_derivk(g, a, c1, 1);
    memcpy(c2, c1, sizeof(cplx) * ns);
    orc_derivk(g, b, c1, 2);
    for (size_t q = 0; q < ns; q++) C2[q] = C2[q] + C1[q];
    orc_derivk(g, c, c1, 3);
    for (size_t q = 0; q < ns; q++) C2[q] = C2[q] + C1[q];
    orc_fftp1d_complex_to_real_z(g, c2);
    add_abs2(g, R1, C2, 1);
    double d = mean_sum(g, R1, diag_tmp(g));
    free(c1); free(c2); free(R1);
    return d;
}

/* variance, src/pseudo/pseudospec_phd.f90:116-196 */
double orc_variance(const orc_grid *g, const double *a_, int kin) {
    const size_t ns = NS(g);
    const cplx *a = (const cplx *)a_;
    cplx *at = malloc(sizeof(cplx) * ns);
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                at[q] = kin == 1 ? a[q] : kk2(g, k, j, i) * a[q];
            }
    orc_fftp1d_complex_to_real_z(g, (double *)at);
    const double tmp = diag_tmp(g);
    double bloc = 0.0;
    for (int j = 0; j < g->ny; j++)
        for (int k = 0; k < g->nz - g->cz; k++) { double m = cabs(at[SIDX(g, k, j, 0)]); bloc = bloc + tmp * (m * m); }
#pragma omp parallel for schedule(static) reduction(+ : bloc)
    for (int i = 1; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz - g->cz; k++) { double m = cabs(at[SIDX(g, k, j, i)]); bloc = bloc + 2 * tmp * (m * m); }
    free(at);
    return bloc;
}

/* product, src/pseudo/pseudospec_phd.f90:199-272 */
double orc_product(const orc_grid *g, const double *a, const double *b) {
    const size_t ns = NS(g);
    cplx *at = malloc(sizeof(cplx) * ns), *bt = malloc(sizeof(cplx) * ns);
    memcpy(at, a, sizeof(cplx) * ns); memcpy(bt, b, sizeof(cplx) * ns);
    orc_fftp1d_complex_to_real_z(g, (double *)at);
    orc_fftp1d_complex_to_real_z(g, (double *)bt);
    const double tmp = diag_tmp(g);
    double cloc = 0.0;
    for (int j = 0; j < g->ny; j++)
        for (int k = 0; k < g->nz - g->cz; k++) { size_t q = SIDX(g, k, j, 0); cloc = cloc + tmp * creal(at[q] * conj(bt[q])); }
#pragma omp parallel for schedule(static) reduction(+ : cloc)
    for (int i = 1; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz - g->cz; k++) { size_t q = SIDX(g, k, j, i); cloc = cloc + 2 * tmp * creal(at[q] * conj(bt[q])); }
    free(at); free(bt);
    return cloc;
}

/* ------------------------------------------------------------------------- */
/* boundary                                                                  */
/* ------------------------------------------------------------------------- */

/* bouncheck_z, src/boundary/boundary_mod.fpp:681-801 */
void orc_bouncheck_z(const orc_grid *g, const double *a, const double *b, double *bot, double *top) {
    const size_t ns = NS(g);
    cplx *C1 = malloc(sizeof(cplx) * ns);
    double *R1 = malloc(sizeof(double) * g->nxh * g->ny), *R2 = malloc(sizeof(double) * g->nxh * g->ny);
    const int w2 = g->nz - g->cz - 1;
    double inv = 1.0 / (double)((long)g->nx * g->ny * g->nz);
    const double tmp = inv * inv;
    memcpy(C1, a, sizeof(cplx) * ns);
    orc_fftp1d_complex_to_real_z(g, (double *)C1);
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++) {
            cplx x = C1[SIDX(g, 0, j, i)], y = C1[SIDX(g, w2, j, i)];
            R1[i * g->ny + j] = creal(x) * creal(x) + cimag(x) * cimag(x);
            R2[i * g->ny + j] = creal(y) * creal(y) + cimag(y) * cimag(y);
        }
    if (b) {
        memcpy(C1, b, sizeof(cplx) * ns);
        orc_fftp1d_complex_to_real_z(g, (double *)C1);
        for (int i = 0; i < g->nxh; i++)
            for (int j = 0; j < g->ny; j++) {
                cplx x = C1[SIDX(g, 0, j, i)], y = C1[SIDX(g, w2, j, i)];
                R1[i * g->ny + j] = R1[i * g->ny + j] + creal(x) * creal(x) + cimag(x) * cimag(x);
                R2[i * g->ny + j] = R2[i * g->ny + j] + creal(y) * creal(y) + cimag(y) * cimag(y);
            }
    }
    double bl = 0.0, tl = 0.0;
    for (int j = 0; j < g->ny; j++) { bl = bl + R1[j] * tmp; tl = tl + R2[j] * tmp; }
    for (int i = 1; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++) { bl = bl + 2 * R1[i * g->ny + j] * tmp; tl = tl + 2 * R2[i * g->ny + j] * tmp; }
    *bot = bl; *top = tl;
    free(C1); free(R1); free(R2);
}

/* poisson_inhomogeneous, src/boundary/boundary_mod.fpp:405-448:
 * d = -im*(kx a + ky b + kz c)/kk2, d(k=0) = 0 (the NaN at k=0 is overwritten) */
static void poisson_inhomogeneous(const orc_grid *g, const cplx *a, const cplx *b, const cplx *c, cplx *d) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                cplx s = g->kx[i] * a[q] + g->ky[j] * b[q] + g->kz[k] * c[q];
                cplx ims = (0.0 * creal(s) - 1.0 * cimag(s)) + I * (0.0 * cimag(s) + 1.0 * creal(s));
                cplx v = -ims;
                double k2 = kk2(g, k, j, i);
                d[q] = creal(v) / k2 + I * (cimag(v) / k2);
            }
    d[0] = 0.0;
}

/* laplace_z, src/boundary/boundary_mod.fpp:451-678 (Dirichlet :490-518, Neumann :521-549,
 * solution and normal derivative :635-675).  Robin combinations are out of scope. */
static int laplace_z(const orc_grid *g, const cplx *bc, cplx *a, cplx *b, int bczsta, int bczend) {
    const int nxh = g->nxh, ny = g->ny, nz = g->nz;
    const double Lz = g->Lz;
    cplx *coef = malloc(sizeof(cplx) * 2 * nxh * ny);
    if (!(bczsta == bczend && (bczsta == 0 || bczsta == 1))) { free(coef); return 3; }
    for (int i = 0; i < nxh; i++)
        for (int j = 0; j < ny; j++) {
            const size_t c = (size_t)i * ny + j;
            const cplx b1 = bc[2 * c], b2 = bc[2 * c + 1];
            const double kh = g->khom[c];
            if (i == 0 && j == 0) {
                if (bczsta == 0) { coef[2 * c] = (b2 - b1) / Lz; coef[2 * c + 1] = b1; }
                else { coef[2 * c] = b1; coef[2 * c + 1] = 0.0; }
                continue;
            }
            const double e = exp(-(kh * Lz));
            if (bczsta == 0) {
                const double tmp = 1.0 / (1 - exp(-(2 * kh * Lz)));
                coef[2 * c] = (b2 - b1 * e) * tmp;
                coef[2 * c + 1] = (b1 - b2 * e) * tmp;
            } else {
                const double tmp = 1.0 / (kh * (1 - exp(-(2 * kh * Lz))));
                coef[2 * c] = (b2 - b1 * e) * tmp;
                coef[2 * c + 1] = (-b1 + b2 * e) * tmp;
            }
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nxh; i++)
        for (int j = 0; j < ny; j++) {
            const size_t c = (size_t)i * ny + j;
            const double kh = g->khom[c];
            const cplx c1 = coef[2 * c], c2 = coef[2 * c + 1];
            for (int k = 0; k < nz; k++) {
                const size_t q = SIDX(g, k, j, i);
                if (i == 0 && j == 0) {
                    a[q] = creal(c1) * g->z[k] + creal(c2);
                    b[q] = creal(c1);
                } else {
                    const double e1 = exp(kh * (g->z[k] - Lz)), e2 = exp(-(kh * g->z[k]));
                    a[q] = c1 * e1 + c2 * e2;
                    b[q] = kh * (c1 * e1 - c2 * e2);
                }
            }
        }
    free(coef);
    return 0;
}

/* sol_project, src/boundary/boundary_mod.fpp:197-402 (bczsta = bczend = 0: homogeneous
 * Dirichlet target; bctarget 1 = Dirichlet on c after projection, 0 = on d) */
int orc_sol_project(const orc_grid *g, double *a_, double *b_, double *c_, double *d_,
                    int bctarget, int bczsta, int bczend) {
    if (bczsta != 0 || bczend != 0 || (bctarget != 0 && bctarget != 1)) return 3;
    const size_t ns = NS(g);
    cplx *a = (cplx *)a_, *b = (cplx *)b_, *c = (cplx *)c_, *d = (cplx *)d_;
    cplx *C1 = malloc(sizeof(cplx) * ns), *C2 = malloc(sizeof(cplx) * ns), *C3 = malloc(sizeof(cplx) * ns);
    cplx *bc = malloc(sizeof(cplx) * 2 * g->nxh * g->ny);
    poisson_inhomogeneous(g, a, b, c, d);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                size_t q = SIDX(g, k, j, i);
                a[q] = a[q] - imk(g->kx[i], d[q]);
                b[q] = b[q] - imk(g->ky[j], d[q]);
                c[q] = c[q] - imk(g->kz[k], d[q]);
            }
    const double tmp = 1.0 / g->nz;
    for (size_t q = 0; q < ns; q++) C1[q] = (bctarget == 0 ? d[q] : c[q]) * tmp;
    orc_fftp1d_complex_to_real_z(g, (double *)C1);
    const int w2 = g->nz - g->cz - 1;
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++) {
            const size_t cc = (size_t)i * g->ny + j;
            cplx x = C1[SIDX(g, 0, j, i)], y = C1[SIDX(g, w2, j, i)];
            bc[2 * cc] = bctarget == 0 ? -x : x;
            bc[2 * cc + 1] = bctarget == 0 ? -y : y;
        }
    int err = laplace_z(g, bc, C2, C3, bczsta + bctarget, bczend + bctarget);
    if (!err) {
        if (bctarget == 0) {
            for (size_t q = 0; q < ns; q++) d[q] = C1[q] + C2[q];
        } else {
            orc_fftp1d_complex_to_real_z(g, d_);
            for (size_t q = 0; q < ns; q++) d[q] = d[q] * tmp + C2[q];
        }
        orc_fftp1d_real_to_complex_z(g, (double *)C2);
        orc_fftp1d_real_to_complex_z(g, (double *)C3);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < g->nxh; i++)
            for (int j = 0; j < g->ny; j++)
                for (int k = 0; k < g->nz; k++) {
                    size_t q = SIDX(g, k, j, i);
                    a[q] = a[q] - imk(g->kx[i], C2[q]);
                    b[q] = b[q] - imk(g->ky[j], C2[q]);
                    c[q] = c[q] - C3[q];
                }
    }
    free(C1); free(C2); free(C3); free(bc);
    return err;
}

/* goto_domain_w_boundaries (z branch), src/boundary/boundary_mod.fpp:72-150 */
static void goto_domain_w_boundaries(const orc_grid *g, cplx *a) {
    const double tmp = 1.0 / (double)g->nz;
    orc_fftp1d_complex_to_real_z(g, (double *)a);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < g->nxh * g->ny; c++)
        for (int k = 0; k < g->nz - g->cz; k++) a[(size_t)c * g->nz + k] = a[(size_t)c * g->nz + k] * tmp;
}

/* noslip_z, src/boundary/vboundary.f90:154-211 */
static void noslip_z(const orc_grid *g, int o, int ord, cplx *vx, cplx *vy, const cplx *pr,
                     const double vbound[2], int pos) {
    const int ind = pos == 0 ? 0 : g->nz - g->cz - 1;
    double tmp = 1 / (double)o;
    if (o != ord) tmp = (double)(o + 1) * tmp;
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++) {
            size_t q = SIDX(g, ind, j, i);
            vx[q] = imk(g->kx[i], pr[q]) * tmp;
            vy[q] = imk(g->ky[j], pr[q]) * tmp;
        }
    vx[SIDX(g, ind, 0, 0)] = (double)(g->nx * g->ny) * vbound[0];
    vy[SIDX(g, ind, 0, 0)] = (double)(g->nx * g->ny) * vbound[1];
}

/* v_imposebc_and_project, src/boundary/vboundary.f90:67-151 (no-slip at both z walls) */
void orc_v_imposebc_and_project(const orc_grid *g, double *vx, double *vy, double *vz, double *pr,
                                int rki, int ord, const double vzsta[2], const double vzend[2]) {
    goto_domain_w_boundaries(g, (cplx *)vx);
    goto_domain_w_boundaries(g, (cplx *)vy);
    noslip_z(g, rki, ord, (cplx *)vx, (cplx *)vy, (const cplx *)pr, vzsta, 0);
    noslip_z(g, rki, ord, (cplx *)vx, (cplx *)vy, (const cplx *)pr, vzend, 1);
    orc_fftp1d_real_to_complex_z(g, vx);
    orc_fftp1d_real_to_complex_z(g, vy);
    orc_sol_project(g, vx, vy, vz, pr, 1, 0, 0);
}

/* s_imposebc + s_constant_z, src/boundary/sboundary.f90:67-165 (wall value hard-coded 0) */
void orc_s_imposebc(const orc_grid *g, double *th_) {
    cplx *th = (cplx *)th_;
    goto_domain_w_boundaries(g, th);
    const int w2 = g->nz - g->cz - 1;
    for (int i = 0; i < g->nxh; i++)
        for (int j = 0; j < g->ny; j++) { th[SIDX(g, 0, j, i)] = 0.0; th[SIDX(g, w2, j, i)] = 0.0; }
    orc_fftp1d_real_to_complex_z(g, th_);
}

/* ------------------------------------------------------------------------- */
/* stage bodies                                                              */
/* ------------------------------------------------------------------------- */

static void rk_update(const orc_grid *g, cplx *v, const cplx *C, const cplx *N, const cplx *f,
                      double dt, double nu, double rmp) {
    const size_t ns = NS(g);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < ns; q++) {
        cplx fv = f ? f[q] : 0.0;
        v[q] = C[q] + dt * (nu * v[q] - N[q] + fv) * rmp;
    }
}

/* hd_rkstep2.f90:1-36 */
void orc_hd_stage(const orc_grid *g, const orc_params *p, int o,
                  double *vx, double *vy, double *vz, double *pr,
                  const double *C1, const double *C2, const double *C3,
                  const double *fx, const double *fy, const double *fz) {
    const size_t ns = NS(g);
    const double rmp = 1 / (double)o;
    double *C4 = malloc(sizeof(cplx) * ns), *C5 = malloc(sizeof(cplx) * ns), *C6 = malloc(sizeof(cplx) * ns);
    orc_gradre(g, vx, vy, vz, C4, C5, C6);
    orc_fc_filter(g, C4); orc_fc_filter(g, C5); orc_fc_filter(g, C6);
    orc_laplak(g, vx, vx); orc_laplak(g, vy, vy); orc_laplak(g, vz, vz);
    rk_update(g, (cplx *)vx, (const cplx *)C1, (const cplx *)C4, (const cplx *)fx, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vy, (const cplx *)C2, (const cplx *)C5, (const cplx *)fy, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vz, (const cplx *)C3, (const cplx *)C6, (const cplx *)fz, p->dt, p->nu, rmp);
    const double zs[2] = {p->vxzsta, p->vyzsta}, ze[2] = {p->vxzend, p->vyzend};
    orc_v_imposebc_and_project(g, vx, vy, vz, pr, o, p->ord, zs, ze);
    free(C4); free(C5); free(C6);
}

/* bouss_rkstep2.f90:1-59 */
void orc_bouss_stage(const orc_grid *g, const orc_params *p, int o,
                     double *vx, double *vy, double *vz, double *th, double *pr,
                     const double *C1, const double *C2, const double *C3, const double *C7,
                     const double *fx, const double *fy, const double *fz, const double *fs) {
    const size_t ns = NS(g), nr = NR(g);
    const double rmp = 1 / (double)o;
    double *C4 = malloc(sizeof(cplx) * ns), *C5 = malloc(sizeof(cplx) * ns), *C6 = malloc(sizeof(cplx) * ns);
    double *C8 = malloc(sizeof(cplx) * ns), *R1 = malloc(sizeof(double) * nr);
    orc_gradre(g, vx, vy, vz, C4, C5, C6);
    orc_advect(g, vx, vy, vz, th, C8);
    {
        cplx *c6 = (cplx *)C6, *c8 = (cplx *)C8;
        const cplx *t = (const cplx *)th, *w = (const cplx *)vz;
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < ns; q++) {
            c6[q] = c6[q] - p->xmom * t[q];
            c8[q] = c8[q] - p->xtemp * w[q];
        }
    }
    orc_fc_filter(g, C4); orc_fc_filter(g, C5); orc_fc_filter(g, C6); orc_fc_filter(g, C8);
    orc_laplak(g, vx, vx); orc_laplak(g, vy, vy); orc_laplak(g, vz, vz); orc_laplak(g, th, th);
    rk_update(g, (cplx *)vx, (const cplx *)C1, (const cplx *)C4, (const cplx *)fx, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vy, (const cplx *)C2, (const cplx *)C5, (const cplx *)fy, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vz, (const cplx *)C3, (const cplx *)C6, (const cplx *)fz, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)th, (const cplx *)C7, (const cplx *)C8, (const cplx *)fs, p->dt, p->kappa, rmp);
    const double zs[2] = {p->vxzsta, p->vyzsta}, ze[2] = {p->vxzend, p->vyzend};
    orc_v_imposebc_and_project(g, vx, vy, vz, pr, o, p->ord, zs, ze);
    orc_s_imposebc(g, th);
    orc_fc_filter(g, th);
    /* c2r -> /nx/ny/nz -> r2c (bouss_rkstep2.f90:56-59) */
    orc_fftp3d_complex_to_real(g, th, R1);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < nr; q++) R1[q] = R1[q] / g->nx / g->ny / g->nz;
    orc_fftp3d_real_to_complex(g, R1, th);
    free(C4); free(C5); free(C6); free(C8); free(R1);
}

/* ROTBOUSS stage, src/include/rotbouss/rotbouss_rkstep2.f90:1-56: the BOUSS stage with the
 * Coriolis term 2 Om x v added to the nonlinear term (:13-17) and without the final theta
 * filter and c2r/r2c round trip. */
void orc_rotbouss_stage(const orc_grid *g, const orc_params *p, const double omega[3], int o,
                        double *vx, double *vy, double *vz, double *th, double *pr,
                        const double *C1, const double *C2, const double *C3, const double *C7) {
    const size_t ns = NS(g);
    const double rmp = 1 / (double)o;
    const double ox = omega[0], oy = omega[1], oz = omega[2];
    double *C4 = malloc(sizeof(cplx) * ns), *C5 = malloc(sizeof(cplx) * ns), *C6 = malloc(sizeof(cplx) * ns);
    double *C8 = malloc(sizeof(cplx) * ns);
    orc_gradre(g, vx, vy, vz, C4, C5, C6);
    orc_advect(g, vx, vy, vz, th, C8);
    {
        cplx *c4 = (cplx *)C4, *c5 = (cplx *)C5, *c6 = (cplx *)C6, *c8 = (cplx *)C8;
        const cplx *t = (const cplx *)th, *u = (const cplx *)vx, *v = (const cplx *)vy, *w = (const cplx *)vz;
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < ns; q++) {
            c4[q] = c4[q] + 2 * (oy * w[q] - oz * v[q]);
            c5[q] = c5[q] + 2 * (oz * u[q] - ox * w[q]);
            c6[q] = c6[q] + 2 * (ox * v[q] - oy * u[q]) - p->xmom * t[q];
            c8[q] = c8[q] - p->xtemp * w[q];
        }
    }
    orc_fc_filter(g, C4); orc_fc_filter(g, C5); orc_fc_filter(g, C6); orc_fc_filter(g, C8);
    orc_laplak(g, vx, vx); orc_laplak(g, vy, vy); orc_laplak(g, vz, vz); orc_laplak(g, th, th);
    rk_update(g, (cplx *)vx, (const cplx *)C1, (const cplx *)C4, NULL, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vy, (const cplx *)C2, (const cplx *)C5, NULL, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)vz, (const cplx *)C3, (const cplx *)C6, NULL, p->dt, p->nu, rmp);
    rk_update(g, (cplx *)th, (const cplx *)C7, (const cplx *)C8, NULL, p->dt, p->kappa, rmp);
    const double zs[2] = {p->vxzsta, p->vyzsta}, ze[2] = {p->vxzend, p->vyzend};
    orc_v_imposebc_and_project(g, vx, vy, vz, pr, o, p->ord, zs, ze);
    orc_s_imposebc(g, th);
    free(C4); free(C5); free(C6); free(C8);
}

/* RK loop of the ROTBOUSS solver (rkstep1 of rotbouss_rkstep1.f90 is the BOUSS one) */
void orc_run_rot(const orc_grid *g, const orc_params *p, const double omega[3], int nsteps,
                 double *vx, double *vy, double *vz, double *th, double *pr) {
    const size_t bytes = sizeof(cplx) * NS(g);
    double *C1 = malloc(bytes), *C2 = malloc(bytes), *C3 = malloc(bytes), *C7 = malloc(bytes);
    for (int t = 0; t < nsteps; t++) {
        memcpy(C1, vx, bytes); memcpy(C2, vy, bytes); memcpy(C3, vz, bytes); memcpy(C7, th, bytes);
        for (int o = p->ord; o >= 1; o--) orc_rotbouss_stage(g, p, omega, o, vx, vy, vz, th, pr, C1, C2, C3, C7);
    }
    free(C1); free(C2); free(C3); free(C7);
}

/* RK loop, src/specter.fpp:1142-1161: rkstep1 copies, then o = ord..1 */
void orc_run(const orc_grid *g, const orc_params *p, int nsteps,
             double *vx, double *vy, double *vz, double *th, double *pr) {
    const size_t bytes = sizeof(cplx) * NS(g);
    double *C1 = malloc(bytes), *C2 = malloc(bytes), *C3 = malloc(bytes), *C7 = th ? malloc(bytes) : NULL;
    for (int t = 0; t < nsteps; t++) {
        memcpy(C1, vx, bytes); memcpy(C2, vy, bytes); memcpy(C3, vz, bytes);
        if (th) memcpy(C7, th, bytes);
        for (int o = p->ord; o >= 1; o--) {
            if (th) orc_bouss_stage(g, p, o, vx, vy, vz, th, pr, C1, C2, C3, C7, NULL, NULL, NULL, NULL);
            else orc_hd_stage(g, p, o, vx, vy, vz, pr, C1, C2, C3, NULL, NULL, NULL);
        }
    }
    free(C1); free(C2); free(C3); free(C7);
}

/* one-off unnormalised 1-D DFT, exposed so the FFT can be checked against numpy.fft */
void orc_fft_1d(int n, double *x, int sign) {
    orc_fftplan *p = orc_fft_plan(n);
    cplx *w = malloc(sizeof(cplx) * orc_fft_work(p));
    orc_fft_exec(p, (cplx *)x, sign, w);
    free(w);
    orc_fft_free(p);
}
