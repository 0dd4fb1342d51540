/*
 * ORACLE — test infrastructure only.
 *
 * A double-precision CPU restatement (C99 + OpenMP) of SPECTER's per-RK-stage
 * hot path, in the reference's own data layouts:
 *   spectral / mixed arrays  C(nz, ny, nx/2+1), z fastest   -> a[(kx*ny + ky)*nz + z]
 *   physical arrays          R(nx, ny, nz),    x fastest   -> r[(z*ny + y)*nx + x]
 * where nz is the TOTAL z size (physical points + continuation points Cz).
 *
 * Parity status: the reference ships no golden vectors and its Fortran/FFTW/MPI
 * build cannot be compiled here (no Fortran compiler, no FFTW).  This oracle
 * is pinned by (1) the reference's own known-answer programs
 * (src/tests/fc_dirichlet.f90, fft.f90, energy.f90, poisson.f90) re-run with
 * explicit thresholds, (2) its FFT checked against numpy.fft, and (3) the
 * transforms checked against an independent numpy restatement
 * (tests/golden/make_golden.py).  Bit-level parity with FFTW is unpinned.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library.  The shipped library (libspecter_gpu.so) never links it.
 */
#ifndef SPECTER_ORACLE_H
#define SPECTER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_grid orc_grid;

typedef struct orc_params {
    double dt, nu, kappa;
    double xmom, xtemp;                 /* already multiplied by gama (specter.fpp:490-491) */
    double vxzsta, vyzsta, vxzend, vyzend;
    int ord;
} orc_params;

/* grid + FC-Gram plan (specter.fpp:683-800, fcgram_mod.f90:49-144,180-257).
 * Lx, Ly in units of 2*pi (periodic), Lz in units of 1 (non-periodic).
 * Returns NULL and sets *err (1 bad shape, 2 missing table). */
orc_grid *orc_create(int nx, int ny, int nz, int cz, int oz, double Lx, double Ly, double Lz,
                     const char *tdir, int *err);
void orc_destroy(orc_grid *g);
void orc_set_threads(int n);
int orc_get_threads(void);
void orc_grid_info(const orc_grid *g, double *kx, double *ky, double *kz, double *z, double *dir);

/* fftp (src/fftp/fftp.fpp) */
void orc_fftp3d_real_to_complex(const orc_grid *g, const double *in, double *out);
void orc_fftp3d_complex_to_real(const orc_grid *g, double *in, double *out); /* in destroyed */
void orc_fftp2d_real_to_complex_xy(const orc_grid *g, const double *in, double *out);
void orc_fftp2d_complex_to_real_xy(const orc_grid *g, const double *in, double *out);
void orc_fftp1d_real_to_complex_z(const orc_grid *g, double *inout);
void orc_fftp1d_complex_to_real_z(const orc_grid *g, double *inout);

/* pseudo (src/pseudo/pseudospec_hd.f90, pseudospec_phd.f90); complex arrays as interleaved doubles */
void orc_derivk(const orc_grid *g, const double *a, double *b, int dir);
void orc_laplak(const orc_grid *g, const double *a, double *b);
void orc_curlk(const orc_grid *g, const double *a, const double *b, double *c, int dir);
void orc_gradre(const orc_grid *g, const double *a, const double *b, const double *c,
                double *d, double *e, double *f);
void orc_advect(const orc_grid *g, const double *a, const double *b, const double *c,
                const double *d, double *e);
void orc_fc_filter(const orc_grid *g, double *a);
double orc_energy(const orc_grid *g, const double *a, const double *b, const double *c, int kin);
double orc_helicity(const orc_grid *g, const double *a, const double *b, const double *c);
double orc_cross(const orc_grid *g, const double *a, const double *b, const double *c,
                 const double *d, const double *e, const double *f, int kin);
double orc_divergence(const orc_grid *g, const double *a, const double *b, const double *c);
double orc_variance(const orc_grid *g, const double *a, int kin);
double orc_product(const orc_grid *g, const double *a, const double *b);

/* boundary (src/boundary/boundary_mod.fpp, vboundary.f90, sboundary.f90) */
void orc_bouncheck_z(const orc_grid *g, const double *a, const double *b, double *bot, double *top);
int orc_sol_project(const orc_grid *g, double *a, double *b, double *c, double *d,
                    int bctarget, int bczsta, int bczend);
void orc_v_imposebc_and_project(const orc_grid *g, double *vx, double *vy, double *vz, double *pr,
                                int rki, int ord, const double vzsta[2], const double vzend[2]);
void orc_s_imposebc(const orc_grid *g, double *th);

/* solver stage bodies (src/include/hd/hd_rkstep2.f90, src/include/bouss/bouss_rkstep2.f90) and the RK loop
 * (specter.fpp:1142-1161).  fx..fs may be NULL for zero forcing. */
void orc_hd_stage(const orc_grid *g, const orc_params *p, int o,
                  double *vx, double *vy, double *vz, double *pr,
                  const double *C1, const double *C2, const double *C3,
                  const double *fx, const double *fy, const double *fz);
void orc_bouss_stage(const orc_grid *g, const orc_params *p, int o,
                     double *vx, double *vy, double *vz, double *th, double *pr,
                     const double *C1, const double *C2, const double *C3, const double *C7,
                     const double *fx, const double *fy, const double *fz, const double *fs);
void orc_fft_1d(int n, double *x, int sign);
/* nsteps full RK steps; th == NULL selects the HD solver */
void orc_run(const orc_grid *g, const orc_params *p, int nsteps,
             double *vx, double *vy, double *vz, double *th, double *pr);
void orc_rotbouss_stage(const orc_grid *g, const orc_params *p, const double omega[3], int o,
                        double *vx, double *vy, double *vz, double *th, double *pr,
                        const double *C1, const double *C2, const double *C3, const double *C7);
void orc_run_rot(const orc_grid *g, const orc_params *p, const double omega[3], int nsteps,
                 double *vx, double *vy, double *vz, double *th, double *pr);

#ifdef __cplusplus
}
#endif
#endif
