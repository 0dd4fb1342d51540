/*
 * specter_gpu.h — C ABI of the GB300 (sm_103a) implementation of SPECTER's per-RK-stage hot path.
 *
 * The Fortran driver reaches these entry points through iso_c_binding; each one replaces the
 * reference routine cited beside it (paths inside specter-cfd/SPECTER).
 *
 * Conventions
 *   - Every function returns an int status: 0 = SPECTER_OK, otherwise one of the codes below;
 *     specter_last_error() returns a message for the last failure on the calling thread.
 *     The reference's equivalent is PRINT + MPI_FINALIZE + STOP (e.g. fcgram_mod.f90:113-141).
 *   - Fields are device-resident handles owned by the library.  Host arrays passed to
 *     specter_field_upload/download use the reference layouts: complex C(nz, ny, nx/2+1)
 *     (z fastest, interleaved re/im) and real R(nx, ny, nz) (x fastest), in the plan's
 *     precision (FP64: double, FP32: float).  nz is the TOTAL z size including Cz.
 *   - All work of a plan runs in order on the plan's CUDA stream; calls return once the work
 *     is enqueued, except reductions (which return a host scalar) and downloads.
 *   - The `comm` argument of the reference (MPI communicator) has no counterpart: one GPU.
 */
#ifndef SPECTER_GPU_H
#define SPECTER_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SPECTER_OK = 0,
    SPECTER_ERR_SHAPE = 1,     /* unsupported grid shape / periodicity */
    SPECTER_ERR_TABLE = 2,     /* FC-Gram table missing or short (fcgram_mod.f90:225-249) */
    SPECTER_ERR_BC = 3,        /* unsupported boundary-condition combination */
    SPECTER_ERR_OOM = 4,       /* device allocation failed */
    SPECTER_ERR_CUDA = 5,      /* CUDA runtime error */
    SPECTER_ERR_NONFINITE = 6, /* non-finite value detected in the state */
    SPECTER_ERR_ARG = 7,       /* bad argument (null handle, wrong field kind, ...) */
    /* 8 is unused (no entry point waits with a time limit) */
    SPECTER_ERR_STATE = 9      /* handle used with a different plan / precision */
};

enum { SPECTER_FP64 = 0, SPECTER_FP32 = 1 };            /* plan precision */
enum { SPECTER_COMPLEX = 0, SPECTER_REAL = 1 };         /* field kind */
enum { SPECTER_HD = 0, SPECTER_BOUSS = 1, SPECTER_ROTBOUSS = 2 };  /* solver (src/include/hd, bouss, rotbouss) */

typedef struct specter_plan specter_plan;
typedef struct specter_field specter_field;
typedef struct specter_solver specter_solver;

const char *specter_last_error(void);
int specter_version(void);
int specter_device_count(int *count);
/* selects the CUDA device used by plans created afterwards on the calling thread */
int specter_set_device(int device);
/* FC-Gram table validation (no device work): reads A{C}-{d}.dat and Q{d}.dat under tdir as
 * load_dirichlet_tables does (src/fftp/fcgram_mod.f90:180-257) and returns
 * out = {max |Q^T Q - I|, max |dir|, max_i sum_j |dir_ij|} for dir = A Q^T: the Gram basis'
 * orthonormality and the continuation's amplification of rounding in the wall-adjacent points. */
int specter_table_check(const char *tdir, int C, int d, double out[3]);
/* free and total device memory of the current device (admission by memory budget) */
int specter_device_memory(unsigned long long *free_bytes, unsigned long long *total_bytes);

/* ---- plan: fcgram_create_plan (src/fftp/fcgram_mod.f90:49-144) + grid/kes setup
 *      (src/specter.fpp:683-800).  n = (nx, ny, nz) totals, c = (Cx, Cy, Cz), o = (ox, oy, oz)
 *      as in the reference (x, y periodic: Cx = Cy = ox = oy = 0).  len = (Lx, Ly, Lz): Lx, Ly
 *      in units of 2*pi, Lz in units of 1 (boxparams namelist, specter.fpp:379-394).
 *      tdir: directory holding A{C}-{d}.dat and Q{d}.dat (load_dirichlet_tables :180-257). */
int specter_plan_create(const int n[3], const int c[3], const int o[3], const double len[3],
                        const char *tdir, int precision, specter_plan **out);
int specter_plan_destroy(specter_plan *plan);            /* fcgram_destroy_plan :147-177 */
/* info[0..7] = nx, ny, nz, Cz, oz, nx/2+1, padded kx stride, precision */
int specter_plan_info(const specter_plan *plan, int info[8]);
/* FFT engine per axis (x = the half length nx/2, y, z): out[4*a + 0..3] = working length L,
 * split L1, L2 of the register four-step kernels (0, 0: the generic engine serves the axis) and
 * 1 when the axis runs Bluestein's algorithm over L.  FP32 plans only choose four-step splits. */
int specter_plan_engines(const specter_plan *plan, int out[12]);
/* kx[nx/2+1], ky[ny], kz[nz], z[nz] (the kes and grid modules), dir[Cz*oz] Fortran order */
int specter_plan_arrays(const specter_plan *plan, double *kx, double *ky, double *kz, double *z, double *dir);
int specter_plan_synchronize(specter_plan *plan);
/* the plan's cudaStream_t, for callers that record CUDA events around library work */
int specter_plan_stream(specter_plan *plan, void **stream);

/* ---- fields (device-resident arrays of the plan's precision) */
int specter_field_create(specter_plan *plan, int kind, specter_field **out);
int specter_field_destroy(specter_field *f);
int specter_field_upload(specter_field *f, const void *host);    /* reference layout */
int specter_field_download(const specter_field *f, void *host);  /* reference layout */
/* several fields of one plan (no reference counterpart): host copies on a copy stream overlap the
 * layout conversions (two staging buffers).  Upload returns with the copies queued (host buffers
 * must stay valid until the plan is synchronised); download returns with the data in host memory. */
int specter_fields_upload(int n, specter_field *const *fields, const void *const *hosts);
int specter_fields_download(int n, specter_field *const *fields, void *const *hosts);
int specter_field_copy(specter_field *dst, const specter_field *src);
int specter_field_zero(specter_field *f);
/* upload/download of a contiguous batch of host rows is the same call with a pinned buffer;
 * the device pointer of a field, for interop.  Device layout: complex fields are
 * f[(z * ny + ky) * ldx + kx] (kx fastest, row stride ldx = nx/2+1 rounded up to 8, info[6] of
 * specter_plan_info); real fields are r[(z * ny + y) * nx + x]. */
int specter_field_device_ptr(specter_field *f, void **ptr, long long *bytes);

/* ---- fftp (src/fftp/fftp.fpp) */
int specter_fftp3d_real_to_complex(specter_plan *plan, const specter_field *in, specter_field *out);   /* :388-425 */
int specter_fftp3d_complex_to_real(specter_plan *plan, specter_field *in, specter_field *out);         /* :789-821, in destroyed */
int specter_fftp2d_real_to_complex_xy(specter_plan *plan, const specter_field *in, specter_field *out);/* :428-524 */
int specter_fftp2d_complex_to_real_xy(specter_plan *plan, const specter_field *in, specter_field *out);/* :824-919 */
int specter_fftp1d_real_to_complex_z(specter_plan *plan, specter_field *inout);                       /* :720-786 */
int specter_fftp1d_complex_to_real_z(specter_plan *plan, specter_field *inout);                       /* :1060-1094 */

/* ---- pseudo (src/pseudo/pseudospec_hd.f90, pseudospec_phd.f90) */
int specter_derivk(specter_plan *plan, const specter_field *a, specter_field *b, int dir);           /* hd :28-94 */
int specter_laplak(specter_plan *plan, const specter_field *a, specter_field *b);                    /* hd :97-127 */
int specter_curlk(specter_plan *plan, const specter_field *a, const specter_field *b,
                  specter_field *c, int dir);                                                        /* hd :130-206 */
int specter_gradre(specter_plan *plan, const specter_field *a, const specter_field *b,
                   const specter_field *c, specter_field *d, specter_field *e, specter_field *f);    /* hd :209-319 */
int specter_advect(specter_plan *plan, const specter_field *a, const specter_field *b,
                   const specter_field *c, const specter_field *d, specter_field *e);                /* phd :23-113 */
int specter_fc_filter(specter_plan *plan, specter_field *a);                                         /* hd :1082-1115 */
int specter_energy(specter_plan *plan, const specter_field *a, const specter_field *b,
                   const specter_field *c, int kin, double *out);                                    /* hd :405-635 */
int specter_helicity(specter_plan *plan, const specter_field *a, const specter_field *b,
                     const specter_field *c, double *out);                                           /* hd :638-775 */
int specter_cross(specter_plan *plan, const specter_field *a, const specter_field *b,
                  const specter_field *c, const specter_field *d, const specter_field *e,
                  const specter_field *f, int kin, double *out);                                     /* hd :778-940 */
int specter_divergence(specter_plan *plan, const specter_field *a, const specter_field *b,
                       const specter_field *c, double *out);                                         /* hd :1118-1235 */
int specter_variance(specter_plan *plan, const specter_field *a, int kin, double *out);              /* phd :116-196 */
int specter_product(specter_plan *plan, const specter_field *a, const specter_field *b, double *out);/* phd :199-272 */

/* ---- boundary (src/boundary/boundary_mod.fpp, vboundary.f90, sboundary.f90) */
int specter_bouncheck_z(specter_plan *plan, const specter_field *a, const specter_field *b,
                        double *bot, double *top);                                                   /* boundary_mod :681-801 (b may be NULL) */
/* Same result as specter_bouncheck_z, computed without allocating any memory.  It has no
 * counterpart in the reference.  For callers that may not allocate once they are running: a
 * serving loop that has committed its device memory budget, or code in the middle of the RK
 * loop that cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  Its working
 * memory is one fixed device array (4 MiB, held on every GPU that loads the library until
 * exit): grids with more than 65536 (kx, ky) columns are rejected with SPECTER_ERR_SHAPE.
 * All calls share that array, so calls that overlap on the GPU race; the first call on a
 * device looks up the array's address and should come before any stream capture. */
int specter_bouncheck_z_static(specter_plan *plan, const specter_field *a, const specter_field *b,
                               double *bot, double *top);
int specter_sol_project(specter_plan *plan, specter_field *a, specter_field *b, specter_field *c,
                        specter_field *d, int bctarget, int bczsta, int bczend);                     /* boundary_mod :197-402 */
int specter_v_imposebc_and_project(specter_plan *plan, specter_field *vx, specter_field *vy,
                                   specter_field *vz, specter_field *pr, int rki, int ord,
                                   const double v_zsta[2], const double v_zend[2]);                  /* vboundary :67-151 */
int specter_s_imposebc(specter_plan *plan, specter_field *th);                                       /* sboundary :67-119 */

/* ---- solver: the RK loop (src/specter.fpp:1142-1161) with the stage bodies
 *      src/include/hd/hd_rkstep2.f90, src/include/bouss/bouss_rkstep2.f90 and
 *      src/include/rotbouss/rotbouss_rkstep2.f90. */
typedef struct specter_solver_params {
    int solver;              /* SPECTER_HD, SPECTER_BOUSS or SPECTER_ROTBOUSS */
    int ord;                 /* RK order (parameter ORD) */
    double dt, nu, kappa;    /* &parameter dt, &velocity nu, &scalar kappa */
    double gama, xmom, xtemp;/* &boussinesq; xmom and xtemp are multiplied by gama (specter.fpp:490-491) */
    double v_zsta[2];        /* &velbound vxzsta, vyzsta */
    double v_zend[2];        /* &velbound vxzend, vyzend */
    int fused;               /* 1: fused GB300 stage kernels; 0: the reference call sequence */
    double omega[3];         /* &rotation omegax, omegay, omegaz (SPECTER_ROTBOUSS) */
    int nl_fp32;             /* the precision form (fused solvers on an FP64 plan; no reference
                              * counterpart): the nonlinear term -- gradre/advect's transforms and
                              * products -- in FP32 on an FP32 copy of the state; the state, the
                              * RK update, the wall round trips with the FC-Gram continuation, the
                              * projection, fc_filter and all reductions in FP64 */
} specter_solver_params;

int specter_solver_create(specter_plan *plan, const specter_solver_params *p, specter_solver **out);
int specter_solver_destroy(specter_solver *s);
/* state handles owned by the solver: vx, vy, vz, th (NULL for HD), pr */
int specter_solver_fields(specter_solver *s, specter_field **vx, specter_field **vy,
                          specter_field **vz, specter_field **th, specter_field **pr);
int specter_solver_step(specter_solver *s, int nsteps);      /* rkstep1 + ORD stages per step */
int specter_solver_stage(specter_solver *s, int o);          /* one stage o (rkstep2 body) */
/* checks the state for non-finite values (SPECTER_ERR_NONFINITE if any) */
int specter_solver_check(specter_solver *s);

/* ---- autotuning and CUDA graphs (no reference counterpart: the ensemble and serving forms).
 * specter_solver_autotune times RK steps of the solver for each tile-width cap of the z, y, x
 *      and fused kernel families and keeps the fastest cap per family in the solver's plan; the
 *      state is restored afterwards; for fused solvers it also picks the one- or two-kernel
 *      velocity stage.  caps (optional, 5 ints) receives the caps (z, y, x, fused) and the
 *      velocity_split choice.
 * specter_plan_tile_caps sets the caps directly (entries <= 0 leave a cap unchanged).
 * specter_graph_create captures nsteps RK steps of n solvers into one CUDA graph: each
 *      solver's kernels stay on its plan stream, the chains of different plans are parallel
 *      branches.  specter_graph_launch runs it, ordered after the work already queued on those
 *      plan streams and before work queued on them afterwards.  The solvers' own state fields
 *      are advanced in place.  Destroy a graph before its solvers. */
typedef struct specter_graph specter_graph;
int specter_solver_autotune(specter_solver *s, int caps[5]);
int specter_plan_tile_caps(specter_plan *plan, const int caps[4]);
/* named plan options: "velocity_split" (0/1: fused velocity stage as one kernel or as a
 * per-component kernel plus a projection kernel), "tile_cap_z|y|x|fused" (1, 2, 4, 8, 16),
 * "ff_threads" (256 or 384: threads per block of the float-float column kernels of nl_fp32
 * solvers on the generic transform engine; the autotuner picks it for those solvers),
 * "ff_engine" (1, the default: those kernels use the three-step register Bluestein engine when
 * nz + C lies in (270, 540]; 0: always the generic engine), "ff_pair_proj" and "ff_pair_cols"
 * (0/1: on that engine, the projection kernel and the other column kernels run as one 576-thread
 * block per SM or as two 288-thread blocks; the autotuner picks them), "ff_zoom" (1, the default:
 * on that engine the wall round trips are window corrections of the spectrum when C + 2d = 35 and
 * nz + C + 34 <= 576; 0: an inverse and a forward transform each) */
int specter_plan_set_option(specter_plan *plan, const char *name, int value);
/* the current value of a named plan option (the names above); no reference counterpart */
int specter_plan_get_option(specter_plan *plan, const char *name, int *value);
int specter_graph_create(specter_solver *const *solvers, int n, int nsteps, specter_graph **out);
int specter_graph_launch(specter_graph *g);
int specter_graph_synchronize(specter_graph *g);
int specter_graph_kernels(specter_graph *g, long long *kernels);  /* kernels per launch */
int specter_graph_query(specter_graph *g, int *done);  /* 1 when every launch so far has finished */
/* device bytes held by the solver: its state, RK and fused-stage buffers and its plan (tables
 * and the scratch fields allocated so far) */
int specter_solver_memory(specter_solver *s, unsigned long long *bytes);
int specter_graph_destroy(specter_graph *g);

/* ---- batched ensembles (no reference counterpart: the ensemble form).
 * specter_batch_create records one RK step of each of n fused FP32 HD solvers (each on a plan
 *      of its own; RK order >= 2; the split velocity stage is selected on their plans) and
 *      captures it as one CUDA graph of batched launches: the i-th kernel of every solver's
 *      step runs as one launch per distinct kernel (FFT length class, tile width) over the tiles
 *      of all the solvers that use it, so an ensemble of uneven grids takes a few dozen
 *      launches a step instead of a few per solver.  Each solver computes exactly what its own
 *      steps would.
 * specter_batch_step advances every solver's state by nsteps RK steps (after the work already
 *      queued on the solvers' plan streams); specter_batch_synchronize waits for it.
 *      specter_batch_kernels gives the launches per step.  Destroy a batch before its solvers. */
typedef struct specter_batch specter_batch;
int specter_batch_create(specter_solver *const *solvers, int n, specter_batch **out);
int specter_batch_step(specter_batch *b, int nsteps);
int specter_batch_synchronize(specter_batch *b);
int specter_batch_kernels(specter_batch *b, long long *kernels);
int specter_batch_destroy(specter_batch *b);

/* ---- timers: out = {ffttime, tratime, comtime, conttime, tottime, stages} in seconds,
 *      accumulated from CUDA events (the reference's fftp_mod.fpp:32-37 accumulators) */
int specter_timers(specter_plan *plan, double out[6]);
int specter_timers_reset(specter_plan *plan);

/* ---- kernel accounting (no reference counterpart; measurement support).
 *      specter_profile(plan, 1) brackets every kernel launch of the plan with CUDA events on
 *      the plan stream; specter_profile_report writes one line per kernel name:
 *      "name launches total_ms algorithmic_bytes\n" (reset with specter_profile(plan, 0)).
 *      specter_launch_count returns the number of kernels the plan has launched. */
int specter_profile(specter_plan *plan, int enable);
int specter_profile_report(specter_plan *plan, char *buf, int buflen);
int specter_launch_count(specter_plan *plan, long long *count);

#ifdef __cplusplus
}
#endif
#endif
