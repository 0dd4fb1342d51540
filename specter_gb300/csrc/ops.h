// Host-side operations on device fields.  Every operation is the GB300 counterpart of one
// reference routine (named in ops.cu) and enqueues kernels on the plan's stream.
#pragma once

#include "plan.h"

namespace sg {

struct StageParams {
    int solver;  // 0 HD, 1 BOUSS, 2 ROTBOUSS
    int ord;
    double dt, nu, kappa, xmom, xtemp;  // xmom, xtemp already multiplied by gama
    double vzsta[2], vzend[2];
    double omega[3];  // rotation rate (ROTBOUSS)
    // 1 on an FP64 plan: the nonlinear term runs in FP32 (on an FP32 copy of the state, through
    // a companion FP32 plan); the state, the RK update, the wall round trips, the projection, the
    // filter and the reductions stay FP64
    int nl_fp32;
};

template <typename T> struct Ops {
    // NL += 2 Om x v, component-wise as rotbouss_rkstep2.f90:13-17
    static int coriolis(Plan &P, void *const N[3], const void *const v[3], const double omega[3]);
    // fftp
    static int fftp1d_r2c_z(Plan &P, void *inout);
    static int fftp1d_c2r_z(Plan &P, void *inout);
    static int fftp2d_r2c_xy(Plan &P, const void *rin, void *cout);
    static int fftp2d_c2r_xy(Plan &P, const void *cin, void *rout);
    static int fftp3d_r2c(Plan &P, const void *rin, void *cout);
    static int fftp3d_c2r(Plan &P, void *cin, void *rout);
    // pseudo
    static int derivk(Plan &P, const void *a, void *b, int dir);
    static int laplak(Plan &P, const void *a, void *b);
    static int curlk(Plan &P, const void *a, const void *b, void *c, int dir);
    static int fc_filter(Plan &P, void *a);
    // NL terms of components [c0, c1) (0..2 velocity, 3 scalar) into out[] (spectral); with
    // `mixed` given, stops before the z transform and returns the mixed-domain NL (scratch)
    static int nonlinear(Plan &P, const void *const v[3], const void *th, void *const out[4], int c0, int c1,
                         const void **mixed = nullptr);
    static int energy(Plan &P, const void *a, const void *b, const void *c, int kin, double *out);
    static int helicity(Plan &P, const void *a, const void *b, const void *c, double *out);
    static int cross(Plan &P, const void *const A[3], const void *const B[3], int kin, double *out);
    static int divergence(Plan &P, const void *a, const void *b, const void *c, double *out);
    static int variance(Plan &P, const void *a, int kin, double *out);
    static int product(Plan &P, const void *a, const void *b, double *out);
    // boundary
    static int bouncheck_z(Plan &P, const void *a, const void *b, double *bot, double *top);
    static int sol_project(Plan &P, void *a, void *b, void *c, void *d, int bctarget);
    static int v_imposebc_and_project(Plan &P, void *vx, void *vy, void *vz, void *pr, int rki, int ord,
                                      const double vzsta[2], const double vzend[2]);
    static int s_imposebc(Plan &P, void *th);
    // stages (composition of the above, the reference's call sequence)
    static int stage(Plan &P, const StageParams &sp, int o, void *const v[4], void *pr, const void *const Cold[4]);
    // helpers
    static int axpy_sub(Plan &P, void *y, const void *x, double s);
    static int rk_update(Plan &P, void *v, const void *Cold, const void *N, double dt, double nu, double rmp);
    static int scale_real(Plan &P, void *r, double s);
};

int check_launch(const char *what);

}  // namespace sg
