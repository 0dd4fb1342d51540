// Elementwise spectral kernels, wall kernels and deterministic FP64 reductions.
#pragma once

#include "kernels.cuh"

namespace sg {

// Grid-stride loop over every (z, ky, kx < nxh) with z in [z0, z1); q is the element offset.
#define SG_ELEMS_BEGIN(g, z0, z1)                                                          \
    {                                                                                      \
        const long long _n = (long long)((z1) - (z0)) * (g).ny * (g).nxh;                  \
        for (long long _i = (long long)blockIdx.x * blockDim.x + threadIdx.x; _i < _n;     \
             _i += (long long)gridDim.x * blockDim.x) {                                    \
            const int kx = (int)(_i % (g).nxh);                                            \
            const int _r = (int)(_i / (g).nxh);                                            \
            const int ky = _r % (g).ny;                                                    \
            const int z = (z0) + _r / (g).ny;                                              \
            const size_t q = ((size_t)z * (g).ny + ky) * (g).ldx + kx;                     \
            (void)z; (void)ky;
#define SG_ELEMS_END \
    }                \
    }

// Coriolis term of the ROTBOUSS nonlinear term, src/include/rotbouss/rotbouss_rkstep2.f90:13-17:
// N += 2 Om x v, each component as the reference writes it.
template <typename T>
__global__ void k_coriolis(Geo g, C2<T> *n0, C2<T> *n1, C2<T> *n2, const C2<T> *vx, const C2<T> *vy,
                           const C2<T> *vz, T ox, T oy, T oz) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
    const C2<T> u = vx[q], v = vy[q], w = vz[q];
    const T two = (T)2;
    n0[q] = mk<T>(n0[q].x + two * (oy * w.x - oz * v.x), n0[q].y + two * (oy * w.y - oz * v.y));
    n1[q] = mk<T>(n1[q].x + two * (oz * u.x - ox * w.x), n1[q].y + two * (oz * u.y - ox * w.y));
    n2[q] = mk<T>(n2[q].x + two * (ox * v.x - oy * u.x), n2[q].y + two * (ox * v.y - oy * u.y));
    SG_ELEMS_END
}

template <typename T>
__device__ __forceinline__ T kk2_at(const Geo &g, int z, int ky, int kx) {
    const T a = g.KX<T>(kx), b = g.KY<T>(ky), c = g.KZ<T>(z);
    return a * a + b * b + c * c;
}

// derivk, src/pseudo/pseudospec_hd.f90:28-94
template <typename T>
__global__ void k_derivk(Geo g, const C2<T> *a, C2<T> *b, int dir) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const T k = dir == 1 ? g.KX<T>(kx) : dir == 2 ? g.KY<T>(ky) : g.KZ<T>(z);
        b[q] = cimk(k, a[q]);
    SG_ELEMS_END
}

// laplak, src/pseudo/pseudospec_hd.f90:97-127
template <typename T>
__global__ void k_laplak(Geo g, const C2<T> *a, C2<T> *b) {
    SG_ELEMS_BEGIN(g, 0, g.nz) b[q] = cscale(a[q], -kk2_at<T>(g, z, ky, kx)); SG_ELEMS_END
}

// curlk, src/pseudo/pseudospec_hd.f90:130-206
template <typename T>
__global__ void k_curlk(Geo g, const C2<T> *a, const C2<T> *b, C2<T> *c, int dir) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const T kx_ = g.KX<T>(kx), ky_ = g.KY<T>(ky), kz_ = g.KZ<T>(z);
        C2<T> r;
        if (dir == 1) r = csub(cimk(ky_, b[q]), cimk(kz_, a[q]));
        else if (dir == 2) r = csub(cimk(kz_, a[q]), cimk(kx_, b[q]));
        else r = csub(cimk(kx_, b[q]), cimk(ky_, a[q]));
        c[q] = r;
    SG_ELEMS_END
}

// fc_filter, src/pseudo/pseudospec_hd.f90:1082-1115 (factors precomputed in FP64)
template <typename T>
__global__ void k_filter(Geo g, C2<T> *a) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        C2<T> v = a[q];
        v = cscale(v, g.FX<T>(kx));
        v = cscale(v, g.FY<T>(ky));
        v = cscale(v, g.FZ<T>(z));
        a[q] = v;
    SG_ELEMS_END
}

// laplak + RK update of one component: v = C + dt*(nu*(-kk2 v) - N)*rmp
// (hd_rkstep2.f90:18-32 with zero forcing; bouss_rkstep2.f90:35-48)
template <typename T>
__global__ void k_rk_update(Geo g, C2<T> *v, const C2<T> *Cold, const C2<T> *N, double dt, double nu, double rmp) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const C2<T> lap = cscale(v[q], -kk2_at<T>(g, z, ky, kx));
        const T dtT = (T)dt, nuT = (T)nu, rT = (T)rmp;
        const C2<T> c = Cold[q], n = N[q];
        v[q] = mk<T>(c.x + dtT * (nuT * lap.x - n.x) * rT, c.y + dtT * (nuT * lap.y - n.y) * rT);
    SG_ELEMS_END
}

// y = y - s*x  (buoyancy C6 -= xmom*th, heat current C8 -= xtemp*vz; bouss_rkstep2.f90:9-18)
template <typename T>
__global__ void k_sub_scaled(Geo g, C2<T> *y, const C2<T> *x, double s) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const C2<T> a = y[q], b = x[q];
        y[q] = mk<T>(a.x - (T)s * b.x, a.y - (T)s * b.y);
    SG_ELEMS_END
}

// divergence field ikx a + iky b + ikz c (pseudospec_hd.f90:1150-1180)
template <typename T>
__global__ void k_div(Geo g, const C2<T> *a, const C2<T> *b, const C2<T> *c, C2<T> *d) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        C2<T> s = cimk(g.KX<T>(kx), a[q]);
        s = cadd(s, cimk(g.KY<T>(ky), b[q]));
        s = cadd(s, cimk(g.KZ<T>(z), c[q]));
        d[q] = s;
    SG_ELEMS_END
}

// out = kk2 * a (variance kin=0, pseudospec_phd.f90:151-155)
template <typename T>
__global__ void k_kk2_mul(Geo g, const C2<T> *a, C2<T> *b) {
    SG_ELEMS_BEGIN(g, 0, g.nz) b[q] = cscale(a[q], kk2_at<T>(g, z, ky, kx)); SG_ELEMS_END
}

// poisson_inhomogeneous (boundary_mod.fpp:405-448) fused with the inhomogeneous
// projection and the scaled copy C1 = (bctarget ? c : d)/nz (sol_project :245-281)
template <typename T>
__global__ void k_poisson(Geo g, C2<T> *a, C2<T> *b, C2<T> *c, C2<T> *d, C2<T> *C1, int bctarget) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const T kx_ = g.KX<T>(kx), ky_ = g.KY<T>(ky), kz_ = g.KZ<T>(z);
        const T k2 = kk2_at<T>(g, z, ky, kx);
        C2<T> A = a[q], B = b[q], Cc = c[q];
        C2<T> s = mk<T>(kx_ * A.x + ky_ * B.x + kz_ * Cc.x, kx_ * A.y + ky_ * B.y + kz_ * Cc.y);
        C2<T> D = mk<T>(s.y / k2, -s.x / k2);  // -i*s/kk2
        if (q == 0) D = mk<T>(0, 0);
        A = csub(A, cimk(kx_, D));
        B = csub(B, cimk(ky_, D));
        Cc = csub(Cc, cimk(kz_, D));
        a[q] = A; b[q] = B; c[q] = Cc; d[q] = D;
        const T tmp = (T)1 / (T)g.nz;
        C1[q] = cscale(bctarget ? Cc : D, tmp);
    SG_ELEMS_END
}

// a -= i kx C2, b -= i ky C2, c -= C3 (sol_project :385-399)
template <typename T>
__global__ void k_proj_sub(Geo g, C2<T> *a, C2<T> *b, C2<T> *c, const C2<T> *A2, const C2<T> *A3) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const C2<T> p = A2[q];
        a[q] = csub(a[q], cimk(g.KX<T>(kx), p));
        b[q] = csub(b[q], cimk(g.KY<T>(ky), p));
        c[q] = csub(c[q], A3[q]);
    SG_ELEMS_END
}

// d = d + C2 over all rows (sol_project bctarget=0, :359-368)
template <typename T>
__global__ void k_add(Geo g, C2<T> *d, const C2<T> *x) {
    SG_ELEMS_BEGIN(g, 0, g.nz) d[q] = cadd(d[q], x[q]); SG_ELEMS_END
}

// Wall values of the inverse z transform of one field: bc[2*col + w] for w = 0 (z index 0)
// and w = 1 (z index nzp-1), accumulated in FP64.  wtw[k] = exp(+2 pi i k (nzp-1)/nz).
template <typename T>
__global__ void k_wall_eval(Geo g, const C2<T> *in, double scale, const double2 *wtw, double2 *bc, int neg) {
    const int kx = blockIdx.x * blockDim.x + threadIdx.x, ky = blockIdx.y;
    if (kx >= g.nxh) return;
    double br = 0, bi = 0, tr = 0, ti = 0;
    for (int k = 0; k < g.nz; k++) {
        const C2<T> v = in[fidx<T>(g, k, ky, kx)];
        const double vr = (double)v.x * scale, vi = (double)v.y * scale;
        const double2 w = wtw[k];
        br += vr; bi += vi;
        tr += vr * w.x - vi * w.y;
        ti += vr * w.y + vi * w.x;
    }
    const int col = kx * g.ny + ky;
    const double s = neg ? -1.0 : 1.0;
    bc[2 * col] = make_double2(s * br, s * bi);
    bc[2 * col + 1] = make_double2(s * tr, s * ti);
}

// laplace_z coefficients (boundary_mod.fpp:481-549): mode 0 Dirichlet, 1 Neumann.  FP64.
static __global__ void k_laplace_coef(Geo g, const double2 *bc, double2 *coef, int mode) {
    const int kx = blockIdx.x * blockDim.x + threadIdx.x, ky = blockIdx.y;
    if (kx >= g.nxh) return;
    const int col = kx * g.ny + ky;
    const double2 b1 = bc[2 * col], b2 = bc[2 * col + 1];
    const double Lz = g.Lz;
    double2 c1, c2;
    if (kx == 0 && ky == 0) {
        if (mode == 0) { c1 = make_double2((b2.x - b1.x) / Lz, (b2.y - b1.y) / Lz); c2 = b1; }
        else { c1 = b1; c2 = make_double2(0.0, 0.0); }
    } else {
        const double kh = sqrt(g.kx[kx] * g.kx[kx] + g.ky[ky] * g.ky[ky]);
        const double e = exp(-(kh * Lz));
        const double tmp = mode == 0 ? 1.0 / (1 - exp(-(2 * kh * Lz))) : 1.0 / (kh * (1 - exp(-(2 * kh * Lz))));
        c1 = make_double2((b2.x - b1.x * e) * tmp, (b2.y - b1.y * e) * tmp);
        if (mode == 0) c2 = make_double2((b1.x - b2.x * e) * tmp, (b1.y - b2.y * e) * tmp);
        else c2 = make_double2((-b1.x + b2.x * e) * tmp, (-b1.y + b2.y * e) * tmp);
    }
    coef[2 * col] = c1;
    coef[2 * col + 1] = c2;
}

// laplace_z solution a and normal derivative b over all nz rows (boundary_mod.fpp:635-675)
template <typename T>
__global__ void k_laplace_profile(Geo g, const double2 *coef, C2<T> *A, C2<T> *B) {
    SG_ELEMS_BEGIN(g, 0, g.nz)
        const int col = kx * g.ny + ky;
        const double2 c1 = coef[2 * col], c2 = coef[2 * col + 1];
        const double zz = g.z[z];
        if (kx == 0 && ky == 0) {
            A[q] = mk<T>((T)(c1.x * zz + c2.x), (T)0);
            B[q] = mk<T>((T)c1.x, (T)0);
        } else {
            const double kh = sqrt(g.kx[kx] * g.kx[kx] + g.ky[ky] * g.ky[ky]);
            double e1, e2;
            if constexpr (sizeof(T) == 8) { e1 = exp(kh * (zz - g.Lz)); e2 = exp(-(kh * zz)); }
            else { e1 = (double)expf((float)(kh * (zz - g.Lz))); e2 = (double)expf((float)(-(kh * zz))); }
            A[q] = mk<T>((T)(c1.x * e1 + c2.x * e2), (T)(c1.y * e1 + c2.y * e2));
            B[q] = mk<T>((T)(kh * (c1.x * e1 - c2.x * e2)), (T)(kh * (c1.y * e1 - c2.y * e2)));
        }
    SG_ELEMS_END
}

// noslip_z at z index 0 and nzp-1 (vboundary.f90:154-211); vb = {vxsta, vysta, vxend, vyend}
struct WallVel { double x, y, z, w; };  // vxzsta, vyzsta, vxzend, vyzend

template <typename T>
__global__ void k_noslip(Geo g, C2<T> *vx, C2<T> *vy, const C2<T> *pr, double tmp, WallVel vb) {
    const int kx = blockIdx.x * blockDim.x + threadIdx.x, ky = blockIdx.y;
    if (kx >= g.nxh) return;
    for (int w = 0; w < 2; w++) {
        const int ind = w == 0 ? 0 : g.nzp - 1;
        const size_t q = fidx<T>(g, ind, ky, kx);
        const C2<T> p = pr[q];
        vx[q] = cscale(cimk(g.KX<T>(kx), p), (T)tmp);
        vy[q] = cscale(cimk(g.KY<T>(ky), p), (T)tmp);
        if (kx == 0 && ky == 0) {
            const double nn = (double)g.nx * g.ny;
            vx[q] = mk<T>((T)(nn * (w == 0 ? vb.x : vb.z)), (T)0);
            vy[q] = mk<T>((T)(nn * (w == 0 ? vb.y : vb.w)), (T)0);
        }
    }
}

// s_constant_z: theta = 0 at both walls (sboundary.f90:122-165)
template <typename T>
__global__ void k_zero_walls(Geo g, C2<T> *th) {
    const int kx = blockIdx.x * blockDim.x + threadIdx.x, ky = blockIdx.y;
    if (kx >= g.nxh) return;
    th[fidx<T>(g, 0, ky, kx)] = mk<T>(0, 0);
    th[fidx<T>(g, g.nzp - 1, ky, kx)] = mk<T>(0, 0);
}

// Deterministic FP64 reduction over the physical rows with weight 1 (kx=0) or 2 (kx>0):
// mode 0: sum_m |f_m|^2 for m < nf;  mode 1: sum_{m<nf/2} Re(f_m conj f_{m+nf/2}).
struct RedArgs {
    const void *f[6];
    int nf;
    int mode;
    int z1;  // rows [0, z1)
};

template <typename T>
__global__ void k_reduce(Geo g, RedArgs a, double *partial) {
    double acc = 0.0;
    SG_ELEMS_BEGIN(g, 0, a.z1)
        double s = 0.0;
        if (a.mode == 0) {
            for (int m = 0; m < a.nf; m++) {
                const C2<T> v = ((const C2<T> *)a.f[m])[q];
                s += (double)v.x * v.x + (double)v.y * v.y;
            }
        } else {
            const int h = a.nf / 2;
            for (int m = 0; m < h; m++) {
                const C2<T> u = ((const C2<T> *)a.f[m])[q], v = ((const C2<T> *)a.f[m + h])[q];
                s += (double)u.x * v.x + (double)u.y * v.y;
            }
        }
        acc += (kx == 0 ? 1.0 : 2.0) * s;
    SG_ELEMS_END
    __shared__ double red[kThreads];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// wall reduction for bouncheck_z: sum over columns of w(kx) * |bc|^2 for walls 0 and 1
static __global__ void k_reduce_walls(Geo g, const double2 *bcA, const double2 *bcB, double *partial) {
    double bot = 0.0, top = 0.0;
    const int ncol = g.nxh * g.ny;
    for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol; col += gridDim.x * blockDim.x) {
        const double w = (col / g.ny) == 0 ? 1.0 : 2.0;
        double2 a0 = bcA[2 * col], a1 = bcA[2 * col + 1];
        double r1 = a0.x * a0.x + a0.y * a0.y, r2 = a1.x * a1.x + a1.y * a1.y;
        if (bcB) {
            const double2 b0 = bcB[2 * col], b1 = bcB[2 * col + 1];
            r1 += b0.x * b0.x + b0.y * b0.y;
            r2 += b1.x * b1.x + b1.y * b1.y;
        }
        bot += w * r1;
        top += w * r2;
    }
    __shared__ double rb[kThreads], rt[kThreads];
    rb[threadIdx.x] = bot;
    rt[threadIdx.x] = top;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { rb[threadIdx.x] += rb[threadIdx.x + s]; rt[threadIdx.x] += rt[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = rb[0]; partial[2 * blockIdx.x + 1] = rt[0]; }
}

}  // namespace sg
