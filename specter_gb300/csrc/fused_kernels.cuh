// Fused RK-stage column kernels.
//
// After the nonlinear terms NL_c = (v.grad)v_c (and v.grad theta) have been brought back to
// the mixed (z, ky, kx) domain by the x/y passes, everything left in a stage acts on single
// (kx, ky) z-columns.  One block keeps a tile of TK columns resident in shared memory and runs,
// without touching HBM in between:
//   velocity:  NL forward z-transform with FC-Gram continuation, buoyancy, fc_filter, laplak and
//              the RK update (hd_rkstep2.f90:1-32 / bouss_rkstep2.f90:1-48), then
//              v_imposebc_and_project (vboundary.f90:67-151): z-inverse, no-slip wall planes
//              from the previous stage's pressure, z-forward with continuation, and sol_project
//              (boundary_mod.fpp:197-402): Poisson, wall values, laplace_z coefficients (FP64),
//              pressure, harmonic correction (from the per-column spectra of the two unit
//              profiles, computed once per plan in FP64: the correction is linear in c1, c2).
//   scalar:    NL forward, heat current, filter, update, s_imposebc (sboundary.f90:67-165),
//              fc_filter and the c2r -> /N -> r2c round trip (bouss_rkstep2.f90:56-59).  That
//              round trip is, exactly, z-inverse, 1/nz, Hermitian symmetrisation of the kx = 0
//              and kx = nx/2 columns over (ky, -ky) (what C2R then R2C does to them), and
//              z-forward with continuation; the symmetrisation pairs columns of different
//              ky, so those two kx columns finish in k_theta_herm.
#pragma once

#include "kernels.cuh"

namespace sg {

struct FusedArgs {
    const void *nl[4];    // NL_x, NL_y, NL_z, NL_theta: mixed domain, rows [0, nzp)
    const void *vin[4];   // stage input state (spectral): vx, vy, vz, theta
    const void *cold[4];  // RK step start C1, C2, C3, C7
    void *vout[4];        // stage output state
    void *pr;             // pressure potential (mixed), walls read, rows [0, nzp) written
    void *side;           // theta rows of the kx = 0 and kx = nx/2 columns: [2][ny][nzp]
    const void *hspec[2]; // E1, E2: z spectra (with continuation) of the unit laplace_z profiles
    void *work[3];        // split velocity form: the updated components between the two kernels
    double dt, nu, kappa, rmp, xmom, xtemp;
    double wall_tmp;      // 1/o, or (o+1)/o when o != ord (noslip_z)
    double vb[4];         // vxzsta, vyzsta, vxzend, vyzend
    double omega[3];      // rotation rate (rot != 0)
    int bouss;
    int rot;              // ROTBOUSS: Coriolis term, no final theta filter / round trip
    int nl32;             // the NL fields are FP32 (nl_fp32 form) while the kernel runs in FP64
    int nl_spec;          // (with nl32) the NL fields are already z spectra: rows [0, nz), the
                          // forward transform with continuation done by the FP32 pipeline
    FFT4Desc z32;         // nl_fp32 on the three-step float-float engine: the FP32 companion plan's
                          // four-step z tables, for the pressure potential's bulk rows (L1 = 0: none)
    float f_dt, f_nu, f_kappa, f_rmp, f_xmom, f_xtemp, f_wall_tmp, f_omega[3];  // FP32 mirrors
    ff q_dt, q_nu, q_kappa, q_rmp, q_xmom, q_xtemp, q_wall_tmp, q_omega[3];      // float-float
    FusedArgs prepared() const {
        FusedArgs b = *this;
        b.f_dt = (float)dt; b.f_nu = (float)nu; b.f_kappa = (float)kappa; b.f_rmp = (float)rmp;
        b.f_xmom = (float)xmom; b.f_xtemp = (float)xtemp; b.f_wall_tmp = (float)wall_tmp;
        for (int i = 0; i < 3; i++) b.f_omega[i] = (float)omega[i];
        b.q_dt = ff(dt); b.q_nu = ff(nu); b.q_kappa = ff(kappa); b.q_rmp = ff(rmp);
        b.q_xmom = ff(xmom); b.q_xtemp = ff(xtemp); b.q_wall_tmp = ff(wall_tmp);
        for (int i = 0; i < 3; i++) b.q_omega[i] = ff(omega[i]);
        return b;
    }
};

// Per-column laplace_z parameters in the kernel's precision: kh = |(kx, ky)| and the
// coefficients c1, c2 (solved in FP64, then rounded); k0 marks the (0, 0) column.
template <typename T>
struct LapCol {
    T kh;
    C2<T> c1, c2;
    int k0;
};

template <typename T> __device__ __forceinline__ T exp_t(T x);
template <> __device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }
// float-float kernels use exp only for the bulk rows of the pressure potential, an output that
// no later stage reads (its wall rows are set exactly); FP32 accuracy there
template <> __device__ __forceinline__ ff exp_t<ff>(ff x) { return ff(expf(x.hi)); }

// The same profile on the bulk rows, in the kernel's precision (they enter the z transform
// in that precision).
template <typename T>
__device__ __forceinline__ void lap_profile_t(const LapCol<T> &p, T zz, T Lz, C2<T> &a, C2<T> &b) {
    if (p.k0) {
        a = mk<T>(p.c1.x * zz + p.c2.x, (T)0);
        b = mk<T>(p.c1.x, (T)0);
        return;
    }
    const T e1 = exp_t<T>(p.kh * (zz - Lz)), e2 = exp_t<T>(-(p.kh * zz));
    a = mk<T>(p.c1.x * e1 + p.c2.x * e2, p.c1.y * e1 + p.c2.y * e2);
    b = mk<T>(p.kh * (p.c1.x * e1 - p.c2.x * e2), p.kh * (p.c1.y * e1 - p.c2.y * e2));
}

// Neumann laplace_z coefficients from the wall values (boundary_mod.fpp:521-549), FP64
__device__ __forceinline__ void lap_coef_neumann(const Geo &g, int kx, int ky, double2 b1, double2 b2,
                                                 double2 &c1, double2 &c2) {
    if (kx == 0 && ky == 0) {
        c1 = b1;
        c2 = make_double2(0.0, 0.0);
        return;
    }
    const double *lc = g.lapc + ((size_t)ky * g.nxh + kx) * 3;  // kh, exp(-kh Lz), 1/(kh (1 - exp(-2 kh Lz)))
    const double e = lc[1], tmp = lc[2];
    c1 = make_double2((b2.x - b1.x * e) * tmp, (b2.y - b1.y * e) * tmp);
    c2 = make_double2((-b1.x + b2.x * e) * tmp, (-b1.y + b2.y * e) * tmp);
}

template <typename T>
__device__ __forceinline__ double2 d2(C2<T> v) { return make_double2((double)v.x, (double)v.y); }

// Wall values of a column as running sums over its spectrum: s0 = sum_k v_k (bottom wall) and
// s1 = sum_k v_k w_k (top wall, w = Geo::wtw).  FP64 sums for the FP32 and FP64 kernels (four
// FP64 fused multiply-adds per point: the FP64 pipe bounds that loop), float-float sums for the
// float-float kernels.  Partials are reduced over a warp by shuffles and stored as two 16-byte
// slots per (warp, column).
template <typename T>
struct WallSum {
    static constexpr bool kFF = is_ff<T>;
    double2 d0, d1;
    ffc q0, q1;
    __device__ __forceinline__ WallSum() {
        d0 = d1 = make_double2(0.0, 0.0);
        q0.x = q0.y = q1.x = q1.y = ff(0);
    }
    __device__ __forceinline__ void add(const Geo &g, C2<T> v, int k) {
        if constexpr (kFF) {
            const ffc w = ldg_v((const ffc *)g.wtwq + k);
            q0.x += v.x;
            q0.y += v.y;
            q1.x += v.x * w.x - v.y * w.y;
            q1.y += v.x * w.y + v.y * w.x;
        } else {
            const double vr = (double)v.x, vi = (double)v.y;
            const double2 w = ((const double2 *)g.wtw)[k];
            d0.x += vr;
            d0.y += vi;
            d1.x = fma(vr, w.x, d1.x);
            d1.x = fma(-vi, w.y, d1.x);
            d1.y = fma(vr, w.y, d1.y);
            d1.y = fma(vi, w.x, d1.y);
        }
    }
    __device__ __forceinline__ static ff shfl(ff v, int off) {
        return ff(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
    }
    // sum over the lanes c, c + TK, ... of a warp
    __device__ __forceinline__ void warp_reduce(int TK) {
        for (int off = TK; off < 32; off <<= 1) {
            if constexpr (kFF) {
                q0.x += shfl(q0.x, off);
                q0.y += shfl(q0.y, off);
                q1.x += shfl(q1.x, off);
                q1.y += shfl(q1.y, off);
            } else {
                d0.x += __shfl_xor_sync(0xffffffffu, d0.x, off);
                d0.y += __shfl_xor_sync(0xffffffffu, d0.y, off);
                d1.x += __shfl_xor_sync(0xffffffffu, d1.x, off);
                d1.y += __shfl_xor_sync(0xffffffffu, d1.y, off);
            }
        }
    }
    __device__ __forceinline__ void store(double2 *slot) const {
        if constexpr (kFF) {
            ((ffc *)slot)[0] = q0;
            ((ffc *)slot)[1] = q1;
        } else {
            slot[0] = d0;
            slot[1] = d1;
        }
    }
    __device__ __forceinline__ void load_add(const double2 *slot) {
        if constexpr (kFF) {
            const ffc a = ((const ffc *)slot)[0], b = ((const ffc *)slot)[1];
            q0.x += a.x; q0.y += a.y; q1.x += b.x; q1.y += b.y;
        } else {
            d0.x += slot[0].x; d0.y += slot[0].y; d1.x += slot[1].x; d1.y += slot[1].y;
        }
    }
    __device__ __forceinline__ double2 bottom() const {
        if constexpr (kFF) return make_double2(ff_to_double(q0.x), ff_to_double(q0.y));
        else return d0;
    }
    __device__ __forceinline__ double2 top() const {
        if constexpr (kFF) return make_double2(ff_to_double(q1.x), ff_to_double(q1.y));
        else return d1;
    }
};

// Tile of NL_c (rows [0, rows), columns col0 + [0, TK)): by asynchronous copies when the NL field
// has the kernel's precision, else (FP32 NL fields in an FP64 kernel, the nl_fp32 form) by
// converting loads, complete for the calling thread on return.  Either way one copy group is
// committed, so the callers' async_wait_n counts hold.
template <typename T>
__device__ __forceinline__ void nl_tile_load(C2<T> *dst, const FusedArgs &a, int c, unsigned col0, unsigned zs, int rows,
                                             int TK, int nv) {
    if constexpr (!is_f32<T>) {
        if (a.nl32) {
            // eight loads per thread in flight before the converting stores (one at a time, each
            // waited for in turn, they left the SM idle for most of the load phase)
            const float2 *src = (const float2 *)a.nl[c] + col0;
            const int lgTK = lg2(TK), total = rows * TK;
            for (int base = threadIdx.x; base < total; base += 8 * blockDim.x) {
                float2 f[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int idx = base + u * blockDim.x;
                    const int k = idx >> lgTK, cc = idx & (TK - 1);
                    f[u] = make_float2(0.f, 0.f);
                    if (idx < total && cc < nv) f[u] = __ldg(src + ((unsigned)k * zs + (unsigned)cc));
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int idx = base + u * blockDim.x;
                    if (idx < total) dst[idx] = from_f2<T>(f[u]);
                }
            }
            async_commit();
            return;
        }
    }
    tile_load_async(dst, (const C2<T> *)a.nl[c] + col0, zs, rows, TK, nv);
}

// Rows of the NL tile to load: the mixed-domain physical rows, or every row of a spectrum.
__device__ __forceinline__ int nl_rows(const Geo &g, const FusedArgs &a) { return a.nl_spec ? g.nz : g.nzp; }

// NL forward z transform with FC-Gram continuation of the tile in X (rows [0, nzp) loaded); with
// a.nl_spec the tile already holds the spectrum in natural order (FP64 kernels only, whose
// generic engine keeps natural order: E::pos(k) = k).  Returns the buffer holding the spectrum.
template <typename T, class E>
__device__ __forceinline__ C2<T> *nl_forward(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, C2<T> *X,
                                             C2<T> *Y, int TK) {
    __syncthreads();
    if constexpr (!is_f32<T>) {
        if (a.nl_spec) return X;
    }
    fc_continuation<T>(g, X, TK);
    __syncthreads();
    return E::run(X, Y, TK, fd, -1);
}

// A wall round trip of the float-float kernels as a window correction (ffzoom.cuh): X holds the
// spectrum (rows [0, nz), natural); window row p is physical row (nzp - d + p) mod nz: p < d the
// top wall-adjacent rows (p = d - 1 the top wall), d <= p < d + C the continuation rows, the rest
// the bottom rows (p = d + C the bottom wall).  The window values of the inverse transform are
// scaled by 1/nz (goto_domain), the wall rows take wall(top, col) when `walls`, the continuation
// rows are rebuilt from the 2d wall-adjacent rows with the float-float sums of fc_continuation,
// and the forward transform of (new - old) is added to X.  X is the updated spectrum, visible to
// all threads, on return.  Scratch: rows [nz, nz + 576 + 2 kWin) of X (the engine's Desc.L).
template <typename T, class E, class Wall>
__device__ __forceinline__ void zoom_round_trip(const Geo &g, const typename E::Desc &fd, C2<T> *X, int TK, bool walls,
                                                Wall wall) {
    using V = C2<T>;
    const int nz = g.nz, d = g.oz, C = g.cz, lgTK = lg2(TK);
    V *W = X + (size_t)nz * TK, *Wv = W + (size_t)FFZTab::L * TK, *Dv = Wv + (size_t)FFZTab::kWin * TK;
    E::window(X, W, Wv, fd, TK);
    const T inz = (T)1 / (T)nz;
    for (int idx = threadIdx.x; idx < FFZTab::kWin * TK; idx += blockDim.x) {
        const int p = idx >> lgTK, c = idx & (TK - 1);
        const V u = cscale(Wv[idx], inz);
        if (walls && (p == d - 1 || p == d + C)) {
            const V w = wall(p == d - 1, c);
            Dv[idx] = csub(w, u);
            Wv[idx] = w;
        } else {
            Dv[idx] = mk<T>(0, 0);
            Wv[idx] = u;
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < C * TK; idx += blockDim.x) {
        const int ii = idx >> lgTK, c = idx & (TK - 1);
        T ar = (T)0, ai = (T)0;
        for (int jj = 0; jj < d; jj++) {
            const V t = Wv[jj * TK + c], b = Wv[(C + 2 * d - 1 - jj) * TK + c];
            const float2 q0 = __ldg((const float2 *)(g.dirq + ii + C * jj));
            const float2 q1 = __ldg((const float2 *)(g.dirq + (C - 1 - ii) + C * jj));
            const T w0 = T(q0.x, q0.y), w1 = T(q1.x, q1.y);
            ar = ar + w0 * t.x + w1 * b.x;
            ai = ai + w0 * t.y + w1 * b.y;
        }
        const int p = d + ii;
        Dv[p * TK + c] = csub(mk<T>(ar, ai), Wv[p * TK + c]);
    }
    __syncthreads();
    E::window_add(X, W, Dv, fd, TK);
}

// ----------------------------------------------------------------------------------------------
// velocity: device functions shared by the one-block-per-tile kernel (k_fused_velocity) and the
// split pair (k_fused_vcomp per component, k_fused_vproj for the projection)
// ----------------------------------------------------------------------------------------------
struct ColTile {
    int kx0, ky, nv, TK, lgTK;
    unsigned zs, col0;  // z stride of a column and the tile's first column offset
};

// bid: the block's index (blockIdx, or its instance-local index in a batched launch)
template <typename T>
__device__ __forceinline__ ColTile col_tile(const Geo &g, int TK, const uint3 &bid) {
    ColTile t;
    t.TK = TK;
    t.lgTK = lg2(TK);
    t.kx0 = bid.x * TK;
    t.ky = bid.y;
    t.nv = min(TK, g.nxh - t.kx0);
    t.zs = (unsigned)g.ny * g.ldx;
    t.col0 = (unsigned)t.ky * g.ldx + t.kx0;
    return t;
}

// Component c3 of the velocity update.  On entry X rows [0, nzp) hold NL_c3 (loads complete
// for the calling thread) and, when buoy, a copy of theta's tile is in flight into Uc.  Forward
// z transform with continuation, + 2 Om x v (ROTBOUSS), - xmom theta (buoy), fc_filter, then
// Uc = cold + dt (nu lap(vin) - n) / o  (hd_rkstep2.f90:1-32, bouss_rkstep2.f90:1-48).
// to_x: leave the updated component in the FFT buffer X (natural rows) instead of Uc, for a
// caller that transforms it next (vel_walls with in_x)
template <typename T, class E>
__device__ void vel_update(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, const ColTile &t, int c3,
                           C2<T> *Uc, C2<T> *X, C2<T> *Y, bool buoy, bool to_x = false) {
    using V = C2<T>;
    const int nz = g.nz, TK = t.TK, lgTK = t.lgTK, kx0 = t.kx0, ky = t.ky, nv = t.nv;
    const int tile = nz * TK;
    const bool stage2 = (size_t)E::kBuffers * fd.L >= 2 * (size_t)nz;  // vin and cold both fit in X
    const T dt = pick<T>(a.dt, a.f_dt, a.q_dt), nu = pick<T>(a.nu, a.f_nu, a.q_nu), rmp = pick<T>(a.rmp, a.f_rmp, a.q_rmp);
    const T xmom = pick<T>(a.xmom, a.f_xmom, a.q_xmom);
    V *R = nl_forward<T, E>(g, fd, a, X, Y, TK);
    if (buoy) {
        async_wait();
        __syncthreads();
    }
    // (a) filtered nonlinear term (+ 2 Om x v, minus buoyancy) -> Uc
    const V *va = (const V *)a.vin[(c3 + 1) % 3], *vb = (const V *)a.vin[(c3 + 2) % 3];
    const T oa = pick<T>(a.omega[(c3 + 1) % 3], a.f_omega[(c3 + 1) % 3], a.q_omega[(c3 + 1) % 3]);
    const T ob = pick<T>(a.omega[(c3 + 2) % 3], a.f_omega[(c3 + 2) % 3], a.q_omega[(c3 + 2) % 3]);
    for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        V n = mk<T>(0, 0);
        if (c < nv) {
            const int kx = kx0 + c;
            n = R[E::pos(k, fd) * TK + c];
            if (a.rot) {
                // component c3 of 2 Om x v = 2 (Om_a v_b - Om_b v_a), (c3, a, b) cyclic
                const unsigned q = fidx<T>(g, k, ky, kx);
                const V pa = va[q], pb = vb[q];
                n = mk<T>(n.x + (T)2 * (oa * pb.x - ob * pa.x), n.y + (T)2 * (oa * pb.y - ob * pa.y));
            }
            if (buoy) { const V th = Uc[idx]; n = mk<T>(n.x - xmom * th.x, n.y - xmom * th.y); }
            n = cscale(n, g.FX<T>(kx));
            n = cscale(n, g.FY<T>(ky));
            n = cscale(n, g.FZ<T>(k));
        }
        Uc[idx] = n;
    }
    __syncthreads();
    // (b) RK update with laplak of the stage input; vin (and cold) staged in the FFT buffer
    const V *cold = (const V *)a.cold[c3];
    tile_load_async(X, (const V *)a.vin[c3] + t.col0, t.zs, nz, TK, nv);
    if (stage2) tile_load_async(X + tile, cold + t.col0, t.zs, nz, TK, nv);
    async_wait();
    __syncthreads();
    V *dst = to_x ? X : Uc;  // X[idx]: each thread reads its own element first
    for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        if (c >= nv) { dst[idx] = mk<T>(0, 0); continue; }
        const int kx = kx0 + c;
        const T k2 = g.KX<T>(kx) * g.KX<T>(kx) + g.KY<T>(ky) * g.KY<T>(ky) + g.KZ<T>(k) * g.KZ<T>(k);
        const V v = X[idx], cv = stage2 ? X[tile + idx] : cold[fidx<T>(g, k, ky, kx)];
        const V n = Uc[idx];
        const V lap = cscale(v, -k2);
        dst[idx] = mk<T>(cv.x + dt * (nu * lap.x - n.x) * rmp, cv.y + dt * (nu * lap.y - n.y) * rmp);
    }
    __syncthreads();
}

// The RK update of one component in the float-float kernels with window tables, without a staging
// buffer: the stage input and the step start are in X and X + tile; the FP32 nonlinear spectrum
// nl and the field ex of the linear coupling (theta for vz's buoyancy, vz for theta's heat
// current; coefficient cx) are read from global memory, four elements per thread in flight:
//   n = fc_filter(nl [+ 2 Om x v] - cx ex),  X = cold + dt (diff lap(X) - n) rmp,
// the operations and their order those of vel_update and the scalar kernel.  rot_c3 >= 0 adds the
// Coriolis term of that velocity component.
template <typename T>
__device__ void update_direct(const Geo &g, const FusedArgs &a, const ColTile &t, C2<T> *X, const float2 *nl,
                              const C2<T> *ex, T cx, T diff, int rot_c3) {
    using V = C2<T>;
    constexpr int kB = 4;
    const int nz = g.nz, TK = t.TK, lgTK = t.lgTK, kx0 = t.kx0, ky = t.ky, nv = t.nv;
    const int tile = nz * TK, total = nz * TK;
    const T dt = pick<T>(a.dt, a.f_dt, a.q_dt), rmp = pick<T>(a.rmp, a.f_rmp, a.q_rmp);
    const float2 *nlc = nl + t.col0;
    const V *exc = ex ? ex + t.col0 : nullptr;
    for (int base = threadIdx.x; base < total; base += kB * blockDim.x) {
        float2 f[kB];
        V e[kB];
#pragma unroll
        for (int u = 0; u < kB; u++) {
            const int idx = base + u * blockDim.x;
            const int k = idx >> lgTK, c = idx & (TK - 1);
            const bool in = idx < total && c < nv;
            const unsigned q = (unsigned)k * t.zs + (unsigned)c;
            f[u] = in ? __ldg(nlc + q) : make_float2(0.f, 0.f);
            e[u] = (in && exc) ? exc[q] : mk<T>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < kB; u++) {
            const int idx = base + u * blockDim.x;
            if (idx >= total) continue;
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) { X[idx] = mk<T>(0, 0); continue; }
            const int kx = kx0 + c;
            V n = from_f2<T>(f[u]);
            if (rot_c3 >= 0) {  // component rot_c3 of 2 Om x v = 2 (Om_a v_b - Om_b v_a), (c3, a, b) cyclic
                const int ia = (rot_c3 + 1) % 3, ib = (rot_c3 + 2) % 3;
                const T oa = pick<T>(a.omega[ia], a.f_omega[ia], a.q_omega[ia]), ob = pick<T>(a.omega[ib], a.f_omega[ib], a.q_omega[ib]);
                const unsigned q = fidx<T>(g, k, ky, kx);
                const V pa = ((const V *)a.vin[ia])[q], pb = ((const V *)a.vin[ib])[q];
                n = mk<T>(n.x + (T)2 * (oa * pb.x - ob * pa.x), n.y + (T)2 * (oa * pb.y - ob * pa.y));
            }
            if (exc) n = mk<T>(n.x - cx * e[u].x, n.y - cx * e[u].y);
            n = cscale(n, g.FX<T>(kx));
            n = cscale(n, g.FY<T>(ky));
            n = cscale(n, g.FZ<T>(k));
            const T k2 = g.KX<T>(kx) * g.KX<T>(kx) + g.KY<T>(ky) * g.KY<T>(ky) + g.KZ<T>(k) * g.KZ<T>(k);
            const V v = X[idx], cv = X[tile + idx];
            const V lap = cscale(v, -k2);
            X[idx] = mk<T>(cv.x + dt * (diff * lap.x - n.x) * rmp, cv.y + dt * (diff * lap.y - n.y) * rmp);
        }
    }
    __syncthreads();
}

// goto_domain_w_boundaries, noslip_z, goto_3d_fourier for component c3 in {0, 1}
// (boundary_mod.fpp:72-194, vboundary.f90:154-211): z-inverse, 1/nz on the physical rows, wall
// rows from the previous stage's pressure, continuation and z-forward; Uc in and out.
// in_x: the component is already in X (vel_update with to_x); wout: store the result to this
// global field instead of Uc.  With a single in-place FFT buffer in natural order (the
// Bluestein four-step engine) the physical rows are finished in X itself.
template <typename T, class E>
__device__ void vel_walls(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, const ColTile &t, int c3,
                          C2<T> *Uc, C2<T> *X, C2<T> *Y, bool in_x = false, C2<T> *wout = nullptr) {
    using V = C2<T>;
    const int nz = g.nz, nzp = g.nzp, TK = t.TK, lgTK = t.lgTK, kx0 = t.kx0, ky = t.ky, nv = t.nv;
    const V *pr = (const V *)a.pr;
    const T wall_tmp = pick<T>(a.wall_tmp, a.f_wall_tmp, a.q_wall_tmp), inz = (T)1 / (T)nz;
    if constexpr (E::kZoom) {
        if (fd.ztab) {
            if (!in_x) {
                for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) X[idx] = Uc[idx];
                __syncthreads();
            }
            // no-slip wall rows from the previous stage's pressure (noslip_z), as below
            auto wall = [&](bool top, int c) -> V {
                if (c >= nv) return mk<T>(0, 0);
                const int kx = kx0 + c, k = top ? nzp - 1 : 0;
                if (kx == 0 && ky == 0) return mk<T>((T)((double)g.nx * g.ny * a.vb[(top ? 2 : 0) + c3]), (T)0);
                const V p = pr[fidx<T>(g, k, ky, kx)];
                return cscale(cimk(c3 == 0 ? g.KX<T>(kx) : g.KY<T>(ky), p), wall_tmp);
            };
            zoom_round_trip<T, E>(g, fd, X, TK, true, wall);
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                const int k = idx >> lgTK, c = idx & (TK - 1);
                if (wout) {
                    if (c < nv) wout[fidx<T>(g, k, ky, kx0 + c)] = X[idx];
                } else {
                    Uc[idx] = X[idx];
                }
            }
            if (!wout) __syncthreads();
            return;
        }
    }
    if (!in_x) {
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) X[idx] = Uc[idx];
        __syncthreads();
    }
    V *R = E::run(X, Y, TK, fd, +1);
    const bool inplace = R == X && fd.blue;  // natural order in X
    V *P = inplace ? X : Uc;                 // physical rows, natural order
    for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        V v = cscale(R[E::pos(k, fd) * TK + c], inz);
        if ((k == 0 || k == nzp - 1) && c < nv) {
            const int kx = kx0 + c;
            const V p = pr[fidx<T>(g, k, ky, kx)];
            v = cscale(cimk(c3 == 0 ? g.KX<T>(kx) : g.KY<T>(ky), p), wall_tmp);
            if (kx == 0 && ky == 0) v = mk<T>((T)((double)g.nx * g.ny * a.vb[(k == 0 ? 0 : 2) + c3]), (T)0);
        }
        P[idx] = v;
    }
    __syncthreads();
    if (!inplace) {
        for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) X[idx] = Uc[idx];
        __syncthreads();
    }
    fc_continuation<T>(g, X, TK);
    __syncthreads();
    R = E::run(X, Y, TK, fd, -1);
    if (wout) {
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c < nv) wout[fidx<T>(g, k, ky, kx0 + c)] = R[E::pos(k, fd) * TK + c];
        }
        return;
    }
    for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        Uc[idx] = R[E::pos(k, fd) * TK + c];
    }
    __syncthreads();
}

// sol_project on the three updated components held in U (boundary_mod.fpp:197-448, 451-678):
// Poisson, FP64 wall values of vz / nz and laplace_z coefficients, pressure IFFT(d)/nz + a(z),
// harmonic correction from the precomputed unit-profile spectra, store of the new velocity.
// red: [blockDim][2] double2, coef: [TK][2] double2 followed by TK LapCol<T>.
template <typename T, class E>
__device__ void vel_project(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, const ColTile &t,
                            C2<T> *U, C2<T> *X, C2<T> *Y, double2 *red, double2 *coef) {
    using V = C2<T>;
    const int nz = g.nz, nzp = g.nzp, TK = t.TK, lgTK = t.lgTK, kx0 = t.kx0, ky = t.ky, nv = t.nv;
    const int tile = nz * TK;
    const bool stage2 = (size_t)E::kBuffers * fd.L >= 2 * (size_t)nz;
    LapCol<T> *lcol = (LapCol<T> *)(coef + 2 * TK);
    // ---- Poisson: d -> X (natural), v -= i k d, wall sums of vz (FP64)
    {
        const int c = threadIdx.x & (TK - 1), k0 = threadIdx.x >> lgTK, kstep = blockDim.x >> lgTK;
        const int kxc = min(kx0 + c, g.nxh - 1);
        const T kx_ = g.KX<T>(kxc), ky_ = g.KY<T>(ky);
        WallSum<T> ws;
        if (threadIdx.x < kstep * TK) {
            for (int k = k0; k < nz; k += kstep) {
                const int idx = k * TK + c;
                const T kz_ = g.KZ<T>(k);
                const T k2 = kx_ * kx_ + ky_ * ky_ + kz_ * kz_;
                V A = U[idx], B = U[tile + idx], Cc = U[2 * tile + idx];
                const V s = mk<T>(kx_ * A.x + ky_ * B.x + kz_ * Cc.x, kx_ * A.y + ky_ * B.y + kz_ * Cc.y);
                V D;
                if constexpr (!is_f64<T>) {  // FP32 and float-float: one reciprocal per point
                    const T ik2 = (T)1 / k2;
                    D = mk<T>(s.y * ik2, -s.x * ik2);
                } else {
                    D = mk<T>(s.y / k2, -s.x / k2);
                }
                if (k == 0 && ky == 0 && kx0 + c == 0) D = mk<T>(0, 0);
                A = csub(A, cimk(kx_, D));
                B = csub(B, cimk(ky_, D));
                Cc = csub(Cc, cimk(kz_, D));
                U[idx] = A; U[tile + idx] = B; U[2 * tile + idx] = Cc;
                X[idx] = D;
                ws.add(g, Cc, k);
            }
        }
        // sum over the threads of a column: shuffles within each warp (the lanes of column c are
        // c, c + TK, ...), then one partial per warp
        ws.warp_reduce(TK);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane < TK) ws.store(red + 2 * (warp * TK + lane));
    }
    __syncthreads();
    if (threadIdx.x < TK) {
        const int c = threadIdx.x, nwarps = blockDim.x >> 5;
        WallSum<T> tot;
        for (int q = 0; q < nwarps; q++) tot.load_add(red + 2 * (q * TK + c));
        double2 b1 = tot.bottom(), b2 = tot.top();
        const double inz = 1.0 / nz;  // wall values of vz / nz
        b1.x *= inz; b1.y *= inz; b2.x *= inz; b2.y *= inz;
        const int kxc = min(kx0 + c, g.nxh - 1);
        double2 c1, c2;
        lap_coef_neumann(g, kxc, ky, b1, b2, c1, c2);
        coef[2 * c] = c1;
        coef[2 * c + 1] = c2;
        LapCol<T> lc;
        lc.kh = (T)g.lapc[((size_t)ky * g.nxh + kxc) * 3];
        lc.c1 = mk<T>((T)c1.x, (T)c1.y);
        lc.c2 = mk<T>((T)c2.x, (T)c2.y);
        lc.k0 = kxc == 0 && ky == 0;
        lcol[c] = lc;
    }
    __syncthreads();
    // ---- pressure: pr = IFFT_z(d)/nz + a(z) on the physical rows
    {
        V *R = E::run(X, Y, TK, fd, +1);
        V *prw = (V *)a.pr;
        const T inz = (T)1 / (T)nz, Lz = (T)g.Lz;
        for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) continue;
            V pa, pb;
            lap_profile_t<T>(lcol[c], g.ZZ<T>(k), Lz, pa, pb);
            if constexpr (is_ff<T>) {
                // the wall rows feed the next stage's no-slip planes: exact profile values there
                // (p1 = exp(-kh Lz), p2 = 1 at z = 0; p1 = 1, p2 = exp(-kh Lz) at z = Lz)
                const LapCol<T> &p = lcol[c];
                if ((k == 0 || k == nzp - 1) && !p.k0) {
                    const ff e(g.lapc[((size_t)ky * g.nxh + min(kx0 + c, g.nxh - 1)) * 3 + 1]);
                    pa = k == 0 ? mk<T>(p.c1.x * e + p.c2.x, p.c1.y * e + p.c2.y)
                                : mk<T>(p.c1.x + p.c2.x * e, p.c1.y + p.c2.y * e);
                }
            }
            const V dv = R[E::pos(k, fd) * TK + c];
            prw[fidx<T>(g, k, ky, kx0 + c)] = mk<T>(dv.x * inz + pa.x, dv.y * inz + pa.y);
        }
        __syncthreads();
    }
    // ---- harmonic correction: the spectra of a = c1 p1 + c2 p2 and b = da/dz are
    //      c1 E1 + c2 E2 and kh (c1 E1 - c2 E2) (for kx = ky = 0: c1 E1 + c2 E2 and c1 E2,
    //      real parts of c1, c2), E1, E2 precomputed per column
    {
        const V *E1 = (const V *)a.hspec[0], *E2 = (const V *)a.hspec[1];
        tile_load_async(X, E1 + t.col0, t.zs, nz, TK, nv);
        if (stage2) tile_load_async(X + tile, E2 + t.col0, t.zs, nz, TK, nv);
        async_wait();
        __syncthreads();
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) continue;
            const LapCol<T> lc = lcol[c];
            const V e1 = X[idx], e2 = stage2 ? X[tile + idx] : E2[fidx<T>(g, k, ky, kx0 + c)];
            V A, B;
            if (lc.k0) {
                A = mk<T>(lc.c1.x * e1.x + lc.c2.x * e2.x, lc.c1.x * e1.y + lc.c2.x * e2.y);
                B = cscale(e2, lc.c1.x);
            } else {
                const V t1 = cmul(lc.c1, e1), t2 = cmul(lc.c2, e2);
                A = cadd(t1, t2);
                B = cscale(csub(t1, t2), lc.kh);
            }
            const int kx = kx0 + c;
            U[idx] = csub(U[idx], cimk(g.KX<T>(kx), A));
            U[tile + idx] = csub(U[tile + idx], cimk(g.KY<T>(ky), A));
            U[2 * tile + idx] = csub(U[2 * tile + idx], B);
        }
        __syncthreads();
    }
    // ---- store the new velocity
    for (int c3 = 0; c3 < 3; c3++) {
        V *vout = (V *)a.vout[c3];
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c < nv) vout[fidx<T>(g, k, ky, kx0 + c)] = U[c3 * tile + idx];
        }
    }
}

// The pressure potential's bulk rows through the FP32 four-step engine of the companion plan:
// pr is an output no later stage reads except at its two wall rows, which come from float-float
// sums over the spectrum (exact like the transform's).  The bulk rows then carry FP32 rounding,
// as their FP32 exponential profile already does.  L1 x L2: the compiled FP32 z splits of the
// lengths this engine serves (1080 = 36 x 30 for nz + C = 538, 576 = 24 x 24 for 282).
template <int L1, int L2>
__device__ __forceinline__ void pressure_fp32(float2 *X32, int TK, const FFT4Desc &d) {
    FourStep<float, L1, L2, true>::run(X32, nullptr, TK, d, +1);
}
__device__ __forceinline__ bool pressure_fp32_ok(const FFT4Desc &d) {
    return d.blue && ((d.L1 == 36 && d.L2 == 30) || (d.L1 == 24 && d.L2 == 24));
}

// sol_project for engines with one in-place FFT buffer (E::kStreamProj: the float-float engine),
// without staging the three components: the Poisson pass reads them from the work fields and keeps
// the potential d (natural rows, Dsv) beside the FFT buffer; after the pressure transform and the
// harmonic coefficients the final pass reads the components again (L2: the same tile was read
// moments before) and forms v - i k d - (harmonic correction) in the same order of operations as
// vel_project.  Shared memory: X[L][TK] + Dsv[nz][TK] + per-warp wall sums (of vz and, for the
// FP32 pressure transform, of d), which at a tile width of 8 fits where vel_project's three
// staged components fit only 4.
template <typename T, class E>
__device__ void vel_project_streamed(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, const ColTile &t,
                                     C2<T> *X, C2<T> *Dsv, double2 *red, double2 *coef) {
    using V = C2<T>;
    const int nz = g.nz, nzp = g.nzp, TK = t.TK, lgTK = t.lgTK, kx0 = t.kx0, ky = t.ky, nv = t.nv;
    const int tile = nz * TK;
    const V *w0 = (const V *)a.work[0], *w1 = (const V *)a.work[1], *w2 = (const V *)a.work[2];
    const int nwarps = blockDim.x >> 5;
    double2 *redd = red + 2 * nwarps * TK;                // wall sums of d
    V *prw_wall = (V *)(coef + 2 * TK);                  // [TK][2]: the two wall rows of IFFT(d)
    LapCol<T> *lcol = (LapCol<T> *)(prw_wall + 2 * TK);
    const bool p32 = pressure_fp32_ok(a.z32);
    float2 *X32 = (float2 *)X;
    // ---- Poisson: d -> X (or its FP32 rounding -> X32) and Dsv (natural), wall sums of
    //      vz - i kz d (and of d)
    {
        const int c = threadIdx.x & (TK - 1), k0 = threadIdx.x >> lgTK, kstep = blockDim.x >> lgTK;
        const int kxc = min(kx0 + c, g.nxh - 1);
        const T kx_ = g.KX<T>(kxc), ky_ = g.KY<T>(ky);
        WallSum<T> ws, wsd;
        if (threadIdx.x < kstep * TK) {
            // the components of two rows requested before either is used (the loop is bound by
            // the latency of these loads)
            V nA = mk<T>(0, 0), nB = mk<T>(0, 0), nC = mk<T>(0, 0);
            if (c < nv && k0 < nz) {
                const unsigned q = fidx<T>(g, k0, ky, kx0 + c);
                nA = ldg_v(w0 + q);
                nB = ldg_v(w1 + q);
                nC = ldg_v(w2 + q);
            }
            for (int k = k0; k < nz; k += kstep) {
                const int idx = k * TK + c;
                V A = nA, B = nB, Cc = nC;
                if (c < nv && k + kstep < nz) {
                    const unsigned q = fidx<T>(g, k + kstep, ky, kx0 + c);
                    nA = ldg_v(w0 + q);
                    nB = ldg_v(w1 + q);
                    nC = ldg_v(w2 + q);
                }
                const T kz_ = g.KZ<T>(k);
                const T k2 = kx_ * kx_ + ky_ * ky_ + kz_ * kz_;
                const V s = mk<T>(kx_ * A.x + ky_ * B.x + kz_ * Cc.x, kx_ * A.y + ky_ * B.y + kz_ * Cc.y);
                const T ik2 = (T)1 / k2;
                V D = mk<T>(s.y * ik2, -s.x * ik2);
                if (k == 0 && ky == 0 && kx0 + c == 0) D = mk<T>(0, 0);
                Cc = csub(Cc, cimk(kz_, D));
                if (p32) {
                    if constexpr (is_ff<T>) X32[idx] = make_float2(D.x.hi + D.x.lo, D.y.hi + D.y.lo);
                    wsd.add(g, D, k);
                } else {
                    X[idx] = D;
                }
                Dsv[idx] = D;
                ws.add(g, Cc, k);
            }
        }
        ws.warp_reduce(TK);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane < TK) ws.store(red + 2 * (warp * TK + lane));
        if (p32) {
            wsd.warp_reduce(TK);
            if (lane < TK) wsd.store(redd + 2 * (warp * TK + lane));
        }
    }
    __syncthreads();
    if (threadIdx.x < TK) {
        const int c = threadIdx.x;
        WallSum<T> tot;
        for (int q = 0; q < nwarps; q++) tot.load_add(red + 2 * (q * TK + c));
        if constexpr (is_ff<T>) {
            if (p32) {
                WallSum<T> td;
                for (int q = 0; q < nwarps; q++) td.load_add(redd + 2 * (q * TK + c));
                prw_wall[2 * c] = td.q0;
                prw_wall[2 * c + 1] = td.q1;
            }
        }
        double2 b1 = tot.bottom(), b2 = tot.top();
        const double inz = 1.0 / nz;
        b1.x *= inz; b1.y *= inz; b2.x *= inz; b2.y *= inz;
        const int kxc = min(kx0 + c, g.nxh - 1);
        double2 c1, c2;
        lap_coef_neumann(g, kxc, ky, b1, b2, c1, c2);
        coef[2 * c] = c1;
        coef[2 * c + 1] = c2;
        LapCol<T> lc;
        lc.kh = (T)g.lapc[((size_t)ky * g.nxh + kxc) * 3];
        lc.c1 = mk<T>((T)c1.x, (T)c1.y);
        lc.c2 = mk<T>((T)c2.x, (T)c2.y);
        lc.k0 = kxc == 0 && ky == 0;
        lcol[c] = lc;
    }
    __syncthreads();
    // ---- pressure: pr = IFFT_z(d)/nz + a(z) on the physical rows
    {
        V *R = X;
        if (p32) {
            if (a.z32.L1 == 36) pressure_fp32<36, 30>(X32, TK, a.z32);
            else pressure_fp32<24, 24>(X32, TK, a.z32);
        } else {
            R = E::run(X, nullptr, TK, fd, +1);
        }
        V *prw = (V *)a.pr;
        const T inz = (T)1 / (T)nz, Lz = (T)g.Lz;
        for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) continue;
            V pa, pb;
            lap_profile_t<T>(lcol[c], g.ZZ<T>(k), Lz, pa, pb);
            if constexpr (is_ff<T>) {
                const LapCol<T> &p = lcol[c];
                if ((k == 0 || k == nzp - 1) && !p.k0) {
                    const ff e(g.lapc[((size_t)ky * g.nxh + min(kx0 + c, g.nxh - 1)) * 3 + 1]);
                    pa = k == 0 ? mk<T>(p.c1.x * e + p.c2.x, p.c1.y * e + p.c2.y)
                                : mk<T>(p.c1.x + p.c2.x * e, p.c1.y + p.c2.y * e);
                }
            }
            V dv;
            if (p32) {
                if (k == 0 || k == nzp - 1) dv = prw_wall[2 * c + (k == 0 ? 0 : 1)];
                else dv = from_f2<T>(X32[k * TK + c]);
            } else {
                dv = R[E::pos(k, fd) * TK + c];
            }
            prw[fidx<T>(g, k, ky, kx0 + c)] = mk<T>(dv.x * inz + pa.x, dv.y * inz + pa.y);
        }
        __syncthreads();
    }
    // ---- v - i k d, then the harmonic correction (as in vel_project), stored
    {
        const V *E1 = (const V *)a.hspec[0], *E2 = (const V *)a.hspec[1];
        tile_load_async(X, E1 + t.col0, t.zs, nz, TK, nv);
        tile_load_async(X + tile, E2 + t.col0, t.zs, nz, TK, nv);
        V *o0 = (V *)a.vout[0], *o1 = (V *)a.vout[1], *o2 = (V *)a.vout[2];
        const T ky_ = g.KY<T>(ky);
        // the components of the next element requested before this one is used (L2 hits: the
        // Poisson pass read them moments before); the first while the spectra tiles arrive
        auto comp = [&](int idx, V &A, V &B, V &Cc) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            A = B = Cc = mk<T>(0, 0);
            if (idx < nz * TK && c < nv) {
                const unsigned q = fidx<T>(g, k, ky, kx0 + c);
                A = ldg_v(w0 + q);
                B = ldg_v(w1 + q);
                Cc = ldg_v(w2 + q);
            }
        };
        V nA, nB, nC;
        comp(threadIdx.x, nA, nB, nC);
        async_wait();
        __syncthreads();
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            V A = nA, B = nB, Cc = nC;
            comp(idx + blockDim.x, nA, nB, nC);
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) continue;
            const int kx = kx0 + c;
            const unsigned q = fidx<T>(g, k, ky, kx);
            const V D = Dsv[idx];
            const T kx_ = g.KX<T>(kx), kz_ = g.KZ<T>(k);
            A = csub(A, cimk(kx_, D));
            B = csub(B, cimk(ky_, D));
            Cc = csub(Cc, cimk(kz_, D));
            const LapCol<T> lc = lcol[c];
            const V e1 = X[idx], e2 = X[tile + idx];
            V Ah, Bh;
            if (lc.k0) {
                Ah = mk<T>(lc.c1.x * e1.x + lc.c2.x * e2.x, lc.c1.x * e1.y + lc.c2.x * e2.y);
                Bh = cscale(e2, lc.c1.x);
            } else {
                const V t1 = cmul(lc.c1, e1), t2 = cmul(lc.c2, e2);
                Ah = cadd(t1, t2);
                Bh = cscale(csub(t1, t2), lc.kh);
            }
            o0[q] = csub(A, cimk(kx_, Ah));
            o1[q] = csub(B, cimk(ky_, Ah));
            o2[q] = csub(Cc, Bh);
        }
    }
}

// One block per column tile for the whole velocity stage: smem = U[3][nz][TK] + FFT buffer(s)
// + small FP64 scratch.  NL_{c+1} (or theta, for the buoyancy of c = z) is copied into the still
// unused slot U[c+1] while component c is transformed.
template <typename T, class E>
__global__ void __launch_bounds__(E::kWideThreads, 1) k_fused_velocity(Geo g, typename E::Desc fd, FusedArgs a, int TK) {
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = g.nz, L = fd.L;
    const ColTile t = col_tile<T>(g, TK, blockIdx);
    const int tile = nz * TK;
    V *U = (V *)smem_raw;                       // 3 components, natural rows
    V *X = U + 3 * tile;                        // FFT work
    V *Y = X + (size_t)L * TK;
    double2 *red = (double2 *)(X + (size_t)E::kBuffers * L * TK);  // [blockDim][2] partial wall sums
    double2 *coef = red + 2 * blockDim.x;                           // [TK][2] + LapCol[TK]
    for (int c3 = 0; c3 < 3; c3++) {
        V *Uc = U + c3 * tile;
        const bool buoy = c3 == 2 && a.bouss;
        if (c3 == 0) {
            nl_tile_load<T>(X, a, 0, t.col0, t.zs, nl_rows(g, a), TK, t.nv);
            nl_tile_load<T>(U + tile, a, 1, t.col0, t.zs, nl_rows(g, a), TK, t.nv);
            async_wait_n<1>();
        } else {
            async_wait();
            __syncthreads();
            for (int idx = threadIdx.x; idx < nl_rows(g, a) * TK; idx += blockDim.x) X[idx] = Uc[idx];
            __syncthreads();
            if (c3 == 1) nl_tile_load<T>(U + 2 * tile, a, 2, t.col0, t.zs, nl_rows(g, a), TK, t.nv);
            else if (buoy) tile_load_async(Uc, (const V *)a.vin[3] + t.col0, t.zs, nz, TK, t.nv);
        }
        vel_update<T, E>(g, fd, a, t, c3, Uc, X, Y, buoy);
    }
    for (int c3 = 0; c3 < 2; c3++) vel_walls<T, E>(g, fd, a, t, c3, U + c3 * tile, X, Y);
    vel_project<T, E>(g, fd, a, t, U, X, Y, red, coef);
}

// Split form, part 1: one block per (column tile, component): the component's update and, for
// vx and vy, the wall round trip; the result goes to W[c] (a stage buffer).  smem = Uc[nz][TK] +
// FFT buffer(s): half the footprint of k_fused_velocity, so two blocks share an SM.
template <typename T, class E, int CTK>
__device__ __forceinline__ void fused_vcomp_body(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, int TKrt, uint3 blockIdx) {
    const int TK = CTK ? CTK : TKrt;  // CTK: the tile width fixed at compile time, else 0
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = g.nz;
    const ColTile t = col_tile<T>(g, TK, blockIdx);
    const int c3 = blockIdx.z;
    V *Uc = (V *)smem_raw;
    V *X = Uc + (size_t)nz * TK;
    V *Y = X + (size_t)fd.L * TK;
    const bool buoy = c3 == 2 && a.bouss;
    V *w = (V *)a.work[c3];
    if constexpr (E::kZoom) {
        if (a.nl_spec && fd.ztab) {
            // no staging buffer (more L1 for the transform tables): vin and cold by asynchronous
            // copies into the FFT buffer, the nonlinear spectrum and theta read in the update
            V *Xz = (V *)smem_raw;
            const int tile = nz * TK;
            tile_load_async(Xz, (const V *)a.vin[c3] + t.col0, t.zs, nz, TK, t.nv);
            tile_load_async(Xz + tile, (const V *)a.cold[c3] + t.col0, t.zs, nz, TK, t.nv);
            async_wait();
            __syncthreads();
            update_direct<T>(g, a, t, Xz, (const float2 *)a.nl[c3], buoy ? (const V *)a.vin[3] : nullptr,
                             pick<T>(a.xmom, a.f_xmom, a.q_xmom), pick<T>(a.nu, a.f_nu, a.q_nu), a.rot ? c3 : -1);
            if (c3 < 2) {
                vel_walls<T, E>(g, fd, a, t, c3, nullptr, Xz, nullptr, true, w);
                return;
            }
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                const int k = idx >> t.lgTK, c = idx & (TK - 1);
                if (c < t.nv) w[fidx<T>(g, k, t.ky, t.kx0 + c)] = Xz[idx];
            }
            return;
        }
    }
    nl_tile_load<T>(X, a, c3, t.col0, t.zs, nl_rows(g, a), TK, t.nv);
    if (buoy) {
        tile_load_async(Uc, (const V *)a.vin[3] + t.col0, t.zs, nz, TK, t.nv);
        async_wait_n<1>();
    } else {
        async_wait();
    }
    if (c3 < 2) {
        // the update stays in the FFT buffer and the wall round trip stores its result directly
        vel_update<T, E>(g, fd, a, t, c3, Uc, X, Y, buoy, true);
        vel_walls<T, E>(g, fd, a, t, c3, Uc, X, Y, true, w);
        return;
    }
    vel_update<T, E>(g, fd, a, t, c3, Uc, X, Y, buoy);
    for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
        const int k = idx >> t.lgTK, c = idx & (TK - 1);
        if (c < t.nv) w[fidx<T>(g, k, t.ky, t.kx0 + c)] = Uc[idx];
    }
}
template <typename T, class E, int CTK = 0>
__global__ void __launch_bounds__(E::kColThreads, E::kMinBlocks) k_fused_vcomp(Geo g, typename E::Desc fd, FusedArgs a, int TKrt) {
    fused_vcomp_body<T, E, CTK>(g, fd, a, TKrt, blockIdx);
}

// Split form, part 2: the projection of the three components written by k_fused_vcomp.
template <typename T, class E, int CTK>
__device__ __forceinline__ void fused_vproj_body(const Geo &g, const typename E::Desc &fd, const FusedArgs &a, int TKrt, uint3 blockIdx) {
    const int TK = CTK ? CTK : TKrt;  // CTK: the tile width fixed at compile time, else 0
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = g.nz;
    const ColTile t = col_tile<T>(g, TK, blockIdx);
    const int tile = nz * TK;
    if constexpr (E::kStreamProj) {
        V *X = (V *)smem_raw;
        V *Dsv = X + (size_t)E::kProjRows * TK;
        double2 *red = (double2 *)(Dsv + tile);
        double2 *coef = red + 4 * (blockDim.x >> 5) * TK;
        vel_project_streamed<T, E>(g, fd, a, t, X, Dsv, red, coef);
        return;
    }
    V *U = (V *)smem_raw;
    V *X = U + 3 * tile;
    V *Y = X + (size_t)fd.L * TK;
    double2 *red = (double2 *)(X + (size_t)E::kBuffers * fd.L * TK);
    double2 *coef = red + 2 * blockDim.x;
    for (int c3 = 0; c3 < 3; c3++) tile_load_async(U + c3 * tile, (const V *)a.work[c3] + t.col0, t.zs, nz, TK, t.nv);
    async_wait();
    __syncthreads();
    vel_project<T, E>(g, fd, a, t, U, X, Y, red, coef);
}
template <typename T, class E, int CTK = 0>
__global__ void __launch_bounds__(E::kColThreads, is_ff<T> ? E::kMinBlocks : 2) k_fused_vproj(Geo g, typename E::Desc fd, FusedArgs a, int TKrt) {
    fused_vproj_body<T, E, CTK>(g, fd, a, TKrt, blockIdx);
}

// ----------------------------------------------------------------------------------------------
// scalar column kernel (Boussinesq): smem = Th[nz][TK] + E::kBuffers * L * TK
// ----------------------------------------------------------------------------------------------
template <typename T, class E, int CTK = 0>
__global__ void __launch_bounds__(E::kColThreads, E::kMinBlocks) k_fused_theta(Geo g, typename E::Desc fd, FusedArgs a, int TKrt) {
    const int TK = CTK ? CTK : TKrt;  // CTK: the tile width fixed at compile time, else 0
    const int lgTK = lg2(TK);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = g.nz, nzp = g.nzp, L = fd.L;
    // float-float kernels with window tables: no staging buffer (the update reads the nonlinear
    // spectrum and vz from global memory), the FFT buffer first
    bool direct = false;
    if constexpr (E::kZoom) direct = fd.ztab && a.nl_spec;
    V *Th = (V *)smem_raw;
    V *X = direct ? Th : Th + (size_t)nz * TK;
    V *Y = X + (size_t)L * TK;
    const int kx0 = blockIdx.x * TK, ky = blockIdx.y;
    const int nv = min(TK, g.nxh - kx0);
    auto colq = [&](int z, int c) { return fidx<T>(g, z, ky, kx0 + c); };
    const T dt = pick<T>(a.dt, a.f_dt, a.q_dt), kap = pick<T>(a.kappa, a.f_kappa, a.q_kappa), rmp = pick<T>(a.rmp, a.f_rmp, a.q_rmp);
    const T inz = (T)1 / (T)nz, xtemp = pick<T>(a.xtemp, a.f_xtemp, a.q_xtemp);
    if (direct) {
        const ColTile t = col_tile<T>(g, TK, blockIdx);
        tile_load_async(X, (const V *)a.vin[3] + t.col0, t.zs, nz, TK, nv);
        tile_load_async(X + (size_t)nz * TK, (const V *)a.cold[3] + t.col0, t.zs, nz, TK, nv);
        async_wait();
        __syncthreads();
        update_direct<T>(g, a, t, X, (const float2 *)a.nl[3], (const V *)a.vin[2], xtemp, kap, -1);
    }
    // 1. NL_theta forward, heat current, filter, laplak, update.  vz is copied into Th while
    //    NL_theta is transformed; theta and cold go into the FFT buffer afterwards.
    if (!direct) {
        const int tile = nz * TK;
        const size_t zs = (size_t)g.ny * g.ldx, col0 = (size_t)ky * g.ldx + kx0;
        const bool stage2 = (size_t)E::kBuffers * L >= 2 * (size_t)nz;
        nl_tile_load<T>(X, a, 3, (unsigned)col0, (unsigned)zs, nl_rows(g, a), TK, nv);
        tile_load_async(Th, (const V *)a.vin[2] + col0, zs, nz, TK, nv);
        async_wait_n<1>();
        V *R = nl_forward<T, E>(g, fd, a, X, Y, TK);
        async_wait();
        __syncthreads();
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            V n = mk<T>(0, 0);
            if (c < nv) {
                const int kx = kx0 + c;
                n = R[E::pos(k, fd) * TK + c];
                const V w = Th[idx];
                n = mk<T>(n.x - xtemp * w.x, n.y - xtemp * w.y);
                n = cscale(n, g.FX<T>(kx));
                n = cscale(n, g.FY<T>(ky));
                n = cscale(n, g.FZ<T>(k));
            }
            Th[idx] = n;
        }
        __syncthreads();
        const V *cold = (const V *)a.cold[3];
        tile_load_async(X, (const V *)a.vin[3] + col0, zs, nz, TK, nv);
        if (stage2) tile_load_async(X + tile, cold + col0, zs, nz, TK, nv);
        async_wait();
        __syncthreads();
        // the updated theta goes straight into the FFT buffer (each thread reads its element first)
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) { X[idx] = mk<T>(0, 0); continue; }
            const int kx = kx0 + c;
            const T k2 = g.KX<T>(kx) * g.KX<T>(kx) + g.KY<T>(ky) * g.KY<T>(ky) + g.KZ<T>(k) * g.KZ<T>(k);
            const V t = X[idx], cv = stage2 ? X[tile + idx] : cold[colq(k, c)];
            const V n = Th[idx];
            const V lap = cscale(t, -k2);
            X[idx] = mk<T>(cv.x + dt * (kap * lap.x - n.x) * rmp, cv.y + dt * (kap * lap.y - n.y) * rmp);
        }
        __syncthreads();
    }
    // 2. s_imposebc (IFFT, 1/nz, walls = 0, continuation + FFT), then fc_filter.  With one
    //    in-place buffer in natural order (the Bluestein four-step engine) every step finishes
    //    in X; otherwise through Th.  Float-float kernels with window tables: as a window
    //    correction of the spectrum (zoom_round_trip).
    bool zoomed = false;
    if constexpr (E::kZoom) {
        if (fd.ztab) {
            zoom_round_trip<T, E>(g, fd, X, TK, true, [&](bool, int) { return mk<T>(0, 0); });
            if (a.rot) {
                V *out = (V *)a.vout[3];
                for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                    const int k = idx >> lgTK, c = idx & (TK - 1);
                    if (c < nv) out[colq(k, c)] = X[idx];
                }
                return;
            }
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                const int k = idx >> lgTK, c = idx & (TK - 1);
                const int kx = min(kx0 + c, g.nxh - 1);
                V v = X[idx];
                v = cscale(v, g.FX<T>(kx));
                v = cscale(v, g.FY<T>(ky));
                v = cscale(v, g.FZ<T>(k));
                X[idx] = v;
            }
            __syncthreads();
            zoomed = true;
        }
    }
    if (!zoomed) {
        V *R = E::run(X, Y, TK, fd, +1);
        bool inplace = R == X && fd.blue;
        V *P = inplace ? X : Th;
        for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            P[idx] = (k == 0 || k == nzp - 1) ? mk<T>(0, 0) : cscale(R[E::pos(k, fd) * TK + c], inz);
        }
        __syncthreads();
        if (!inplace) {
            for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) X[idx] = Th[idx];
            __syncthreads();
        }
        fc_continuation<T>(g, X, TK);
        __syncthreads();
        R = E::run(X, Y, TK, fd, -1);
        if (a.rot) {  // ROTBOUSS ends the scalar update with s_imposebc (rotbouss_rkstep2.f90:56)
            V *out = (V *)a.vout[3];
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                const int k = idx >> lgTK, c = idx & (TK - 1);
                if (c < nv) out[colq(k, c)] = R[E::pos(k, fd) * TK + c];
            }
            return;
        }
        inplace = R == X && fd.blue;
        P = inplace ? X : Th;
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            const int kx = min(kx0 + c, g.nxh - 1);
            V v = R[E::pos(k, fd) * TK + c];
            v = cscale(v, g.FX<T>(kx));
            v = cscale(v, g.FY<T>(ky));
            v = cscale(v, g.FZ<T>(k));
            P[idx] = v;
        }
        __syncthreads();
        if (!inplace) {
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) X[idx] = Th[idx];
            __syncthreads();
        }
    }
    // 3. c2r -> /(nx ny nz) -> r2c: z-inverse and 1/nz here; kx = 0 and nx/2 go to the side buffer.
    //    Tiles without those two columns, with window tables: continuation rows rebuilt as a
    //    window correction (no wall rows change).
    if constexpr (E::kZoom) {
        if (fd.ztab && kx0 > 0 && kx0 + TK < g.nxh) {
            zoom_round_trip<T, E>(g, fd, X, TK, false, [&](bool, int) { return mk<T>(0, 0); });
            V *out = (V *)a.vout[3];
            for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
                const int k = idx >> lgTK, c = idx & (TK - 1);
                if (c < nv) out[colq(k, c)] = X[idx];
            }
            return;
        }
    }
    {
        V *R = E::run(X, Y, TK, fd, +1);
        const bool inplace = R == X && fd.blue;
        V *P = inplace ? X : Th;
        V *side = (V *)a.side;
        for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            const V v = cscale(R[E::pos(k, fd) * TK + c], inz);
            P[idx] = v;
            const int kx = kx0 + c;
            if (c < nv && (kx == 0 || kx == g.nxh - 1))
                side[((unsigned)(kx == 0 ? 0 : 1) * g.ny + ky) * nzp + k] = v;
        }
        __syncthreads();
        if (!inplace) {
            for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) X[idx] = Th[idx];
            __syncthreads();
        }
        fc_continuation<T>(g, X, TK);
        __syncthreads();
        R = E::run(X, Y, TK, fd, -1);
        V *out = (V *)a.vout[3];
        for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            const int kx = kx0 + c;
            if (c < nv && kx != 0 && kx != g.nxh - 1) out[colq(k, c)] = R[E::pos(k, fd) * TK + c];
        }
    }
}

// kx = 0 and kx = nx/2 columns of the theta round trip: (X(ky) + conj X(-ky))/2, then continuation
// and forward z transform.  One block per (kx column, ky pair); two columns per block.
template <typename T, class E>
__global__ void __launch_bounds__(E::kColThreads, E::kMinBlocks) k_theta_herm(Geo g, typename E::Desc fd, FusedArgs a) {
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nzp = g.nzp, nz = g.nz, L = fd.L;
    const int TK = 2, lgTK = 1;
    V *X = (V *)smem_raw, *Y = X + (size_t)L * TK;
    const int sel = blockIdx.y;                 // 0: kx = 0, 1: kx = nx/2
    const int kx = sel == 0 ? 0 : g.nxh - 1;
    const int ky = blockIdx.x, kym = (g.ny - ky) % g.ny;
    if (ky > kym) return;                       // each pair once (ky <= -ky mod ny)
    const V *side = (const V *)a.side;
    const V *s1 = side + ((size_t)sel * g.ny + ky) * nzp, *s2 = side + ((size_t)sel * g.ny + kym) * nzp;
    for (int idx = threadIdx.x; idx < nzp * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        const V p = s1[k], m = s2[k];
        // column c = 0 holds ky, c = 1 holds -ky
        const T half = T(0.5f);
        const V h = c == 0 ? mk<T>(half * (p.x + m.x), half * (p.y - m.y)) : mk<T>(half * (m.x + p.x), half * (m.y - p.y));
        X[idx] = h;
    }
    __syncthreads();
    fc_continuation<T>(g, X, TK);
    __syncthreads();
    V *R = E::run(X, Y, TK, fd, -1);
    V *out = (V *)a.vout[3];
    for (int idx = threadIdx.x; idx < nz * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        if (c == 1 && kym == ky) continue;
        out[fidx<T>(g, k, c == 0 ? ky : kym, kx)] = R[E::pos(k, fd) * TK + c];
    }
}

// batched split velocity stage (batch.h): the two kernels over the tiles of several solvers
template <typename T, class E>
__global__ void __launch_bounds__(E::kColThreads, E::kMinBlocks) k_fused_vcomp_batch(const PassRec<E, FusedArgs> *recs, int n) {
    uint3 bid;
    const PassRec<E, FusedArgs> &r = batch_rec(recs, n, bid);
    fused_vcomp_body<T, E, 0>(r.g, r.fd, r.a, r.tk, bid);
}
template <typename T, class E>
__global__ void __launch_bounds__(E::kColThreads, is_ff<T> ? 1 : 2) k_fused_vproj_batch(const PassRec<E, FusedArgs> *recs, int n) {
    uint3 bid;
    const PassRec<E, FusedArgs> &r = batch_rec(recs, n, bid);
    fused_vproj_body<T, E, 0>(r.g, r.fd, r.a, r.tk, bid);
}

}  // namespace sg
