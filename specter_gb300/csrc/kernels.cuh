// Pass kernels over the device field layout.
//
// Device layout of every complex field (spectral (kz,ky,kx) or mixed (z,ky,kx)):
//     f[(z*ny + ky)*ldx + kx],  kx fastest, kx < nx/2+1 <= ldx (ldx padded to 8).
// The reference stores the same arrays z-fastest, C(nz,ny,nx/2+1); with kx fastest
// every pass is a batched strided FFT whose loads and stores are coalesced along kx,
// so no global transpose is needed: the x/y/z passes read (TK kx) x (length) tiles.
// Physical (real) fields use the reference layout r[(z*ny + y)*nx + x].
//
// Every pass kernel is templated on an FFT policy E:
//   GenericFFT<T>          Stockham / Bluestein over two smem buffers, any length (fft.cuh)
//   FourStep<T, L1, L2>    register four-step over one smem buffer, L = L1*L2 (fft4.cuh)
// E::run transforms rows [0, n) held in X and returns the buffer with the result;
// E::pos(k) is the smem row that holds output k.
#pragma once

#include "batch.h"
#include "fft.cuh"
#include "fft4.cuh"
#include "plan.h"

namespace sg {

constexpr int kThreads = 256;
constexpr int kMaxF = 4;  // fields per launch (blockIdx.z)

// element offset in a field; fields hold fewer than 2^32 elements (checked at plan creation), so
// offsets stay 32-bit (64-bit multiplies per element cost several instructions)
template <typename T>
__device__ __forceinline__ unsigned fidx(const Geo &g, int z, int ky, int kx) {
    return ((unsigned)z * (unsigned)g.ny + (unsigned)ky) * (unsigned)g.ldx + (unsigned)kx;
}

// A double kernel parameter in the kernel's precision.  FP32 kernels read the float mirror that
// the launcher fills (Args::prepared()): converting the double inside a kernel running at its
// register cap gets rematerialised per element on the FP64 pipe (1/64 rate here).
template <typename T>
__device__ __forceinline__ T pick(double d, float f) {
    if constexpr (is_f64<T>) return d;
    else return f;
}
// the same with a float-float mirror, for kernels that also run in float-float
template <typename T>
__device__ __forceinline__ T pick(double d, float f, ff q) {
    if constexpr (is_f64<T>) return d;
    else if constexpr (is_f32<T>) return f;
    else return q;
}

// NT: threads per block of the column kernels that run this engine (kColThreads).  The
// float-float column kernels take 255 registers a thread, so one block fills an SM's register
// file at 256 threads; 384 threads at a 170-register cap give 12 warps instead of 8 to hide
// the latency of the dependent float-float chains (plan option "ff_threads").
template <typename T, int NT = kThreads>
struct GenericFFT {
    using Desc = FFTDesc;
    static constexpr int kBuffers = 2;
    static constexpr bool kStreamProj = false;
    static constexpr int kProjRows = 0;
    static constexpr bool kZoom = false;
    static constexpr int kMinBlocks = 1;
    static constexpr int kColThreads = NT;
    static constexpr int kWideThreads = NT;
    static int wide_threads(int) { return NT; }
    static __device__ __forceinline__ C2<T> *run(C2<T> *X, C2<T> *Y, int B, const Desc &d, int sign) {
        return fft_exec<T>(X, Y, B, d, sign);
    }
    // input at rows pos(k), output in natural order
    static __device__ __forceinline__ C2<T> *run_perm(C2<T> *X, C2<T> *Y, int B, const Desc &d, int sign) {
        return fft_exec<T>(X, Y, B, d, sign);
    }
    static __device__ __forceinline__ int pos(int k, const Desc &) { return k; }
    // pos(m + D) - pos(m) for every m, or -1 when that is not a constant
    static __device__ __forceinline__ int pos_stride(int D, const Desc &) { return D; }
};

// OUTLINE = true calls the transforms out of line (kernels with many call sites).
template <typename T, int L1, int L2, bool OUTLINE = false>
struct FourStep {
    using Desc = FFT4Desc;
    static constexpr int kBuffers = 1;
    static constexpr bool kStreamProj = false;
    static constexpr int kProjRows = 0;
    static constexpr bool kZoom = false;
    static constexpr int kMinBlocks = 2;  // cap registers at 128 so two blocks share an SM
    static constexpr int kColThreads = kThreads;
    // Kernels that run one block per SM (the fused velocity kernel) may take enough threads for
    // one item per thread in both steps at a tile width of 8: 8 * max(L1, L2) rounded up to a
    // warp, at least kThreads.  With 36 x 30 that is 288, so the 288 items of step B do not leave
    // a one-warp second round behind a barrier.
    static constexpr int kWideThreads =
        (8 * (L1 > L2 ? L1 : L2) + 31) / 32 * 32 > kThreads ? (8 * (L1 > L2 ? L1 : L2) + 31) / 32 * 32 : kThreads;
    static int wide_threads(int tk) {
        const int need = (tk * (L1 > L2 ? L1 : L2) + 31) / 32 * 32;
        return need > kThreads && need <= kWideThreads ? need : kThreads;
    }
    static __device__ __forceinline__ C2<T> *run(C2<T> *X, C2<T> *, int B, const Desc &d, int sign) {
        if constexpr (OUTLINE) {
            if (d.blue) fft4_bluestein_ni<T, L1, L2>(X, B, d, sign);
            else if (sign < 0) fft4_np_ni<T, L1, L2, -1>(X, B, d);
            else fft4_np_ni<T, L1, L2, +1>(X, B, d);
            return X;
        }
        if (d.blue) {
            if (sign < 0) fft4_bluestein<T, L1, L2, -1>(X, B, d);
            else fft4_bluestein<T, L1, L2, +1>(X, B, d);
        } else {
            if (sign < 0) fft4_np<T, L1, L2, -1>(X, B, d);
            else fft4_np<T, L1, L2, +1>(X, B, d);
        }
        return X;
    }
    // input at rows pos(k) (permuted unless Bluestein), output in natural order
    static __device__ __forceinline__ C2<T> *run_perm(C2<T> *X, C2<T> *Y, int B, const Desc &d, int sign) {
        if (d.blue) return run(X, Y, B, d, sign);
        if (sign < 0) fft4_pn<T, L1, L2, -1>(X, B, d);
        else fft4_pn<T, L1, L2, +1>(X, B, d);
        return X;
    }
    // run(+1 or -1) that also completes the calling thread's asynchronous copies before its final
    // barrier (copies issued before the call are visible to the block on return)
    static __device__ __forceinline__ C2<T> *run_wait(C2<T> *X, C2<T> *Y, int B, const Desc &d, int sign) {
        if (d.blue) {
            C2<T> *R = run(X, Y, B, d, sign);
            async_wait();
            __syncthreads();
            return R;
        }
        if (sign < 0) fft4_np_impl<T, L1, L2, -1, true, true>(X, B, d);
        else fft4_np_impl<T, L1, L2, +1, true, true>(X, B, d);
        return X;
    }
    static __device__ __forceinline__ int pos(int k, const Desc &d) { return d.blue ? k : perm_pos<L1, L2>(k); }
    // pos(m + D) - pos(m) for every m, or -1 when that is not a constant
    static __device__ __forceinline__ int pos_stride(int D, const Desc &d) {
        return d.blue ? D : (D % L1 == 0 ? D / L1 : -1);
    }
};

// ---------------------------------------------------------------------------------
// z pass, inverse: out0 = scale * IFFT_z(in) (+ add), out1 = scale * IFFT_z(i kz in).
// Rows [0, nrows) are written.  fftp1d_complex_to_real_z, src/fftp/fftp.fpp:1060-1094.
// ---------------------------------------------------------------------------------
struct ZInvArgs {
    const void *in[kMaxF];
    void *out0[kMaxF];
    void *out1[kMaxF];
    const void *add[kMaxF];
    int nrows;
    int scale_rows;   // rows [0, scale_rows) scaled, the rest copied unscaled
    double scale;
    int staged;       // 1: the input tile is staged once in smem (some field has two outputs)
    int in_ff;        // FP32 kernels: the inputs are float-float fields, read as the rounded sum of
                      // each pair (the precision form's nonlinear term reads its state so)
    float scale_f;
    ZInvArgs prepared() const { ZInvArgs b = *this; b.scale_f = (float)scale; return b; }
};

// [rows][TK] tile of a float-float complex field as FP32 values (the rounded sum of each pair),
// element (k, c) from src[k * stride + c] for c < nv, zero for nv <= c < TK; eight 16-byte loads
// per thread in flight.  Visible to the block after the caller's barrier.
__device__ __forceinline__ void tile_load_ff_as_f32(float2 *dst, const ffc *src, unsigned stride, int rows, int TK,
                                                    int nv) {
    const int lgTK = lg2(TK), total = rows * TK;
    for (int base = threadIdx.x; base < total; base += 8 * blockDim.x) {
        float4 f[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int idx = base + u * blockDim.x;
            const int k = idx >> lgTK, c = idx & (TK - 1);
            f[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (idx < total && c < nv) f[u] = __ldg((const float4 *)(src + ((unsigned)k * stride + (unsigned)c)));
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int idx = base + u * blockDim.x;
            if (idx < total) dst[idx] = make_float2(f[u].x + f[u].y, f[u].z + f[u].w);
        }
    }
}

template <typename T, class E, int CTK>
__device__ __forceinline__ void z_inverse_body(const Geo &g, const typename E::Desc &fd, const ZInvArgs &a, int TKrt, uint3 blockIdx) {
    const int TK = CTK ? CTK : TKrt;  // CTK: the tile width fixed at compile time, else 0
    const int lgTK = lg2(TK);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *X = (V *)smem_raw, *Y = X + (size_t)fd.L * TK;
    V *S = X + (size_t)E::kBuffers * fd.L * TK;  // staged input tile (a.staged)
    const int kx0 = blockIdx.x * TK, ky = blockIdx.y, f = blockIdx.z;
    const V *in = (const V *)a.in[f];
    const int nv = min(TK, g.nxh - kx0);
    const unsigned zstride = (unsigned)g.ny * g.ldx;
    const V *src = in + (unsigned)ky * g.ldx + kx0;
    const T sc = pick<T>(a.scale, a.scale_f);
    // float-float inputs (FP32 kernels only): converting loads in place of the asynchronous copies
    auto load_tile = [&](V *dst) {
        if constexpr (is_f32<T>) {
            if (a.in_ff) {
                tile_load_ff_as_f32(dst, (const ffc *)a.in[f] + (unsigned)ky * g.ldx + kx0, zstride, g.nz, TK, nv);
                return;
            }
        }
        tile_load_async(dst, src, zstride, g.nz, TK, nv);
    };
    if (a.staged) load_tile(S);
    for (int pass = 1; pass >= 0; pass--) {  // derivative output first: out0 may alias in
        V *out = (V *)(pass == 0 ? a.out0[f] : a.out1[f]);
        if (!out) continue;
        if (a.staged) {
            async_wait();
            __syncthreads();
            for (int idx = threadIdx.x; idx < g.nz * TK; idx += blockDim.x) {
                const V v = S[idx];
                X[idx] = pass == 1 ? cimk(g.KZ<T>(idx >> lgTK), v) : v;
            }
        } else {
            load_tile(X);
            async_wait();
            if (pass == 1) {
                __syncthreads();
                for (int idx = threadIdx.x; idx < g.nz * TK; idx += blockDim.x) X[idx] = cimk(g.KZ<T>(idx >> lgTK), X[idx]);
            }
        }
        __syncthreads();
        V *R = E::run(X, Y, TK, fd, +1);
        const V *add = (const V *)a.add[f];
        for (int idx = threadIdx.x; idx < a.nrows * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c >= nv) continue;
            V v = R[E::pos(k, fd) * TK + c];
            if (k < a.scale_rows) v = cscale(v, sc);
            const unsigned q = fidx<T>(g, k, ky, kx0 + c);
            if (pass == 0 && add) v = cadd(v, add[q]);
            out[q] = v;
        }
        __syncthreads();
    }
}
template <typename T, class E, int CTK = 0>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_z_inverse(Geo g, typename E::Desc fd, ZInvArgs a, int TKrt) {
    z_inverse_body<T, E, CTK>(g, fd, a, TKrt, blockIdx);
}

// ---------------------------------------------------------------------------------
// z pass, forward with FC-Gram continuation: rows [0, nzp) are read (times in_scale),
// rows [nzp, nz) are rebuilt from the first and last d rows with dir = A.Q^T in FP64
// (src/fftp/fftp.fpp:755-773), then the forward FFT (:780) writes all nz rows.
// ---------------------------------------------------------------------------------
struct ZFwdArgs {
    const void *in[kMaxF];
    void *out[kMaxF];
    double in_scale;
    float in_scale_f;
    ZFwdArgs prepared() const { ZFwdArgs b = *this; b.in_scale_f = (float)in_scale; return b; }
};

constexpr int kMaxOz = 9;   // largest d of the FC-Gram tables (Q3 .. Q9)
constexpr int kMaxTile = 16; // largest tile width of the column passes

// Called by every thread of the block with X rows [0, nzp) filled and visible; returns with the
// continuation rows written (visible after the caller's next barrier).
template <typename T>
__device__ __forceinline__ void fc_continuation(const Geo &g, C2<T> *X, int TK) {
    // the 2d wall-adjacent values of each column in FP64, converted once per column rather than
    // once per continued row: wv[j][c] = row nzp-d+j (j < d), row d-1-(j-d) (j >= d)
    __shared__ double2 wv[2 * kMaxOz * kMaxTile];
    const int lgTK = lg2(TK);
    const int C = g.cz, d = g.oz, n = g.nz;
    if constexpr (is_ff<T>) {
        // float-float kernels: the sums in float-float with dir split into float-float pairs
        for (int idx = threadIdx.x; idx < C * TK; idx += blockDim.x) {
            const int ii = idx >> lgTK, c = idx & (TK - 1);
            ff ar(0), ai(0);
            for (int jj = 0; jj < d; jj++) {
                const C2<T> t = X[(n - C - d + jj) * TK + c], b = X[(d - 1 - jj) * TK + c];
                const float2 q0 = __ldg((const float2 *)(g.dirq + ii + C * jj));
                const float2 q1 = __ldg((const float2 *)(g.dirq + (C - 1 - ii) + C * jj));
                const ff w0(q0.x, q0.y), w1(q1.x, q1.y);
                ar = ar + w0 * t.x + w1 * b.x;
                ai = ai + w0 * t.y + w1 * b.y;
            }
            C2<T> r;
            r.x = ar;
            r.y = ai;
            X[(n - C + ii) * TK + c] = r;
        }
    } else {
        for (int idx = threadIdx.x; idx < 2 * d * TK; idx += blockDim.x) {
            const int j = idx >> lgTK, c = idx & (TK - 1);
            const int row = j < d ? n - C - d + j : d - 1 - (j - d);
            const C2<T> v = X[row * TK + c];
            wv[idx] = make_double2((double)v.x, (double)v.y);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < C * TK; idx += blockDim.x) {
            const int ii = idx >> lgTK, c = idx & (TK - 1);
            const double2 t0 = wv[c], b0 = wv[d * TK + c];
            const double a0 = __ldg(g.dir + ii), a1 = __ldg(g.dir + (C - 1 - ii));
            double ar = a0 * t0.x + a1 * b0.x;
            double ai = a0 * t0.y + a1 * b0.y;
            for (int jj = 1; jj < d; jj++) {
                const double2 t = wv[jj * TK + c], b = wv[(d + jj) * TK + c];
                const double w0 = __ldg(g.dir + ii + C * jj), w1 = __ldg(g.dir + (C - 1 - ii) + C * jj);
                ar = ar + w0 * t.x + w1 * b.x;
                ai = ai + w0 * t.y + w1 * b.y;
            }
            X[(n - C + ii) * TK + c] = mk<T>((T)ar, (T)ai);
        }
    }
}

template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_z_forward(Geo g, typename E::Desc fd, ZFwdArgs a, int TK) {
    const int lgTK = lg2(TK);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *X = (V *)smem_raw, *Y = X + (size_t)fd.L * TK;
    const int kx0 = blockIdx.x * TK, ky = blockIdx.y, f = blockIdx.z;
    const V *in = (const V *)a.in[f];
    V *out = (V *)a.out[f];
    const int nv = min(TK, g.nxh - kx0);
    const T s = pick<T>(a.in_scale, a.in_scale_f);
    tile_load_async(X, in + (unsigned)ky * g.ldx + kx0, (unsigned)g.ny * g.ldx, g.nzp, TK, nv);
    async_wait();
    if (a.in_scale != 1.0) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < g.nzp * TK; idx += blockDim.x) X[idx] = cscale(X[idx], s);
    }
    __syncthreads();
    fc_continuation<T>(g, X, TK);
    __syncthreads();
    V *R = E::run(X, Y, TK, fd, -1);
    for (int idx = threadIdx.x; idx < g.nz * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        if (c < nv) out[fidx<T>(g, k, ky, kx0 + c)] = R[E::pos(k, fd) * TK + c];
    }
}

// ---------------------------------------------------------------------------------
// y pass: out0 = scale * FFT_y^sign(in), out1 = scale * FFT_y^sign(i ky in), planes [0, nplanes).
// ---------------------------------------------------------------------------------
struct YArgs {
    const void *in[kMaxF];
    void *out0[kMaxF];
    void *out1[kMaxF];
    int sign;
    double scale;
    int staged;       // 1: the input tile is staged once in smem (some field has two outputs)
    float scale_f;
    YArgs prepared() const { YArgs b = *this; b.scale_f = (float)scale; return b; }
};

// CTK: the tile width when fixed at compile time, else 0 and the runtime TKrt
template <typename T, class E, int CTK>
__device__ __forceinline__ void y_pass_body(const Geo &g, const typename E::Desc &fd, const YArgs &a, int TKrt, uint3 blockIdx) {
    const int TK = CTK ? CTK : TKrt;
    const int lgTK = CTK ? (CTK == 16 ? 4 : CTK == 8 ? 3 : CTK == 4 ? 2 : CTK == 2 ? 1 : 0) : lg2(TKrt);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *X = (V *)smem_raw, *Y = X + (size_t)fd.L * TK;
    V *S = X + (size_t)E::kBuffers * fd.L * TK;  // staged input tile (a.staged)
    const int kx0 = blockIdx.x * TK, z = blockIdx.y, f = blockIdx.z;
    const V *in = (const V *)a.in[f];
    const int nv = min(TK, g.nxh - kx0);
    const T sc = pick<T>(a.scale, a.scale_f);
    const bool scaled = is_f64<T> ? a.scale != 1.0 : a.scale_f != 1.0f;
    const V *src = in + (unsigned)z * g.ny * g.ldx + kx0;
    if (a.staged) tile_load_async(S, src, (unsigned)g.ldx, g.ny, TK, nv);
    for (int pass = 1; pass >= 0; pass--) {  // derivative output first: out0 may alias in
        V *out = (V *)(pass == 0 ? a.out0[f] : a.out1[f]);
        if (!out) continue;
        if (a.staged) {
            async_wait();
            __syncthreads();
            for (int idx = threadIdx.x; idx < g.ny * TK; idx += blockDim.x) {
                const V v = S[idx];
                X[idx] = pass == 1 ? cimk(g.KY<T>(idx >> lgTK), v) : v;
            }
        } else {
            tile_load_async(X, src, (unsigned)g.ldx, g.ny, TK, nv);
            async_wait();
            if (pass == 1) {
                __syncthreads();
                for (int idx = threadIdx.x; idx < g.ny * TK; idx += blockDim.x) X[idx] = cimk(g.KY<T>(idx >> lgTK), X[idx]);
            }
        }
        __syncthreads();
        V *R = E::run(X, Y, TK, fd, a.sign);
        for (int idx = threadIdx.x; idx < g.ny * TK; idx += blockDim.x) {
            const int k = idx >> lgTK, c = idx & (TK - 1);
            if (c < nv) {
                V v = R[E::pos(k, fd) * TK + c];
                if (scaled) v = cscale(v, sc);
                out[fidx<T>(g, z, k, kx0 + c)] = v;
            }
        }
        __syncthreads();
    }
}
template <typename T, class E, int CTK>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_y_pass_t(Geo g, typename E::Desc fd, YArgs a, int TKrt) {
    y_pass_body<T, E, CTK>(g, fd, a, TKrt, blockIdx);
}

// ---------------------------------------------------------------------------------
// x pass helpers: real rows of length nx = 2H through a complex FFT of length H.
// A block takes RB rows.  Rows move between HBM and shared memory through a staging
// buffer S[k][r] of row stride SP = RB + 1 (odd, so that both the row-contiguous global
// side and the column-contiguous shared side run without bank conflicts); the FFT buffer
// X[pos][r] has stride RB.
// ---------------------------------------------------------------------------------

// Build Z (H rows, natural order) for a C2R from the half spectrum S (nxh rows):
// Z_k = (X_k + conj X_{H-k}) + i e^{+2 pi i k/nx} (X_k - conj X_{H-k}); Im X_0 = Im X_H = 0.
// dx = 1 first multiplies the spectrum by i kx (the x derivative).  With e, o the two terms of
// Z_k, Z_{H-k} = conj(e) + i conj(o): one thread forms the pair (k, H-k) from the same two
// loads and one twiddle (k = 0 pairs X_0 with X_H and forms Z_0 only).
template <typename T>
__device__ __forceinline__ void c2r_pre(const Geo &g, const C2<T> *S, C2<T> *Z, int RB, int SP, int dx = 0) {
    const int lgRB = lg2(RB);
    using V = C2<T>;
    const V *xtw = (const V *)g.xtw;
    const int H = g.H, Hh = H >> 1;
    for (int idx = threadIdx.x; idx < (Hh + 1) * RB; idx += blockDim.x) {
        const int k = idx >> lgRB, r = idx & (RB - 1);
        V xk = S[k * SP + r], xm = S[(H - k) * SP + r];
        if (dx) {
            xk = cimk(g.KX<T>(k), xk);
            xm = cimk(g.KX<T>(H - k), xm);
        }
        if (k == 0) { xk.y = 0; xm.y = 0; }
        const V xmc = cconj(xm);
        const V e = cadd(xk, xmc);
        V w = __ldg(xtw + k);
        w.y = -w.y;  // exp(+2 pi i k / nx)
        const V o = cmul(csub(xk, xmc), w);
        Z[idx] = mk<T>(e.x - o.y, e.y + o.x);
        if (k != 0 && 2 * k != H) Z[(H - k) * RB + r] = mk<T>(e.x + o.y, o.x - e.y);
    }
}

// From Z = FFT_H(packed real row), write the half spectrum X_0..X_H into S:
//   X_k = (Z_k + conj Z_{H-k})/2 - (i/2) e^{-2 pi i k/nx} (Z_k - conj Z_{H-k}).
// With e = Z_k + conj Z_{H-k} and t = e^{-2 pi i k/nx} (Z_k - conj Z_{H-k}), X_k = (e - i t)/2
// and X_{H-k} = (conj(e) - i conj(t))/2: one thread forms the pair (k, H-k); k = 0 also gives
// X_H.
// Output k of Z sits at row E::pos(k), or at row k when NAT.
template <typename T, class E, bool NAT = false>
__device__ __forceinline__ void r2c_post(const Geo &g, const typename E::Desc &fd, const C2<T> *Z, C2<T> *S, int RB,
                                         int SP) {
    const int lgRB = lg2(RB);
    using V = C2<T>;
    const V *xtw = (const V *)g.xtw;
    const int H = g.H, Hh = H >> 1;
    for (int idx = threadIdx.x; idx < (Hh + 1) * RB; idx += blockDim.x) {
        const int k = idx >> lgRB, r = idx & (RB - 1);
        const int km = k ? H - k : 0;
        const int p0 = NAT ? k : E::pos(k, fd), p1 = NAT ? km : E::pos(km, fd);
        const V zk = Z[p0 * RB + r], zm = cconj(Z[p1 * RB + r]);
        const V e = cadd(zk, zm), d = csub(zk, zm);
        const V t = cmul(d, __ldg(xtw + k));
        S[k * SP + r] = mk<T>((T)0.5 * (e.x + t.y), (T)0.5 * (e.y - t.x));
        if (2 * k != H) S[(H - k) * SP + r] = mk<T>((T)0.5 * (e.x - t.y), (T)-0.5 * (e.y + t.x));
    }
}

// shared [rows][SP] staging -> rows of a global array (row stride ld), rows < nv
template <typename V>
__device__ __forceinline__ void rows_store(V *out, unsigned ld, const V *S, int rows, int SP, int nv) {
    // (r, k) = divmod(idx, rows), advanced by blockDim.x without dividing per element
    const int sr = blockDim.x / rows, sk = blockDim.x - sr * rows;
    int r = threadIdx.x / rows, k = threadIdx.x - r * rows;
    for (int idx = threadIdx.x; idx < rows * nv; idx += blockDim.x) {
        out[(unsigned)r * ld + k] = S[k * SP + r];
        r += sr;
        k += sk;
        if (k >= rows) { k -= rows; r++; }
    }
}

// x pass R2C of real rows: out[row] = FFT_x(r[row]) for rows (z,y), z < nrows.
struct XArgs {
    const void *in[kMaxF];
    void *out[kMaxF];
    int nrows;  // z planes
    double scale;
    float scale_f;
    XArgs prepared() const { XArgs b = *this; b.scale_f = (float)scale; return b; }
};

// shared memory of the x pass kernels: FFT buffer(s) + staging, for RB rows
template <class E>
__host__ __device__ inline size_t x_pass_elems(const typename E::Desc &fd, int nxh, int RB) {
    return (size_t)E::kBuffers * fd.L * RB + (size_t)nxh * (RB + 1);
}

template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_x_r2c(Geo g, typename E::Desc fd, XArgs a, int RB) {
    const int lgRB = lg2(RB);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int SP = RB + 1;
    V *X = (V *)smem_raw, *Y = X + (size_t)fd.L * RB, *S = X + (size_t)E::kBuffers * fd.L * RB;
    const int f = blockIdx.z;
    const int row0 = blockIdx.x * RB, nrows = a.nrows * g.ny;
    const int nv = min(RB, nrows - row0);
    const T *in = (const T *)a.in[f];
    V *out = (V *)a.out[f];
    const int H = g.H;
    // packed real row: element m = (x_{2m}, x_{2m+1})
    rows_load_async(S, (const V *)(in + (size_t)row0 * g.nx), (unsigned)H, H, RB, nv, SP);
    async_wait();
    __syncthreads();
    for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x) X[idx] = S[(idx >> lgRB) * SP + (idx & (RB - 1))];
    __syncthreads();
    V *R = E::run(X, Y, RB, fd, -1);
    r2c_post<T, E>(g, fd, R, S, RB, SP);
    __syncthreads();
    if (a.scale != 1.0) {
        const T sc = pick<T>(a.scale, a.scale_f);
    const bool scaled = is_f64<T> ? a.scale != 1.0 : a.scale_f != 1.0f;
        for (int idx = threadIdx.x; idx < g.nxh * SP; idx += blockDim.x) S[idx] = cscale(S[idx], sc);
    }
    __syncthreads();
    rows_store(out + (size_t)row0 * g.ldx, (unsigned)g.ldx, S, g.nxh, SP, nv);
}

// x pass C2R: r[row] = IFFT_x(in[row]) (Hermitian half spectrum; Im of kx=0, nx/2 ignored)
template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_x_c2r(Geo g, typename E::Desc fd, XArgs a, int RB) {
    const int lgRB = lg2(RB);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int SP = RB + 1;
    V *X = (V *)smem_raw, *Y = X + (size_t)fd.L * RB, *S = X + (size_t)E::kBuffers * fd.L * RB;
    const int f = blockIdx.z;
    const int row0 = blockIdx.x * RB, nrows = a.nrows * g.ny;
    const int nv = min(RB, nrows - row0);
    const V *in = (const V *)a.in[f];
    T *out = (T *)a.out[f];
    rows_load_async(S, in + (size_t)row0 * g.ldx, (unsigned)g.ldx, g.nxh, RB, nv, SP);
    async_wait();
    __syncthreads();
    c2r_pre<T>(g, S, X, RB, SP);
    __syncthreads();
    V *R = E::run(X, Y, RB, fd, +1);
    const int H = g.H;
    const T sc = pick<T>(a.scale, a.scale_f);
    const bool scaled = is_f64<T> ? a.scale != 1.0 : a.scale_f != 1.0f;
    for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x) {
        const int m = idx >> lgRB, r = idx & (RB - 1);
        V v = R[E::pos(m, fd) * RB + r];
        if (scaled) v = cscale(v, sc);
        S[m * SP + r] = v;
    }
    __syncthreads();
    rows_store((V *)(out + (size_t)row0 * g.nx), (unsigned)H, S, H, SP, nv);
}

// ---------------------------------------------------------------------------------
// Fused x pass for the nonlinear terms (gradre, pseudospec_hd.f90:209-319, and advect,
// pseudospec_phd.f90:23-113).  Per (y,z) row, inputs are the y-inverse-transformed rows
// U_j (velocity), DY_i = d/dy v_i, DZ_i = d/dz v_i (and theta's).  d/dx is i*kx applied
// to the spectral row.  Physical rows stay packed as H complex numbers
// (x_{2m} + i x_{2m+1}); products act on real and imaginary parts separately.
//   NL_i = ((u_x d_x v_i + u_y d_y v_i) + u_z d_z v_i) * 1/(nx ny nz)^2
// then a forward R2C of each NL_i.
// ---------------------------------------------------------------------------------
struct XNLArgs {
    const void *u[4];    // v_x, v_y, v_z, theta rows (z,y,kx); u[3] only when c1 == 4
    const void *dy[4];   // d/dy v_x, v_y, v_z, theta
    const void *dz[4];   // d/dz v_x, v_y, v_z, theta
    void *out[4];        // NL_x, NL_y, NL_z, NL_theta  (z,y,kx)
    int c0, c1;          // components [c0, c1) are formed (0..2 velocity, 3 scalar)
    int nrows;           // physical z planes
    double tmp;          // 1/(nx ny nz)^2
    float tmp_f;
    XNLArgs prepared() const { XNLArgs b = *this; b.tmp_f = (float)tmp; return b; }
};

// Input t of the nonlinear x pass: t < 3 the velocity rows; then per component i in [c0, c1)
// the three rows v_i (to be multiplied by i kx), d/dy v_i, d/dz v_i (term = 0, 1, 2).
template <typename T>
__device__ __forceinline__ const C2<T> *xnl_input(const XNLArgs &a, int t, int &term, int &i) {
    if (t < 3) { term = -1; i = t; return (const C2<T> *)a.u[t]; }
    t -= 3;
    term = t % 3;
    i = a.c0 + t / 3;
    return (const C2<T> *)(term == 0 ? a.u[i] : term == 1 ? a.dy[i] : a.dz[i]);
}

// ---- pipelined form (four-step engine, FP32, fixed row count) --------------------------------
// Two FFT buffers: the pre-processing of input t+1 runs in the same phase as the products of
// input t, and the copy of input t+2 into the staging buffer is completed inside the transform
// of input t+1 (FourStep::run_wait), so each input costs one barrier besides the transform's
// two.  The staging buffer is row-major, S[r * SK + k] (16-byte copies of (k, k+1) pairs; with
// SK = 4 mod 16 the column reads of the pre-processing fall two to a bank), and
// the forward R2C post-processing writes a row-major copy into the accumulator, free by then.
__host__ __device__ inline int x_stage_stride(int nxh) { return ((nxh - 4 + 15) / 16) * 16 + 4; }

__host__ __device__ inline size_t x_nl_pipe_elems(int nxh, int H, int RB) {
    const size_t sk = (size_t)RB * x_stage_stride(nxh);
    return (size_t)2 * H * RB + sk + (size_t)3 * H * RB + (sk > (size_t)H * RB ? sk : (size_t)H * RB);
}

// rows r < nv of a complex field (row stride ld) -> S[r * SK + k], k < nxh; rows nv <= r < RB are zero
template <typename V>
__device__ __forceinline__ void rows_load_rm(V *S, const V *src, unsigned ld, int nxh, int RB, int nv, int SK) {
    static_assert(sizeof(V) == 8, "16-byte pair copies of single-precision complex values");
    const int PP = (nxh + 1) >> 1;  // (k, k+1) pairs per row
    const int sr = blockDim.x / PP, sp = blockDim.x - sr * PP;
    int r = threadIdx.x / PP, p = threadIdx.x - r * PP;
    for (int idx = threadIdx.x; idx < RB * PP; idx += blockDim.x) {
        const int k = 2 * p;
        V *d = S + r * SK + k;
        if (r < nv) {
            const V *gsrc = src + ((unsigned)r * ld + (unsigned)k);
            if (k + 1 < nxh) cp_async<16>(d, gsrc);
            else cp_async<8>(d, gsrc);
        } else {
            V z;
            z.x = 0;
            z.y = 0;
            d[0] = z;
            if (k + 1 < nxh) d[1] = z;
        }
        r += sr;
        p += sp;
        if (p >= PP) { p -= PP; r++; }
    }
    async_commit();
}

// c2r_pre from the row-major staging (same arithmetic)
template <typename T>
__device__ __forceinline__ void c2r_pre_rm(const Geo &g, const C2<T> *S, int SK, C2<T> *Z, int RB, int lgRB, int dx) {
    using V = C2<T>;
    const V *xtw = (const V *)g.xtw;
    const int H = g.H, Hh = H >> 1;
    for (int idx = threadIdx.x; idx < (Hh + 1) * RB; idx += blockDim.x) {
        const int k = idx >> lgRB, r = idx & (RB - 1);
        V xk = S[r * SK + k], xm = S[r * SK + H - k];
        if (dx) {
            xk = cimk(g.KX<T>(k), xk);
            xm = cimk(g.KX<T>(H - k), xm);
        }
        if (k == 0) { xk.y = 0; xm.y = 0; }
        const V xmc = cconj(xm);
        const V e = cadd(xk, xmc);
        V w = __ldg(xtw + k);
        w.y = -w.y;  // exp(+2 pi i k / nx)
        const V o = cmul(csub(xk, xmc), w);
        Z[idx] = mk<T>(e.x - o.y, e.y + o.x);
        if (k != 0 && 2 * k != H) Z[(H - k) * RB + r] = mk<T>(e.x + o.y, o.x - e.y);
    }
}

// r2c_post into a row-major buffer: Z (output k of the forward transform from permuted input,
// E::run_perm, which leaves natural order: row k) -> O[r * SK + k], k <= H
template <typename T, class E>
__device__ __forceinline__ void r2c_post_rm(const Geo &g, const typename E::Desc &fd, const C2<T> *Z, C2<T> *O, int SK,
                                            int RB, int lgRB) {
    using V = C2<T>;
    const V *xtw = (const V *)g.xtw;
    const int H = g.H, Hh = H >> 1;
    (void)fd;
    for (int idx = threadIdx.x; idx < (Hh + 1) * RB; idx += blockDim.x) {
        const int k = idx >> lgRB, r = idx & (RB - 1);
        const V zk = Z[k * RB + r], zm = cconj(Z[(k ? H - k : 0) * RB + r]);
        const V e = cadd(zk, zm), d = csub(zk, zm);
        const V t = cmul(d, __ldg(xtw + k));
        O[r * SK + k] = mk<T>((T)0.5 * (e.x + t.y), (T)0.5 * (e.y - t.x));
        if (2 * k != H) O[r * SK + H - k] = mk<T>((T)0.5 * (e.x - t.y), (T)-0.5 * (e.y + t.x));
    }
}

// rows r < nv of O[r * SK + k] -> out[r * ld + k], k < nxh, 16-byte stores of (k, k+1) pairs
template <typename V>
__device__ __forceinline__ void rows_store_rm(V *out, unsigned ld, const V *O, int SK, int nxh, int nv) {
    static_assert(sizeof(V) == 8, "16-byte pair stores of single-precision complex values");
    const int PP = (nxh + 1) >> 1;
    const int sr = blockDim.x / PP, sp = blockDim.x - sr * PP;
    int r = threadIdx.x / PP, p = threadIdx.x - r * PP;
    for (int idx = threadIdx.x; idx < nv * PP; idx += blockDim.x) {
        const int k = 2 * p;
        V *d = out + ((unsigned)r * ld + (unsigned)k);
        const V *o = O + r * SK + k;
        if (k + 1 < nxh) {
            const float4 v = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
            *(float4 *)d = v;
        } else {
            d[0] = o[0];
        }
        r += sr;
        p += sp;
        if (p >= PP) { p -= PP; r++; }
    }
}

template <typename T, class E, int RB>
__device__ __forceinline__ void x_nonlinear_pipe(const Geo &g, const typename E::Desc &fd, const XNLArgs &a) {
    constexpr int lgRB = RB == 16 ? 4 : RB == 8 ? 3 : RB == 4 ? 2 : RB == 2 ? 1 : 0;
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int H = g.H, nxh = g.nxh, SK = x_stage_stride(nxh);
    V *Xb[2];
    Xb[0] = (V *)smem_raw;                 // two FFT buffers of H x RB
    Xb[1] = Xb[0] + (size_t)H * RB;
    V *S = Xb[1] + (size_t)H * RB;         // RB x SK row-major staging
    V *U = S + (size_t)RB * SK;            // 3 x H x RB physical velocity rows
    V *A = U + (size_t)3 * H * RB;         // H x RB accumulator; RB x SK output staging after term 2
    const int nc = a.c1 - a.c0, T_in = 3 + 3 * nc;
    const int row0 = blockIdx.x * RB, nv = min(RB, a.nrows * g.ny - row0);
    const T tmp = pick<T>(a.tmp, a.tmp_f);
    const size_t off = (size_t)row0 * g.ldx;
    const unsigned ld = (unsigned)g.ldx;
    int term, i, tn, in_;
    // input 0 into Xb[0]; input 1 copied into S during the first transform
    rows_load_rm(S, xnl_input<T>(a, 0, term, i) + off, ld, nxh, RB, nv, SK);
    async_wait();
    __syncthreads();
    c2r_pre_rm<T>(g, S, SK, Xb[0], RB, lgRB, term == 0);
    __syncthreads();
    if (T_in > 1) rows_load_rm(S, xnl_input<T>(a, 1, tn, in_) + off, ld, nxh, RB, nv, SK);
    E::run_wait(Xb[0], nullptr, RB, fd, +1);
    // output m of a transform sits at row E::pos(m); m advances by D per iteration, so the row
    // advances by a constant when the engine's permutation is affine along that stride
    const int D = blockDim.x >> lgRB, ps = E::pos_stride(D, fd), r0 = threadIdx.x & (RB - 1);
    for (int t = 0; t < T_in; t++) {
        xnl_input<T>(a, t, term, i);
        V *R = Xb[t & 1], *Xn = Xb[(t + 1) & 1];
        // S holds input t+1, completed inside the transform of input t: pre-process it
        // beside the products of input t
        if (t + 1 < T_in) {
            xnl_input<T>(a, t + 1, tn, in_);
            c2r_pre_rm<T>(g, S, SK, Xn, RB, lgRB, tn == 0);
        }
        int q = E::pos(threadIdx.x >> lgRB, fd) * RB + r0;
        if (term < 2) {
            for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x, q += ps * RB) {
                if (ps < 0) q = E::pos(idx >> lgRB, fd) * RB + r0;
                const V p = R[q];
                if (term < 0) {
                    U[i * H * RB + idx] = p;
                } else if (term == 0) {
                    const V u = U[idx];
                    A[idx] = mk<T>(u.x * p.x, u.y * p.y);
                } else {
                    const V u = U[H * RB + idx];
                    A[idx] = mk<T>(A[idx].x + u.x * p.x, A[idx].y + u.y * p.y);
                }
            }
        } else {
            // (acc + u_z d/dz v_i) * tmp in place
            for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x, q += ps * RB) {
                if (ps < 0) q = E::pos(idx >> lgRB, fd) * RB + r0;
                const V u = U[2 * H * RB + idx], p = R[q], acc = A[idx];
                R[q] = mk<T>((acc.x + u.x * p.x) * tmp, (acc.y + u.y * p.y) * tmp);
            }
        }
        __syncthreads();  // S consumed, Xn pre-processed, the products of input t done
        if (t + 2 < T_in) rows_load_rm(S, xnl_input<T>(a, t + 2, tn, in_) + off, ld, nxh, RB, nv, SK);
        if (term == 2) {
            // forward transform from permuted order; R2C post-processing into A (free until the
            // next component's first product, which comes after the next transform's barriers)
            E::run_perm(R, nullptr, RB, fd, -1);
            r2c_post_rm<T, E>(g, fd, R, A, SK, RB, lgRB);
            __syncthreads();
            rows_store_rm((V *)a.out[i] + off, ld, A, SK, nxh, nv);
        }
        if (t + 1 < T_in) E::run_wait(Xn, nullptr, RB, fd, +1);
    }
}

// shared memory of k_x_nonlinear: X, S, U[3][H], A[H] for RB rows
template <class E>
__host__ __device__ inline size_t x_nl_elems(const typename E::Desc &fd, int nxh, int H, int RB) {
    return x_pass_elems<E>(fd, nxh, RB) + (size_t)4 * H * RB;
}

// Components are formed one after another: the three physical velocity rows stay in U, the
// product accumulates in A, and the last product is formed in place in the FFT buffer, at
// the permuted positions where the inverse transform left it, so the forward transform
// starts from permuted input (E::run_perm) and no copy is needed.  Input t+1 is copied into
// S while input t is transformed.
// CRB: the rows per block when fixed at compile time (index arithmetic and the FFT's row offsets
// become constants), else 0 and the runtime RBrt.
template <typename T, class E, int CRB>
__device__ __forceinline__ void x_nonlinear_body(const Geo &g, const typename E::Desc &fd, const XNLArgs &a, int RBrt, uint3 blockIdx) {
    const int RB = CRB ? CRB : RBrt;
    const int lgRB = CRB ? (CRB == 16 ? 4 : CRB == 8 ? 3 : CRB == 4 ? 2 : CRB == 2 ? 1 : 0) : lg2(RBrt);
    using V = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int H = g.H, L = fd.L, nxh = g.nxh, SP = RB + 1;
    V *X = (V *)smem_raw;
    V *Y = X + (size_t)L * RB;
    V *S = X + (size_t)E::kBuffers * L * RB;   // nxh x SP spectral row staging
    V *U = S + (size_t)nxh * SP;               // 3 x H x RB physical velocity rows
    V *A = U + (size_t)3 * H * RB;             // H x RB accumulator
    const int nc = a.c1 - a.c0;
    const int row0 = blockIdx.x * RB, nrows = a.nrows * g.ny;
    const int nv = min(RB, nrows - row0);
    const int T_in = 3 + 3 * nc;
    const T tmp = pick<T>(a.tmp, a.tmp_f);
    const size_t off = (size_t)row0 * g.ldx;
    int term, i;
    rows_load_async(S, xnl_input<T>(a, 0, term, i) + off, (unsigned)g.ldx, nxh, RB, nv, SP);
    for (int t = 0; t < T_in; t++) {
        xnl_input<T>(a, t, term, i);
        async_wait();
        __syncthreads();  // S holds input t; the previous iteration is complete
        c2r_pre<T>(g, S, X, RB, SP, term == 0);
        __syncthreads();  // S is free
        if (term != 2 && t + 1 < T_in) {
            int tn, in_;
            rows_load_async(S, xnl_input<T>(a, t + 1, tn, in_) + off, (unsigned)g.ldx, nxh, RB, nv, SP);
        }
        V *R = E::run(X, Y, RB, fd, +1);
        // output m of R sits at row E::pos(m); m advances by D per iteration, so the row
        // advances by a constant when the engine's permutation is affine along that stride
        const int D = blockDim.x >> lgRB, ps = E::pos_stride(D, fd), r0 = threadIdx.x & (RB - 1);
        if (term < 2) {
            int q = E::pos(threadIdx.x >> lgRB, fd) * RB + r0;
            for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x, q += ps * RB) {
                if (ps < 0) q = E::pos(idx >> lgRB, fd) * RB + r0;
                const V p = R[q];
                if (term < 0) {
                    U[i * H * RB + idx] = p;
                } else if (term == 0) {
                    const V u = U[idx];
                    A[idx] = mk<T>(u.x * p.x, u.y * p.y);
                } else {
                    const V u = U[H * RB + idx];
                    A[idx] = mk<T>(A[idx].x + u.x * p.x, A[idx].y + u.y * p.y);
                }
            }
        } else {
            // (acc + u_z d/dz v_i) * tmp in place, forward transform from permuted order, R2C
            int q = E::pos(threadIdx.x >> lgRB, fd) * RB + r0;
            for (int idx = threadIdx.x; idx < H * RB; idx += blockDim.x, q += ps * RB) {
                if (ps < 0) q = E::pos(idx >> lgRB, fd) * RB + r0;
                const V u = U[2 * H * RB + idx], p = R[q], acc = A[idx];
                R[q] = mk<T>((acc.x + u.x * p.x) * tmp, (acc.y + u.y * p.y) * tmp);
            }
            __syncthreads();
            V *Z = E::run_perm(R, R == X ? Y : X, RB, fd, -1);
            r2c_post<T, E, true>(g, fd, Z, S, RB, SP);
            __syncthreads();
            rows_store((V *)a.out[i] + off, (unsigned)g.ldx, S, nxh, SP, nv);
            if (t + 1 < T_in) {
                __syncthreads();
                int tn, in_;
                rows_load_async(S, xnl_input<T>(a, t + 1, tn, in_) + off, (unsigned)g.ldx, nxh, RB, nv, SP);
            }
        }
    }
}
template <typename T, class E, int CRB = 0>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_x_nonlinear(Geo g, typename E::Desc fd, XNLArgs a, int RBrt) {
    if constexpr (E::kBuffers == 1 && CRB != 0 && sizeof(T) == 4) {
        x_nonlinear_pipe<T, E, CRB>(g, fd, a);  // four-step engine, FP32, fixed row count
    } else {
        x_nonlinear_body<T, E, CRB>(g, fd, a, RBrt, blockIdx);
    }
}

// ---------------------------------------------------------------------------------
// Batched launches (batch.h): one launch runs the blocks of several solvers' launches of the
// same kernel; flat block b belongs to the record with the largest block0 <= b, and runs the
// kernel body with that record's arguments and its instance-local block index.
// ---------------------------------------------------------------------------------
template <class Rec>
__device__ __forceinline__ const Rec &batch_rec(const Rec *recs, int n, uint3 &bid) {
    int lo = 0, hi = n - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (recs[mid].grid.block0 <= b) lo = mid;
        else hi = mid - 1;
    }
    const Rec &r = recs[lo];
    const int l = b - r.grid.block0;
    bid = make_uint3((unsigned)(l % r.grid.nbx), (unsigned)((l / r.grid.nbx) % r.grid.nby),
                     (unsigned)(l / (r.grid.nbx * r.grid.nby)));
    return r;
}

// the arguments of one pass launch (grid first: batch_add reads it)
template <class E, class Args>
struct PassRec {
    BatchGrid grid;
    Geo g;
    typename E::Desc fd;
    Args a;
    int tk;
};

template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_z_inverse_batch(const PassRec<E, ZInvArgs> *recs, int n) {
    uint3 bid;
    const PassRec<E, ZInvArgs> &r = batch_rec(recs, n, bid);
    z_inverse_body<T, E, 0>(r.g, r.fd, r.a, r.tk, bid);
}
template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_y_pass_batch(const PassRec<E, YArgs> *recs, int n) {
    uint3 bid;
    const PassRec<E, YArgs> &r = batch_rec(recs, n, bid);
    y_pass_body<T, E, 0>(r.g, r.fd, r.a, r.tk, bid);
}
template <typename T, class E>
__global__ void __launch_bounds__(kThreads, E::kMinBlocks) k_x_nonlinear_batch(const PassRec<E, XNLArgs> *recs, int n) {
    uint3 bid;
    const PassRec<E, XNLArgs> &r = batch_rec(recs, n, bid);
    x_nonlinear_body<T, E, 0>(r.g, r.fd, r.a, r.tk, bid);
}

// host: the launch of a batched kernel over n records and `blocks` blocks in all
template <class Rec, auto Kern, int NT>
void batch_launch(const void *recs, int n, int blocks, size_t smem, cudaStream_t s, bool setup_only) {
    batch_launch_impl<Rec>(Kern, recs, n, blocks, smem, NT, s, setup_only);
}

}  // namespace sg
