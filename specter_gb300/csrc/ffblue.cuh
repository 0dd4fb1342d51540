// Float-float Bluestein z transform for the headline z length (device side).
//
// The precision form keeps the state in float-float (ff.cuh) and transforms its z columns
// (n = nz + C = 538 = 2 * 269 points) by Bluestein's algorithm over L = 1080 = 8 * 15 * 9.  The
// generic engine (fft.cuh) spends one shared-memory pass, one barrier and one global table load
// per element for each of its 2 x 5 radix stages and 3 pointwise passes.  Here the length-L
// convolution runs as five register steps with one barrier each, in place in one buffer:
//
//   A   thread (col, n' = n3 + 9 n2): x[n' + 135 n1], n1 < 4 (the rest is Bluestein's zero
//       padding), times the chirp; DFT_8 over n1; times w_120^(n2 k1)       -> row n' + 135 k1
//   B   thread (col, k1, n3): rows n3 + 9 n2 + 135 k1, n2 < 15; DFT_15;
//       times w_1080^(n3 (k1 + 8 k2))                                       -> row n3 + 9 k2 + 135 k1
//   C   thread (col, k1, k2): the 9 contiguous rows 9 k2 + 135 k1 + n3; DFT_9 gives frequency
//       k1 + 8 k2 + 120 k3; times the filter; inverse DFT_9; times w_1080^(-m3 (k1 + 8 k2))
//   B'  inverse DFT_15 over k2; times w_120^(-m2 k1)
//   A'  inverse DFT_8 over k1: output m = m3 + 9 m2 + 135 m1 in natural order; times the chirp
//
// (the three-factor form of the four-step split: X[k1 + L1 k2 + L1 L2 k3] with
// n = n3 + L3 n2 + L2 L3 n1 needs the twiddles w_{L1 L2}^{n2 k1} after the first step and
// w_L^{n3 (k1 + L1 k2)} after the second; the inverse runs the transposed sequence).  As in the
// FP32 engine (fft4.cuh) only the inverse transform's chirp and filter are stored, and the forward
// transform is conj(inverse(conj x)), the conjugations folded into the chirp multiplies.
//
// The register DFTs are written for float-float, where an addition (TwoSum, 8 flops) costs twice
// a product by a constant (4 flops, ff_mulc): DFT_3 and DFT_5 use the forms with the fewest
// additions (the DFT_5 pair (c1 + c2)/2 = -1/4, (c1 - c2)/2 = sqrt(5)/4), scalings by 1/2 and
// 1/4 are exact, DFT_15 is the prime-factor (Good-Thomas) 5 x 3 form without twiddles, DFT_9 the
// 3 x 3 Cooley-Tukey form with four constant twiddles, DFT_8 two DFT_4 and the w_8 rotations.
//
// Tables (FFBTab, ffc units): twiddles, chirp and filter, 45.5 KB per length, read through the
// read-only cache (a copy staged in shared memory measured no faster).  Any n <= L/2 = 540 runs
// on the same split; the plans use it for 270 < n <= 540.
#pragma once

#include "common.cuh"

namespace sg {

// table layout (ffc units); padded strides keep the rows of neighbouring threads in different
// shared-memory banks
struct FFBTab {
    static constexpr int L1 = 8, L2 = 15, L3 = 9, L = L1 * L2 * L3, M = L2 * L3, J = L1 * L2;
    static constexpr int kMaxN = L / 2;               // Bluestein bound n <= L/2 (zero half of step A)
    static constexpr int kTw1S = 9;                   // tw1[n2][k1] = w_120^(n2 k1), n2 < 15, k1 < 8
    static constexpr int kTw2S = 121;                 // tw2[n3][j]  = w_1080^(n3 j), n3 < 9, j < 120
    static constexpr int kOffTw1 = 0;
    static constexpr int kOffTw2 = kOffTw1 + L2 * kTw1S;
    static constexpr int kOffChirp = kOffTw2 + L3 * kTw2S;   // exp(+i pi k^2 / n), k < n
    static constexpr int kOffFilt = kOffChirp + kMaxN;      // filt[j][k3], j = k1 * 15 + k2
    static constexpr int kLen = kOffFilt + J * L3;
    static constexpr int kBytes = kLen * 16;
};

struct FFBDesc {
    int n, L, blue;   // L: rows of the kernels' FFT buffer (>= the transform's 1080)
    const ffc *tab;   // FFBTab::kLen entries (global memory, or shared once staged)
    const ffc *ztab;  // wall round trips as window corrections (ffzoom.cuh), or null
    int zj0;          // first window row (nzp - d)
};

namespace ffb {

using Q = ffc;

// a * c for a constant c: exact leading product, cross terms in the error word, no
// renormalisation (the additions that follow take unnormalised pairs)
__device__ __forceinline__ ff mulc(ff a, ff c) {
    const float p = a.hi * c.hi;
    float e = fmaf(a.hi, c.hi, -p);
    e = fmaf(a.hi, c.lo, e);
    e = fmaf(a.lo, c.hi, e);
    return ff(p, e);
}
__device__ __forceinline__ Q qadd(Q a, Q b) { Q r; r.x = ff_add(a.x, b.x); r.y = ff_add(a.y, b.y); return r; }
__device__ __forceinline__ Q qsub(Q a, Q b) { Q r; r.x = ff_sub(a.x, b.x); r.y = ff_sub(a.y, b.y); return r; }
__device__ __forceinline__ Q qmc(Q a, ff c) { Q r; r.x = mulc(a.x, c); r.y = mulc(a.y, c); return r; }
// exact scaling by a power of two
__device__ __forceinline__ Q qpow2(Q a, float s) {
    Q r;
    r.x = ff(a.x.hi * s, a.x.lo * s);
    r.y = ff(a.y.hi * s, a.y.lo * s);
    return r;
}
// i * S * a, S = +-1 (exact)
template <int S>
__device__ __forceinline__ Q qi(Q a) {
    Q r;
    if constexpr (S > 0) { r.x = ff_neg(a.y); r.y = a.x; }
    else { r.x = a.y; r.y = ff_neg(a.x); }
    return r;
}
__device__ __forceinline__ Q qconj(Q a) { a.y = ff_neg(a.y); return a; }
// Complex products by the twiddles, chirp and filter (ff.cuh ff_dot2: exact leading products,
// one TwoSum, renormalised).  These are where a step's values are stored, so renormalising here
// bounds the growth of the unnormalised error words along the additions of the next DFT (without
// it the transforms measured 2.5e-14 instead of 1.1e-14 against a long-double DFT).
__device__ __forceinline__ Q qmul(Q a, Q b) { return cmul(a, b); }
// a * conj(b)
__device__ __forceinline__ Q qmulc(Q a, Q b) {
    Q r;
    r.x = ff_dot2(a.x, b.x, a.y, b.y);
    r.y = ff_dot2(a.y, b.x, ff_neg(a.x), b.y);
    return r;
}
__device__ __forceinline__ Q qzero() { Q r; r.x = ff(0.f, 0.f); r.y = ff(0.f, 0.f); return r; }

// ---- register DFTs, X_k = sum_j a_j exp(S 2 pi i j k / N) --------------------------------------
constexpr ff kK3(0.8660254037844386);    // sqrt(3)/2
constexpr ff kK54(0.5590169943749475);   // sqrt(5)/4 = (cos(2 pi/5) - cos(4 pi/5)) / 2
constexpr ff kS51(0.9510565162951535);   // sin(2 pi/5)
constexpr ff kS52(0.5877852522924732);   // sin(4 pi/5)
constexpr ff kH(0.7071067811865476);     // sqrt(1/2)
constexpr ff kC91(0.766044443118978), kS91(0.6427876096865393);     // w_9
constexpr ff kC92(0.17364817766693041), kS92(0.984807753012208);    // w_9^2
constexpr ff kC94(-0.9396926207859083), kS94(0.3420201433256689);   // w_9^4

template <int S>
__device__ __forceinline__ void dft3(Q &a0, Q &a1, Q &a2) {
    const Q t = qadd(a1, a2), d = qsub(a1, a2);
    const Q m = qsub(a0, qpow2(t, 0.5f));
    a0 = qadd(a0, t);
    const Q r = qmc(qi<S>(d), kK3);
    a1 = qadd(m, r);
    a2 = qsub(m, r);
}
template <int S>
__device__ __forceinline__ void dft4(Q &a0, Q &a1, Q &a2, Q &a3) {
    const Q t0 = qadd(a0, a2), t1 = qsub(a0, a2), t2 = qadd(a1, a3), t3 = qi<S>(qsub(a1, a3));
    a0 = qadd(t0, t2);
    a2 = qsub(t0, t2);
    a1 = qadd(t1, t3);
    a3 = qsub(t1, t3);
}
template <int S>
__device__ __forceinline__ void dft5(Q &a0, Q &a1, Q &a2, Q &a3, Q &a4) {
    const Q t1 = qadd(a1, a4), t2 = qadd(a2, a3), t3 = qsub(a1, a4), t4 = qsub(a2, a3);
    const Q u = qadd(t1, t2), v = qsub(t1, t2);
    const Q b = qsub(a0, qpow2(u, 0.25f));
    a0 = qadd(a0, u);
    const Q dv = qmc(v, kK54);
    const Q m1 = qadd(b, dv), m2 = qsub(b, dv);
    const Q n1 = qi<S>(qadd(qmc(t3, kS51), qmc(t4, kS52)));
    const Q n2 = qi<S>(qsub(qmc(t3, kS52), qmc(t4, kS51)));
    a1 = qadd(m1, n1);
    a4 = qsub(m1, n1);
    a2 = qadd(m2, n2);
    a3 = qsub(m2, n2);
}
// w_8^(S k) rotations of the odd half
template <int S>
__device__ __forceinline__ void rot8(Q &o1, Q &o2, Q &o3) {
    o1 = qmc(qadd(o1, qi<S>(o1)), kH);                 // (1 + S i) / sqrt 2
    o2 = qi<S>(o2);
    o3 = qmc(qsub(qi<S>(o3), o3), kH);                 // (-1 + S i) / sqrt 2
}
template <int S>
__device__ __forceinline__ void dft8(Q (&a)[8]) {
    Q e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6], o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
    dft4<S>(e0, e1, e2, e3);
    dft4<S>(o0, o1, o2, o3);
    rot8<S>(o1, o2, o3);
    a[0] = qadd(e0, o0); a[4] = qsub(e0, o0);
    a[1] = qadd(e1, o1); a[5] = qsub(e1, o1);
    a[2] = qadd(e2, o2); a[6] = qsub(e2, o2);
    a[3] = qadd(e3, o3); a[7] = qsub(e3, o3);
}
// DFT_8 of a[0..3] with a[4..7] = 0 (not read)
template <int S>
__device__ __forceinline__ void dft8_hz(Q (&a)[8]) {
    const Q x0 = a[0], x1 = a[1], x2 = a[2], x3 = a[3];
    const Q ix2 = qi<S>(x2), ix3 = qi<S>(x3);
    const Q e0 = qadd(x0, x2), e1 = qadd(x0, ix2), e2 = qsub(x0, x2), e3 = qsub(x0, ix2);
    Q o0 = qadd(x1, x3), o1 = qadd(x1, ix3), o2 = qsub(x1, x3), o3 = qsub(x1, ix3);
    rot8<S>(o1, o2, o3);
    a[0] = qadd(e0, o0); a[4] = qsub(e0, o0);
    a[1] = qadd(e1, o1); a[5] = qsub(e1, o1);
    a[2] = qadd(e2, o2); a[6] = qsub(e2, o2);
    a[3] = qadd(e3, o3); a[7] = qsub(e3, o3);
}
// DFT_9 = 3 x 3: DFT_3 over p of a[3p + q], twiddle w_9^(S q r), DFT_3 over q -> X[r + 3 s]
template <int S>
__device__ __forceinline__ void dft9(Q (&a)[9]) {
#pragma unroll
    for (int q = 0; q < 3; q++) dft3<S>(a[q], a[3 + q], a[6 + q]);
    // a[3 r + q] now holds Y[q][r]
    Q w1, w2, w4;
    w1.x = kC91; w1.y = S > 0 ? kS91 : ff_neg(kS91);
    w2.x = kC92; w2.y = S > 0 ? kS92 : ff_neg(kS92);
    w4.x = kC94; w4.y = S > 0 ? kS94 : ff_neg(kS94);
    a[4] = qmul(a[4], w1);  // q = 1, r = 1
    a[7] = qmul(a[7], w2);  // q = 1, r = 2
    a[5] = qmul(a[5], w2);  // q = 2, r = 1
    a[8] = qmul(a[8], w4);  // q = 2, r = 2
    Q y[9];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        Q b0 = a[3 * r], b1 = a[3 * r + 1], b2 = a[3 * r + 2];
        dft3<S>(b0, b1, b2);
        y[r] = b0;
        y[r + 3] = b1;
        y[r + 6] = b2;
    }
#pragma unroll
    for (int i = 0; i < 9; i++) a[i] = y[i];
}
// DFT_15, prime-factor 5 x 3: input a[(3 n1 + 5 n2) mod 15], output k = (6 k1 + 10 k2) mod 15
template <int S>
__device__ __forceinline__ void dft15(Q (&a)[15]) {
    Q y[5][3];
#pragma unroll
    for (int n1 = 0; n1 < 5; n1++)
#pragma unroll
        for (int n2 = 0; n2 < 3; n2++) y[n1][n2] = a[(3 * n1 + 5 * n2) % 15];
#pragma unroll
    for (int n1 = 0; n1 < 5; n1++) dft3<S>(y[n1][0], y[n1][1], y[n1][2]);
#pragma unroll
    for (int k2 = 0; k2 < 3; k2++) {
        Q c0 = y[0][k2], c1 = y[1][k2], c2 = y[2][k2], c3 = y[3][k2], c4 = y[4][k2];
        dft5<S>(c0, c1, c2, c3, c4);
        a[(10 * k2) % 15] = c0;
        a[(6 + 10 * k2) % 15] = c1;
        a[(12 + 10 * k2) % 15] = c2;
        a[(18 + 10 * k2) % 15] = c3;
        a[(24 + 10 * k2) % 15] = c4;
    }
}

__device__ __forceinline__ Q tab_ld(const Q *p) { return ldg_v(p); }

constexpr int ct_log2(int b) { return b <= 1 ? 0 : 1 + ct_log2(b / 2); }

// Bluestein transform of the n natural rows of X (TK columns, X[row * TK + col]); rows [n, L) are
// scratch.  sign > 0: X_j = sum_k x_k exp(+2 pi i j k / n) (z-inverse); sign < 0: the forward
// transform.  NT threads run the block's loops; the tables are read through the read-only cache.
// Barriers: one after each step; the caller syncs after filling X.
template <int TK, int NT>
__device__ __forceinline__ void bluestein(Q *X, const Q *tab, int n, int sign) {
    using T = FFBTab;
    constexpr int lgTK = ct_log2(TK);
    const Q *tw1 = tab + T::kOffTw1, *tw2 = tab + T::kOffTw2, *chirp = tab + T::kOffChirp, *filt = tab + T::kOffFilt;
    const bool fwd = sign < 0;
    // step A: chirp, DFT_8 over n1 (upper half zero), w_120^(n2 k1)
    for (int idx = threadIdx.x; idx < TK * T::M; idx += NT) {
        const int c = idx & (TK - 1), np = idx >> lgTK;
        const int n2 = np / T::L3;
        Q a[8];
#pragma unroll
        for (int n1 = 0; n1 < 4; n1++) {
            const int row = np + T::M * n1;
            if (row < n) {
                Q x = X[row * TK + c];
                if (fwd) x = qconj(x);
                a[n1] = qmul(x, tab_ld(chirp + row));
            } else {
                a[n1] = qzero();
            }
        }
        dft8_hz<-1>(a);
#pragma unroll
        for (int k1 = 1; k1 < 8; k1++) a[k1] = qmul(a[k1], tab_ld(tw1 + n2 * T::kTw1S + k1));
#pragma unroll
        for (int k1 = 0; k1 < 8; k1++) X[(np + T::M * k1) * TK + c] = a[k1];
    }
    __syncthreads();
    // step B: DFT_15 over n2, w_1080^(n3 (k1 + 8 k2))
    for (int idx = threadIdx.x; idx < TK * T::L1 * T::L3; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L3, n3 = j - T::L3 * k1;
        const int base = n3 + T::M * k1;
        Q b[15];
#pragma unroll
        for (int n2 = 0; n2 < 15; n2++) b[n2] = X[(base + T::L3 * n2) * TK + c];
        dft15<-1>(b);
        const Q *tw = tw2 + n3 * T::kTw2S + k1;
#pragma unroll
        for (int k2 = 0; k2 < 15; k2++) X[(base + T::L3 * k2) * TK + c] = qmul(b[k2], tab_ld(tw + T::L1 * k2));
    }
    __syncthreads();
    // step C: DFT_9 over n3, filter, inverse DFT_9, w_1080^(-m3 (k1 + 8 k2))
    for (int idx = threadIdx.x; idx < TK * T::J; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L2, k2 = j - T::L2 * k1;
        const int base = T::L3 * k2 + T::M * k1;
        Q d[9];
#pragma unroll
        for (int n3 = 0; n3 < 9; n3++) d[n3] = X[(base + n3) * TK + c];
        // DFT_9, filter, inverse DFT_9 with one DFT_9 body (the inverse is conj(DFT_9(conj x))):
        // half the instruction footprint of the step
        const Q *fl = filt + j * T::L3;
#pragma unroll 1
        for (int pass = 0; pass < 2; pass++) {
            dft9<-1>(d);
            if (pass == 0) {
#pragma unroll
                for (int k3 = 0; k3 < 9; k3++) d[k3] = qconj(qmul(d[k3], tab_ld(fl + k3)));
            }
        }
        const Q *tw = tw2 + k1 + T::L1 * k2;
        X[base * TK + c] = qconj(d[0]);
#pragma unroll
        for (int m3 = 1; m3 < 9; m3++) X[(base + m3) * TK + c] = qconj(qmul(d[m3], tab_ld(tw + m3 * T::kTw2S)));
    }
    __syncthreads();
    // step B': inverse DFT_15 over k2, w_120^(-m2 k1)
    for (int idx = threadIdx.x; idx < TK * T::L1 * T::L3; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L3, m3 = j - T::L3 * k1;
        const int base = m3 + T::M * k1;
        Q b[15];
#pragma unroll
        for (int k2 = 0; k2 < 15; k2++) b[k2] = X[(base + T::L3 * k2) * TK + c];
        dft15<+1>(b);
        X[base * TK + c] = b[0];
#pragma unroll
        for (int m2 = 1; m2 < 15; m2++) X[(base + T::L3 * m2) * TK + c] = qmulc(b[m2], tab_ld(tw1 + m2 * T::kTw1S + k1));
    }
    __syncthreads();
    // step A': inverse DFT_8 over k1 -> m = m' + 135 m1 (natural), chirp; rows >= n are dropped
    for (int idx = threadIdx.x; idx < TK * T::M; idx += NT) {
        const int c = idx & (TK - 1), mp = idx >> lgTK;
        Q a[8];
#pragma unroll
        for (int k1 = 0; k1 < 8; k1++) a[k1] = X[(mp + T::M * k1) * TK + c];
        dft8<+1>(a);
#pragma unroll
        for (int m1 = 0; m1 < 4; m1++) {
            const int row = mp + T::M * m1;
            if (row < n) {
                Q o = qmul(a[m1], tab_ld(chirp + row));
                if (fwd) o = qconj(o);
                X[row * TK + c] = o;
            }
        }
    }
    __syncthreads();
}

// One out-of-line copy per tile width: the column kernels transform at several call sites.
template <int TK, int NT>
__device__ __noinline__ void run_out(Q *X, const Q *tab, int n, int sign) {
    bluestein<TK, NT>(X, tab, n, sign);
}

}  // namespace ffb

}  // namespace sg
