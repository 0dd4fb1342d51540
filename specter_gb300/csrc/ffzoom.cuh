// Wall round trips of the float-float column kernels as spectral corrections (device side).
//
// A round trip of the fused stage -- z-inverse, new values on the wall rows (no-slip, the scalar's
// Dirichlet walls), continuation rows rebuilt from the 2d wall-adjacent rows, z-forward -- changes
// the physical column only on the window of M = C + 2d rows that starts d rows below the top wall
// and wraps round to d rows above the bottom one (rows nzp-d .. n-1 and 0 .. d-1, contiguous
// modulo n).  With u = IFFT(u^)/n and u' = u + delta (delta zero outside the window), the forward
// transform of u' is exactly u^ + FFT(delta).  So a round trip needs
//   (1) the M window values of the inverse transform of the spectrum, and
//   (2) the forward transform of an M-point window,
// and both are chirp-z transforms (Bluestein 1970 / Rabiner et al. 1969): with
// c_k = exp(+i pi k^2 / n) (period n for even n) and jk = (j^2 + k^2 - (j-k)^2)/2,
//   (1) y_{j0+m} = c_{j0+m} sum_k (u^_k c_k) conj(c_{j0+m-k}),         m < M,
//   (2) X_k      = conj(c_k) sum_p (delta_p conj(c_{j0+p})) c_{k-j0-p},  k < n,
// linear convolutions of n and M points that fit a cyclic convolution of L = 576 >= n + M - 1
// (n = 538, M = 35).  Each is one forward and one inverse 576-point transform with the filter
// spectrum in between -- against two 1080-point Bluestein transforms for the plain round trip --
// and the sparse ends trim them further: in (1) only 35 of 576 outputs are needed (the last step
// keeps output 0 of its DFT_8, a sum), in (2) only 35 of 576 inputs are non-zero (the first step
// is one product per output).  The bulk of the spectrum is never transformed, so it also keeps no
// rounding from the round trip.
//
// The 576-point transforms use the three-step register form of ffblue.cuh with
// 576 = 8 x 8 x 9: n = n3 + 9 n2 + 72 n1, k = k1 + 8 k2 + 64 k3, twiddles w_64^(n2 k1) after the
// first step and w_576^(n3 (k1 + 8 k2)) after the second; frequency k sits at row
// k3 + 9 k2 + 72 k1 after the third step, where the filter is applied in registers between
// DFT_9 and its inverse.
#pragma once

#include <cmath>
#include <complex>
#include <vector>

#include "ffblue.cuh"

namespace sg {

struct FFZTab {
    static constexpr int L1 = 8, L2 = 8, L3 = 9, L = L1 * L2 * L3, M = L2 * L3, J = L1 * L2;
    static constexpr int kWin = 35;                   // window rows (C + 2d for C = 25, d = 5)
    static constexpr int kMaxN = L - kWin + 1;        // n + kWin - 1 <= L
    static constexpr int kTw1S = 9;                   // tw1[n2][k1] = w_64^(n2 k1)
    static constexpr int kTw2S = 65;                  // tw2[n3][j]  = w_576^(n3 j), j < 64
    static constexpr int kOffTw1 = 0;
    static constexpr int kOffTw2 = kOffTw1 + L2 * kTw1S;
    static constexpr int kOffChirp = kOffTw2 + L3 * kTw2S;  // c_k = exp(+i pi k^2 / n), k < n
    static constexpr int kOffG = kOffChirp + kMaxN;         // (1): FFT_L(g) / L at [j][k3], j = k1 * 8 + k2
    static constexpr int kOffH = kOffG + J * L3;            // (2): FFT_L(h) / L
    static constexpr int kLen = kOffH + J * L3;
    static constexpr int kBytes = kLen * 16;
};

namespace ffz {

using namespace ffb;
using T = FFZTab;

__device__ __forceinline__ Q ldq(const Q *p) { return ldg_v(p); }

// the forward steps B and C (with the filter) and the inverse step C' of a 576-point
// convolution held at W[row * TK + col]; B_HZ: only rows with n3 + 9 n2 < 36 are non-zero
template <int TK, int NT, bool B_HZ>
__device__ __forceinline__ void steps_bcc(Q *W, const Q *tab, const Q *filt) {
    constexpr int lgTK = ct_log2(TK);
    const Q *tw2 = tab + T::kOffTw2;
    for (int idx = threadIdx.x; idx < TK * T::L1 * T::L3; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L3, n3 = j - T::L3 * k1;
        const int base = n3 + T::M * k1;
        Q b[8];
        if constexpr (B_HZ) {
#pragma unroll
            for (int n2 = 0; n2 < 4; n2++) b[n2] = W[(base + T::L3 * n2) * TK + c];
            dft8_hz<-1>(b);
        } else {
#pragma unroll
            for (int n2 = 0; n2 < 8; n2++) b[n2] = W[(base + T::L3 * n2) * TK + c];
            dft8<-1>(b);
        }
        const Q *tw = tw2 + n3 * T::kTw2S + k1;
#pragma unroll
        for (int k2 = 0; k2 < 8; k2++) W[(base + T::L3 * k2) * TK + c] = qmul(b[k2], ldq(tw + T::L1 * k2));
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < TK * T::J; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j >> 3, k2 = j & 7;
        const int base = T::L3 * k2 + T::M * k1;
        Q d[9];
#pragma unroll
        for (int n3 = 0; n3 < 9; n3++) d[n3] = W[(base + n3) * TK + c];
        // DFT_9, filter, inverse DFT_9 with one DFT_9 body (half the instruction footprint of
        // this, the largest step): the inverse is conj(DFT_9(conj x)), so the first pass leaves
        // the conjugated filtered values and the second pass's result is the conjugated inverse
        const Q *fl = filt + j * T::L3;
#pragma unroll 1
        for (int pass = 0; pass < 2; pass++) {
            dft9<-1>(d);
            if (pass == 0) {
#pragma unroll
                for (int k3 = 0; k3 < 9; k3++) d[k3] = qconj(qmul(d[k3], ldq(fl + k3)));
            }
        }
        // inverse output conj(d) times conj(w): conj(d w)
        const Q *tw = tw2 + k1 + T::L1 * k2;
        W[base * TK + c] = qconj(d[0]);
#pragma unroll
        for (int m3 = 1; m3 < 9; m3++) W[(base + m3) * TK + c] = qconj(qmul(d[m3], ldq(tw + m3 * T::kTw2S)));
    }
    __syncthreads();
}

// (1) window values of the unnormalised inverse z transform: Wv[m][col] = sum_k X_k
// exp(+2 pi i (j0 + m) k / n), m < kWin.  X: spectrum rows [0, n); W: scratch [L][TK].
// Barriers: one per step; the caller syncs after filling X, Wv is visible on return.
template <int TK, int NT>
__device__ __forceinline__ void window_values(const Q *X, Q *W, Q *Wv, const Q *tab, int n, int j0) {
    constexpr int lgTK = ct_log2(TK);
    const Q *tw1 = tab + T::kOffTw1, *chirp = tab + T::kOffChirp;
    // A: a_k = X_k c_k (k < n), DFT_8 over n1, w_64^(n2 k1)
    for (int idx = threadIdx.x; idx < TK * T::M; idx += NT) {
        const int c = idx & (TK - 1), np = idx >> lgTK;
        const int n2 = np / T::L3;
        Q a[8];
#pragma unroll
        for (int n1 = 0; n1 < 8; n1++) {
            const int k = np + T::M * n1;
            a[n1] = k < n ? qmul(X[k * TK + c], ldq(chirp + k)) : qzero();
        }
        dft8<-1>(a);
        W[np * TK + c] = a[0];
#pragma unroll
        for (int k1 = 1; k1 < 8; k1++) W[(np + T::M * k1) * TK + c] = qmul(a[k1], ldq(tw1 + n2 * T::kTw1S + k1));
    }
    __syncthreads();
    steps_bcc<TK, NT, false>(W, tab, tab + T::kOffG);
    // B': inverse DFT_8 over k2; only m2 < 4 (rows m3 + 9 m2 < 36) feed the window
    for (int idx = threadIdx.x; idx < TK * T::L1 * T::L3; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L3, m3 = j - T::L3 * k1;
        const int base = m3 + T::M * k1;
        Q b[8];
#pragma unroll
        for (int k2 = 0; k2 < 8; k2++) b[k2] = W[(base + T::L3 * k2) * TK + c];
        dft8<+1>(b);
        W[base * TK + c] = b[0];
#pragma unroll
        for (int m2 = 1; m2 < 4; m2++) W[(base + T::L3 * m2) * TK + c] = qmulc(b[m2], ldq(tw1 + m2 * T::kTw1S + k1));
    }
    __syncthreads();
    // A': output m = m' < kWin is output 0 of the inverse DFT_8 over k1 (the sum), times c_{j0+m}
    for (int idx = threadIdx.x; idx < TK * T::kWin; idx += NT) {
        const int c = idx & (TK - 1), mp = idx >> lgTK;
        Q s = W[mp * TK + c];
#pragma unroll
        for (int k1 = 1; k1 < 8; k1++) s = qadd(s, W[(mp + T::M * k1) * TK + c]);
        int r = j0 + mp;
        if (r >= n) r -= n;
        Wv[mp * TK + c] = qmul(s, ldq(chirp + r));
    }
    __syncthreads();
}

// (2) X_k += sum_p Dv[p] exp(-2 pi i (j0 + p) k / n), k < n: the forward z transform of the
// window corrections added to the spectrum.  W: scratch [L][TK].
template <int TK, int NT>
__device__ __forceinline__ void add_window_transform(Q *X, Q *W, const Q *Dv, const Q *tab, int n, int j0) {
    constexpr int lgTK = ct_log2(TK);
    const Q *tw1 = tab + T::kOffTw1, *chirp = tab + T::kOffChirp;
    // A: input rows p < kWin only (n1 = 0): a'_p = Dv[p] conj(c_{j0+p}); its DFT_8 over n1 is
    // constant, times w_64^(n2 k1)
    for (int idx = threadIdx.x; idx < TK * T::M; idx += NT) {
        const int c = idx & (TK - 1), np = idx >> lgTK;
        if (np < T::kWin) {
            const int n2 = np / T::L3;
            int r = j0 + np;
            if (r >= n) r -= n;
            const Q x = qmulc(Dv[np * TK + c], ldq(chirp + r));
            W[np * TK + c] = x;
#pragma unroll
            for (int k1 = 1; k1 < 8; k1++) W[(np + T::M * k1) * TK + c] = qmul(x, ldq(tw1 + n2 * T::kTw1S + k1));
        } else {
#pragma unroll
            for (int k1 = 0; k1 < 8; k1++) W[(np + T::M * k1) * TK + c] = qzero();
        }
    }
    __syncthreads();
    steps_bcc<TK, NT, true>(W, tab, tab + T::kOffH);
    // B': inverse DFT_8 over k2, w_64^(-m2 k1)
    for (int idx = threadIdx.x; idx < TK * T::L1 * T::L3; idx += NT) {
        const int c = idx & (TK - 1), j = idx >> lgTK;
        const int k1 = j / T::L3, m3 = j - T::L3 * k1;
        const int base = m3 + T::M * k1;
        Q b[8];
#pragma unroll
        for (int k2 = 0; k2 < 8; k2++) b[k2] = W[(base + T::L3 * k2) * TK + c];
        dft8<+1>(b);
        W[base * TK + c] = b[0];
#pragma unroll
        for (int m2 = 1; m2 < 8; m2++) W[(base + T::L3 * m2) * TK + c] = qmulc(b[m2], ldq(tw1 + m2 * T::kTw1S + k1));
    }
    __syncthreads();
    // A': inverse DFT_8 over k1 -> k = m' + 72 m1 < n, times conj(c_k), added to X
    for (int idx = threadIdx.x; idx < TK * T::M; idx += NT) {
        const int c = idx & (TK - 1), mp = idx >> lgTK;
        Q a[8];
#pragma unroll
        for (int k1 = 0; k1 < 8; k1++) a[k1] = W[(mp + T::M * k1) * TK + c];
        dft8<+1>(a);
#pragma unroll
        for (int m1 = 0; m1 < 8; m1++) {
            const int k = mp + T::M * m1;
            if (k < n) X[k * TK + c] = qadd(X[k * TK + c], qmulc(a[m1], ldq(chirp + k)));
        }
    }
    __syncthreads();
}

// out-of-line copies (the column kernels call them at several sites)
template <int TK, int NT>
__device__ __noinline__ void window_values_out(const Q *X, Q *W, Q *Wv, const Q *tab, int n, int j0) {
    window_values<TK, NT>(X, W, Wv, tab, n, j0);
}
template <int TK, int NT>
__device__ __noinline__ void add_window_transform_out(Q *X, Q *W, const Q *Dv, const Q *tab, int n, int j0) {
    add_window_transform<TK, NT>(X, W, Dv, tab, n, j0);
}

}  // namespace ffz

// Engine interface of the fused column kernels (kernels.cuh: GenericFFT, FourStep) for the
// float-float kernels on this transform: one in-place buffer, natural order in and out, tables
// through the read-only cache (measured as fast as staging them in shared memory), NT threads,
// MINB blocks per SM.
template <int NT, int MINB = 1>
struct FFBlue {
    using Desc = FFBDesc;
    static constexpr int kBuffers = 1;
    static constexpr bool kStreamProj = true;  // the projection without staged components
    static constexpr int kProjRows = FFBTab::L;  // its FFT buffer rows (no window scratch)
    static constexpr bool kZoom = true;          // wall round trips by window corrections
    static constexpr int kMinBlocks = MINB;
    static constexpr int kColThreads = NT;
    static constexpr int kWideThreads = NT;
    static int wide_threads(int) { return NT; }
    static __device__ __forceinline__ ffc *run(ffc *X, ffc *, int B, const Desc &d, int sign) {
        if (B == 8) ffb::run_out<8, NT>(X, d.tab, d.n, sign);
        else if (B == 4) ffb::run_out<4, NT>(X, d.tab, d.n, sign);
        else if (B == 2) ffb::run_out<2, NT>(X, d.tab, d.n, sign);
        else ffb::run_out<1, NT>(X, d.tab, d.n, sign);
        return X;
    }
    static __device__ __forceinline__ ffc *run_perm(ffc *X, ffc *Y, int B, const Desc &d, int sign) { return run(X, Y, B, d, sign); }
    // window values (1) and window transform added to the spectrum (2) of ffzoom.cuh; scratch W,
    // window rows Wv / Dv (FFZTab::L and kWin rows of B columns)
    static __device__ __forceinline__ void window(const ffc *X, ffc *W, ffc *Wv, const Desc &d, int B) {
        if (B == 8) ffz::window_values_out<8, NT>(X, W, Wv, d.ztab, d.n, d.zj0);
        else if (B == 4) ffz::window_values_out<4, NT>(X, W, Wv, d.ztab, d.n, d.zj0);
        else if (B == 2) ffz::window_values_out<2, NT>(X, W, Wv, d.ztab, d.n, d.zj0);
        else ffz::window_values_out<1, NT>(X, W, Wv, d.ztab, d.n, d.zj0);
    }
    static __device__ __forceinline__ void window_add(ffc *X, ffc *W, const ffc *Dv, const Desc &d, int B) {
        if (B == 8) ffz::add_window_transform_out<8, NT>(X, W, Dv, d.ztab, d.n, d.zj0);
        else if (B == 4) ffz::add_window_transform_out<4, NT>(X, W, Dv, d.ztab, d.n, d.zj0);
        else if (B == 2) ffz::add_window_transform_out<2, NT>(X, W, Dv, d.ztab, d.n, d.zj0);
        else ffz::add_window_transform_out<1, NT>(X, W, Dv, d.ztab, d.n, d.zj0);
    }
    static __device__ __forceinline__ int pos(int k, const Desc &) { return k; }
    static __device__ __forceinline__ int pos_stride(int D, const Desc &) { return D; }
};

// Host (fused_ffb.cu): the table for z length n and window start j0; empty when n is odd or too
// long for the window convolution.
std::vector<ffc> ffz_table_host(int n, int j0);

}  // namespace sg
