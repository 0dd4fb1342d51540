// Batched shared-memory FFT engine (device side).
//
// A thread block transforms B columns at once.  Column c, element k lives at
// buf[k*B + c] (element-major, column fastest), so that consecutive threads
// touch consecutive words.  Lengths factor into radices 2,3,4,5,7,8,11,13 and
// are evaluated by the Stockham autosort scheme (ping-pong between two smem
// buffers, no bit reversal); any other length runs Bluestein's chirp-z
// algorithm over a {2,3,5}-smooth padded length M >= 2n-1.  The transform is
// the unnormalised DFT  X_j = sum_k x_k exp(sign*2*pi*i*j*k/n)  used by FFTW.
#pragma once

#include "common.cuh"

namespace sg {

constexpr int kMaxStages = 16;

struct FFTDesc {
    int n;      // logical length
    int L;      // working length: n, or the Bluestein length M
    int nst;    // Stockham stages over L
    int blue;   // 1 when Bluestein is used
    int radix[kMaxStages];
    const void *tw;     // C2<T>[L]  exp(-2*pi*i*t/L)
    const void *chirp;  // C2<T>[n]  exp(-i*pi*k^2/n)
    const void *filtf;  // C2<T>[L]  FFT_L of the forward chirp filter, times 1/L
    const void *filtb;  // same for the backward sign
};

template <typename T>
__device__ __forceinline__ C2<T> tw_at(const C2<T> *tw, int t, int sign) {
    C2<T> w = ldg_v(tw + t);
    if (sign > 0) w.y = -w.y;
    return w;
}

template <typename T, int R>
__device__ __forceinline__ void butterfly(C2<T> *a, int s, const C2<T> *tw, int LoverR) {
    using V = C2<T>;
    if constexpr (R == 2) {
        V t = a[0];
        a[0] = cadd(t, a[1]);
        a[1] = csub(t, a[1]);
    } else if constexpr (R == 3) {
        constexpr T k3 = T(0.86602540378443864676372317075294), half = T(0.5);
        const T s3 = s * k3;
        V t1 = cadd(a[1], a[2]);
        V t2 = cmuli(cscale(csub(a[1], a[2]), s3), 1);
        V m1 = mk<T>(a[0].x - half * t1.x, a[0].y - half * t1.y);
        a[0] = cadd(a[0], t1);
        a[1] = cadd(m1, t2);
        a[2] = csub(m1, t2);
    } else if constexpr (R == 4) {
        V t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]);
        V t2 = cadd(a[1], a[3]), t3 = cmuli(csub(a[1], a[3]), s);
        a[0] = cadd(t0, t2); a[2] = csub(t0, t2);
        a[1] = cadd(t1, t3); a[3] = csub(t1, t3);
    } else if constexpr (R == 5) {
        constexpr T c1 = T(0.30901699437494742410229341718282), c2 = T(-0.80901699437494742410229341718282);
        constexpr T s1 = T(0.95105651629515357211643933337938), s2 = T(0.58778525229247312916870595463907);
        V t1 = cadd(a[1], a[4]), t2 = cadd(a[2], a[3]);
        V t3 = csub(a[1], a[4]), t4 = csub(a[2], a[3]);
        V m1 = mk<T>(a[0].x + c1 * t1.x + c2 * t2.x, a[0].y + c1 * t1.y + c2 * t2.y);
        V m2 = mk<T>(a[0].x + c2 * t1.x + c1 * t2.x, a[0].y + c2 * t1.y + c1 * t2.y);
        V n1 = cmuli(mk<T>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y), s);
        V n2 = cmuli(mk<T>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y), s);
        a[0] = cadd(a[0], cadd(t1, t2));
        a[1] = cadd(m1, n1); a[4] = csub(m1, n1);
        a[2] = cadd(m2, n2); a[3] = csub(m2, n2);
    } else if constexpr (R == 8) {
        constexpr T h = T(0.70710678118654752440084436210485);
        V e[4] = {a[0], a[2], a[4], a[6]}, o[4] = {a[1], a[3], a[5], a[7]};
        butterfly<T, 4>(e, s, tw, LoverR);
        butterfly<T, 4>(o, s, tw, LoverR);
        // o_r *= w8^r, w8 = (1 + s i)/sqrt2
        o[1] = mk<T>(h * (o[1].x - s * o[1].y), h * (o[1].y + s * o[1].x));
        o[2] = cmuli(o[2], s);
        o[3] = mk<T>(h * (-o[3].x - s * o[3].y), h * (-o[3].y + s * o[3].x));
#pragma unroll
        for (int r = 0; r < 4; r++) { a[r] = cadd(e[r], o[r]); a[r + 4] = csub(e[r], o[r]); }
    } else {
        // direct radix-R DFT: exp(s*2*pi*i*m/R) = tw[m*(L/R)]
        V b[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            V acc = a[0];
#pragma unroll
            for (int q = 1; q < R; q++) acc = cadd(acc, cmul(a[q], tw_at<T>(tw, ((q * r) % R) * LoverR, s)));
            b[r] = acc;
        }
#pragma unroll
        for (int r = 0; r < R; r++) a[r] = b[r];
    }
}

template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const C2<T> *__restrict__ X, C2<T> *__restrict__ Y, int B, int L,
                                               int Ns, int sign, const C2<T> *tw) {
    const int nR = L / R, step = L / (Ns * R);
    const int total = B * nR, lgB = lg2(B);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int c = idx & (B - 1), j = idx >> lgB;
        const int k = j % Ns;
        C2<T> a[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            a[q] = X[(j + q * nR) * B + c];
            if (q && k) a[q] = cmul(a[q], tw_at<T>(tw, q * k * step, sign));
        }
        butterfly<T, R>(a, sign, tw, nR);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; q++) Y[(base + q * Ns) * B + c] = a[q];
    }
}

// Stockham FFT of length d.L over B columns; returns the buffer that holds the result.
template <typename T>
__device__ __noinline__ C2<T> *stockham(C2<T> *X, C2<T> *Y, int B, const FFTDesc &d, int sign) {
    const C2<T> *tw = (const C2<T> *)d.tw;
    int Ns = 1;
    for (int s = 0; s < d.nst; s++) {
        const int R = d.radix[s];
        switch (R) {
        case 2: stockham_stage<T, 2>(X, Y, B, d.L, Ns, sign, tw); break;
        case 3: stockham_stage<T, 3>(X, Y, B, d.L, Ns, sign, tw); break;
        case 4: stockham_stage<T, 4>(X, Y, B, d.L, Ns, sign, tw); break;
        case 5: stockham_stage<T, 5>(X, Y, B, d.L, Ns, sign, tw); break;
        case 7: stockham_stage<T, 7>(X, Y, B, d.L, Ns, sign, tw); break;
        case 8: stockham_stage<T, 8>(X, Y, B, d.L, Ns, sign, tw); break;
        case 11: stockham_stage<T, 11>(X, Y, B, d.L, Ns, sign, tw); break;
        case 13: stockham_stage<T, 13>(X, Y, B, d.L, Ns, sign, tw); break;
        default: break;
        }
        __syncthreads();
        Ns *= R;
        C2<T> *t = X; X = Y; Y = t;
    }
    return X;
}

// Full transform of rows [0, d.n) held in X (B columns).  X and Y must each hold d.L*B
// elements.  Returns the buffer (X or Y) that holds the n outputs in rows [0, n).
// Callers __syncthreads() after filling X; the result is visible to all threads on return.
template <typename T>
__device__ __noinline__ C2<T> *fft_exec(C2<T> *X, C2<T> *Y, int B, const FFTDesc &d, int sign) {
    if (!d.blue) return stockham<T>(X, Y, B, d, sign);
    const C2<T> *chirp = (const C2<T> *)d.chirp;
    const C2<T> *filt = (const C2<T> *)(sign < 0 ? d.filtf : d.filtb);
    const int n = d.n, L = d.L, lgB = lg2(B);
    for (int idx = threadIdx.x; idx < L * B; idx += blockDim.x) {
        const int k = idx >> lgB;
        if (k < n) X[idx] = cmul(X[idx], tw_at<T>(chirp, k, sign));
        else X[idx] = mk<T>(0, 0);
    }
    __syncthreads();
    C2<T> *R = stockham<T>(X, Y, B, d, -1);
    for (int idx = threadIdx.x; idx < L * B; idx += blockDim.x) R[idx] = cmul(R[idx], ldg_v(filt + (idx >> lgB)));
    __syncthreads();
    C2<T> *O = (R == X) ? Y : X;
    R = stockham<T>(R, O, B, d, +1);
    for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) R[idx] = cmul(R[idx], tw_at<T>(chirp, idx >> lgB, sign));
    __syncthreads();
    return R;
}

}  // namespace sg
