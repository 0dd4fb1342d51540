// Register-resident four-step FFT over shared-memory column tiles (device side).
//
// A length L = L1*L2 transform of B columns held in smem at X[pos*B + col] runs in two
// exchange steps instead of one smem round trip per radix stage:
//   step A  thread (col, n2): loads x[n2 + L2*n1], n1 < L1, does DFT_L1 in registers,
//           multiplies by w_L^{n2*k1}, stores back to the same positions n2 + L2*k1;
//   step B  thread (col, k1): loads the contiguous run L2*k1 + n2, n2 < L2, does DFT_L2 in
//           registers and stores frequency k1 + L1*k2 at position L2*k1 + k2 ("permuted").
// The inverse-order pair (B' then A') takes permuted input to natural output.  Bluestein's
// algorithm fuses as  A (input * chirp) | B, *filter, B' (all in registers) | A' (* chirp):
// two barriers and two smem round trips for a convolution of length L.
//
// Register DFTs are unrolled mixed-radix Stockham sequences with compile-time radices; their
// internal twiddles come from a __constant__ table (uniform address -> constant-bank operand).
// Both tables are filled per translation unit by fft4_init_tables().
#pragma once

#include "common.cuh"
#include "fft.cuh"
#include "plan.h"

namespace sg {

// ---- register DFT sizes served by the constant twiddle table -------------------------------
constexpr int kRegSizes[] = {4, 6, 8, 9, 10, 12, 15, 16, 18, 20, 24, 27, 30, 32, 36, 40, 45, 48, 64};
constexpr int kNumRegSizes = sizeof(kRegSizes) / sizeof(int);
constexpr int reg_offset(int N) {
    int off = 0;
    for (int i = 0; i < kNumRegSizes; i++) {
        if (kRegSizes[i] == N) return off;
        off += kRegSizes[i];
    }
    return -1;
}
constexpr int kRegTableLen = reg_offset(64) + 64;

constexpr int pick_radix(int m) {
    return m % 4 == 0 ? 4 : m % 2 == 0 ? 2 : m % 3 == 0 ? 3 : m % 5 == 0 ? 5 : m;
}

// per translation unit: w_N^t = exp(-2 pi i t / N) for every N in kRegSizes
static __constant__ float2 c_regtw_f[kRegTableLen];
static __constant__ double2 c_regtw_d[kRegTableLen];
static __constant__ ffc c_regtw_q[kRegTableLen];  // float-float

template <typename T> __device__ __forceinline__ C2<T> regtw(int i);
template <> __device__ __forceinline__ float2 regtw<float>(int i) { return c_regtw_f[i]; }
template <> __device__ __forceinline__ double2 regtw<double>(int i) { return c_regtw_d[i]; }
template <> __device__ __forceinline__ ffc regtw<ff>(int i) { return c_regtw_q[i]; }

// upload the constant tables of this translation unit (host)
static inline cudaError_t fft4_init_tables() {
    static float2 hf[kRegTableLen];
    static double2 hd[kRegTableLen];
    static ffc hq[kRegTableLen];
    const long double pi = 3.14159265358979323846264338327950288L;
    for (int i = 0; i < kNumRegSizes; i++) {
        const int N = kRegSizes[i], off = reg_offset(N);
        for (int t = 0; t < N; t++) {
            long double a = -2.0L * pi * t / N;
            hd[off + t] = make_double2((double)cosl(a), (double)sinl(a));
            hf[off + t] = make_float2((float)cosl(a), (float)sinl(a));
            hq[off + t].x = ff_split(cosl(a));
            hq[off + t].y = ff_split(sinl(a));
        }
    }
    cudaError_t e = cudaMemcpyToSymbol(c_regtw_f, hf, sizeof hf);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_regtw_d, hd, sizeof hd);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_regtw_q, hq, sizeof hq);
    return e;
}

// The tables are per translation unit: every TU that launches four-step kernels calls this
// before its launches (uploads once per device).
static inline cudaError_t fft4_ensure_tables() {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    cudaError_t e = fft4_init_tables();
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

// one register Stockham stage chain: a holds the data, b is scratch; result ends in `a`.
// HZ: the upper half of the input (a[i], i >= N/2) is zero and never read.  The first stage
// (Ns = 1, no twiddles) then reads only inputs q < R/2 of each butterfly, which for radix 4 is
// y0 = x0 + x1, y1 = x0 + s i x1, y2 = x0 - x1, y3 = x0 - s i x1; the later stages are unchanged.
template <typename T, int N, int SIGN, int Ns, bool HZ = false>
struct RegStages {
    static __device__ __forceinline__ void run(C2<T> *a, C2<T> *b) {
        if constexpr (Ns < N) {
            constexpr int R = pick_radix(N / Ns);
            constexpr int nR = N / R;
            constexpr int step = N / (Ns * R);
            constexpr int off = reg_offset(N);
            static_assert(!HZ || (Ns == 1 && (R == 4 || R == 2)), "half-zero input needs a first radix of 2 or 4");
#pragma unroll
            for (int j = 0; j < nR; j++) {
                const int k = j % Ns;
                C2<T> t[R];
                if constexpr (HZ) {
                    const C2<T> x0 = a[j];
                    if constexpr (R == 4) {
                        const C2<T> x1 = a[j + nR], ix1 = cmuli(x1, SIGN);
                        t[0] = cadd(x0, x1);
                        t[1] = cadd(x0, ix1);
                        t[2] = csub(x0, x1);
                        t[3] = csub(x0, ix1);
                    } else {
                        t[0] = x0;
                        t[1] = x0;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < R; q++) {
                        t[q] = a[j + q * nR];
                        if (q && k) {
                            C2<T> w = regtw<T>(off + q * k * step);
                            if (SIGN > 0) w.y = -w.y;
                            t[q] = cmul(t[q], w);
                        }
                    }
                    butterfly<T, R>(t, SIGN, nullptr, 0);
                }
                const int base = (j / Ns) * Ns * R + k;
#pragma unroll
                for (int q = 0; q < R; q++) b[base + q * Ns] = t[q];
            }
#pragma unroll
            for (int i = 0; i < N; i++) a[i] = b[i];
            RegStages<T, N, SIGN, Ns * R>::run(a, b);
        }
    }
};

template <typename T, int N, int SIGN>
__device__ __forceinline__ void dft_reg(C2<T> (&a)[N]) {
    static_assert(reg_offset(N) >= 0, "register DFT size not in the constant table");
    C2<T> b[N];
    RegStages<T, N, SIGN, 1>::run(a, b);
}

// DFT of N points whose upper half a[N/2 .. N) is zero (those entries are not read)
template <typename T, int N, int SIGN>
__device__ __forceinline__ void dft_reg_hz(C2<T> (&a)[N]) {
    static_assert(reg_offset(N) >= 0 && N % 2 == 0, "register DFT size not in the constant table");
    C2<T> b[N];
    RegStages<T, N, SIGN, 1, true>::run(a, b);
}

// ---- Good-Thomas (prime-factor) register DFTs -----------------------------------------------
// For N = N1 * N2 with gcd(N1, N2) = 1 the DFT needs no twiddles: with the input map
// n = (N2 n1 + N1 n2) mod N and the output map k = CRT(k1 mod N1, k2 mod N2), X[k] is the
// N1 x N2 two-dimensional DFT of the reindexed input (Good 1958, Thomas 1963).  Both maps are
// compile-time register renamings, so only the short DFTs remain: DFT30 = 2 x 3 x 5 and
// DFT36 = 4 x 9 lose the 30 and 24 complex twiddle products of the mixed-radix chain.  Lengths
// without a coprime split (powers of two, 9, 27) use the Stockham chain (dft_reg).
constexpr int gcd_c(int a, int b) { return b ? gcd_c(b, a % b) : a; }
constexpr int inv_mod_c(int a, int m) {
    int x = 1;
    while (x < m && (a * x) % m != 1) x++;
    return x;
}
// first factor of a coprime split of N (the largest prime-power factor first), or 0
constexpr int pfa_n1(int N) {
    const int c[] = {16, 8, 4, 9, 27, 5, 3, 2};
    for (int i = 0; i < 8; i++)
        if (c[i] < N && N % c[i] == 0 && gcd_c(c[i], N / c[i]) == 1) return c[i];
    return 0;
}

template <typename T, int N, int SIGN>
__device__ __forceinline__ void dft_pfa(C2<T> (&a)[N]) {
    constexpr int N1 = pfa_n1(N);
    if constexpr (N1 == 0) {
        if constexpr (N == 2 || N == 3 || N == 4 || N == 5) butterfly<T, N>(a, SIGN, nullptr, 0);
        else dft_reg<T, N, SIGN>(a);
    } else {
        constexpr int N2 = N / N1;
        constexpr int e1 = N2 * inv_mod_c(N2 % N1, N1);  // k = (e1 k1 + e2 k2) mod N
        constexpr int e2 = N1 * inv_mod_c(N1 % N2, N2);
        C2<T> y[N1][N2];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++)
#pragma unroll
            for (int n2 = 0; n2 < N2; n2++) y[n1][n2] = a[(N2 * n1 + N1 * n2) % N];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) dft_pfa<T, N2, SIGN>(y[n1]);
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
            C2<T> col[N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; n1++) col[n1] = y[n1][k2];
            dft_pfa<T, N1, SIGN>(col);
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) a[(e1 * k1 + e2 * k2) % N] = col[k1];
        }
    }
}

// twiddle w_L^{SIGN * t} from a global table tw[t] = exp(-2 pi i t / L)
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> gtw(const C2<T> *tw, int t) {
    C2<T> w = __ldg(tw + t);
    if (SIGN > 0) w.y = -w.y;
    return w;
}

// Four-step tables of one length (FFT4Desc, plan.h), in global memory per plan:
//   tw4[n2*L1 + k1] = w_L^{n2*k1}               (inter-step twiddles)
//   chirp[k]        = exp(+i pi k^2 / n), k < n   (Bluestein only: the inverse transform's chirp)
//   filtb[k1*L2 + k2] = FFT_L(exp(-i pi m^2 / n), m = -(n-1)..n-1) at frequency k1 + L1*k2,
//                       times 1/L (Bluestein only)

// Tile widths 8 and 16 (the usual autotuned ones) get their own instantiation of the Bluestein
// body, so the row offsets (n*B) are compile-time immediates; other widths use the runtime form.
constexpr int ct_lg2(int b) { return b <= 1 ? 0 : 1 + ct_lg2(b / 2); }

// ---- natural -> permuted (steps A, B) ---------------------------------------------------------
// PFA: prime-factor register DFTs (dft_pfa) instead of the mixed-radix chain (dft_reg).
// WAIT: complete the calling thread's asynchronous copies before the final barrier, so that
// copies issued before the transform are visible to the whole block when it returns.
template <typename T, int L1, int L2, int SIGN, bool PFA = true, bool WAIT = false>
__device__ __forceinline__ void fft4_np_impl(C2<T> *X, int B, const FFT4Desc &d) {
    const int lgB = lg2(B);
    constexpr int L = L1 * L2;
    const C2<T> *tw4 = (const C2<T> *)d.tw4;
    for (int idx = threadIdx.x; idx < B * L2; idx += blockDim.x) {
        const int c = idx & (B - 1), n2 = idx >> lgB;
        C2<T> a[L1];
#pragma unroll
        for (int n1 = 0; n1 < L1; n1++) a[n1] = X[(n2 + L2 * n1) * B + c];
        if constexpr (PFA) dft_pfa<T, L1, SIGN>(a); else dft_reg<T, L1, SIGN>(a);
#pragma unroll
        for (int k1 = 1; k1 < L1; k1++) a[k1] = cmul(a[k1], gtw<T, SIGN>(tw4, n2 * L1 + k1));
#pragma unroll
        for (int k1 = 0; k1 < L1; k1++) X[(n2 + L2 * k1) * B + c] = a[k1];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < B * L1; idx += blockDim.x) {
        const int c = idx & (B - 1), k1 = idx >> lgB;
        C2<T> b[L2];
#pragma unroll
        for (int n2 = 0; n2 < L2; n2++) b[n2] = X[(L2 * k1 + n2) * B + c];
        if constexpr (PFA) dft_pfa<T, L2, SIGN>(b); else dft_reg<T, L2, SIGN>(b);
#pragma unroll
        for (int k2 = 0; k2 < L2; k2++) X[(L2 * k1 + k2) * B + c] = b[k2];
    }
    if constexpr (WAIT) async_wait();
    __syncthreads();
    (void)L;
}

// Three width-specialised bodies per call site made the x and y passes slower; instead the
// kernels come in fixed-width copies whose constant width reaches these bodies by inlining.
template <typename T, int L1, int L2, int SIGN>
__device__ __forceinline__ void fft4_np(C2<T> *X, int B, const FFT4Desc &d) {
    fft4_np_impl<T, L1, L2, SIGN>(X, B, d);
}

// ---- permuted -> natural (steps B', A') -------------------------------------------------------
// PFA: prime-factor register DFTs (dft_pfa) instead of the mixed-radix chain (dft_reg)
template <typename T, int L1, int L2, int SIGN, bool PFA = true>
__device__ __forceinline__ void fft4_pn_impl(C2<T> *X, int B, const FFT4Desc &d) {
    const int lgB = lg2(B);
    const C2<T> *tw4 = (const C2<T> *)d.tw4;
    for (int idx = threadIdx.x; idx < B * L1; idx += blockDim.x) {
        const int c = idx & (B - 1), k1 = idx >> lgB;
        C2<T> b[L2];
#pragma unroll
        for (int k2 = 0; k2 < L2; k2++) b[k2] = X[(L2 * k1 + k2) * B + c];
        if constexpr (PFA) dft_pfa<T, L2, SIGN>(b); else dft_reg<T, L2, SIGN>(b);
#pragma unroll
        for (int m2 = 1; m2 < L2; m2++) b[m2] = cmul(b[m2], gtw<T, SIGN>(tw4, m2 * L1 + k1));
#pragma unroll
        for (int m2 = 0; m2 < L2; m2++) X[(L2 * k1 + m2) * B + c] = b[m2];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < B * L2; idx += blockDim.x) {
        const int c = idx & (B - 1), m2 = idx >> lgB;
        C2<T> a[L1];
#pragma unroll
        for (int k1 = 0; k1 < L1; k1++) a[k1] = X[(L2 * k1 + m2) * B + c];
        if constexpr (PFA) dft_pfa<T, L1, SIGN>(a); else dft_reg<T, L1, SIGN>(a);
#pragma unroll
        for (int m1 = 0; m1 < L1; m1++) X[(m2 + L2 * m1) * B + c] = a[m1];
    }
    __syncthreads();
}

template <typename T, int L1, int L2, int SIGN>
__device__ __forceinline__ void fft4_pn(C2<T> *X, int B, const FFT4Desc &d) {
    fft4_pn_impl<T, L1, L2, SIGN>(X, B, d);
}

// position in the permuted layout of frequency k
template <int L1, int L2>
__device__ __forceinline__ int perm_pos(int k) { return L2 * (k % L1) + k / L1; }

// ---- Bluestein over L = L1*L2: natural rows [0, n) in, natural rows [0, n) out -------------------
// Rows [n, L) are never read.  The caller fills rows [0, n) and syncs first.  The direction
// Only the inverse transform's tables are kept (chirp, filtb): the forward transform is computed
// as conj(inverse(conj(x))), the conjugations folded into the chirp multiplies of steps A and
// A', so one chirp and one filter table serve both directions (and one body, as the direction
// is a runtime sign).
// Bluestein pads to L >= 2n - 1, so n <= L/2 = L2 * (L1/2) (L even, checked where the tables
// are built): in step A the inputs n1 >= L1/2 are the zero padding and in step A' the outputs
// m1 >= L1/2 are discarded, so both steps work on half of their DFT_L1 ends.
// CB: the tile width when known at compile time, else 0
// Step B's DFTs always use the prime-factor form (dft_pfa).  PFA: step A' too; the out-of-line
// copies called by the fused column kernels (fft4_bluestein_ni, fft4_np_ni) keep the
// mixed-radix DFT there, whose smaller register footprint costs the callers fewer saves around
// the call (measured with the prime-factor form in every step: fused_theta 10 % slower,
// z_inverse 5 % faster; in step B only: fused_vcomp and fused_theta 2-3 % faster).
template <typename T, int L1, int L2, int CB, bool PFA>
__device__ __forceinline__ void fft4_bluestein_impl(C2<T> *X, int Brt, const FFT4Desc &d, int sign) {
    static_assert(L1 % 2 == 0, "Bluestein four-step needs an even L1");
    constexpr int kH = L1 / 2;
    const int B = CB ? CB : Brt;
    const int lgB = CB ? ct_lg2(CB) : lg2(Brt);
    const C2<T> *tw4 = (const C2<T> *)d.tw4;
    const C2<T> *chirp = (const C2<T> *)d.chirp;
    const C2<T> *filt = (const C2<T> *)d.filtb;
    const int n = d.n;
    const T cs = sign < 0 ? (T)-1 : (T)1;  // forward: conjugate input and output
    // step A (forward FFT of the convolution): conj^(sign<0)(input) * chirp
    for (int idx = threadIdx.x; idx < B * L2; idx += blockDim.x) {
        const int c = idx & (B - 1), n2 = idx >> lgB;
        C2<T> a[L1];
#pragma unroll
        for (int n1 = 0; n1 < kH; n1++) {
            const int pos = n2 + L2 * n1;
            const C2<T> w = pos < n ? __ldg(chirp + pos) : mk<T>(0, 0);
            C2<T> xv = pos < n ? X[pos * B + c] : mk<T>(0, 0);
            xv.y *= cs;
            a[n1] = cmul(xv, w);
        }
#pragma unroll
        for (int n1 = kH; n1 < L1; n1++) a[n1] = mk<T>(0, 0);  // not read by dft_reg_hz
        dft_reg_hz<T, L1, -1>(a);
#pragma unroll
        for (int k1 = 1; k1 < L1; k1++) a[k1] = cmul(a[k1], gtw<T, -1>(tw4, n2 * L1 + k1));
#pragma unroll
        for (int k1 = 0; k1 < L1; k1++) X[(n2 + L2 * k1) * B + c] = a[k1];
    }
    __syncthreads();
    // step B (forward), filter, step B' (inverse): all in registers
    for (int idx = threadIdx.x; idx < B * L1; idx += blockDim.x) {
        const int c = idx & (B - 1), k1 = idx >> lgB;
        C2<T> b[L2];
#pragma unroll
        for (int n2 = 0; n2 < L2; n2++) b[n2] = X[(L2 * k1 + n2) * B + c];
        dft_pfa<T, L2, -1>(b);
#pragma unroll
        for (int k2 = 0; k2 < L2; k2++) b[k2] = cmul(b[k2], __ldg(filt + k1 * L2 + k2));
        dft_pfa<T, L2, +1>(b);
#pragma unroll
        for (int m2 = 1; m2 < L2; m2++) b[m2] = cmul(b[m2], gtw<T, +1>(tw4, m2 * L1 + k1));
#pragma unroll
        for (int m2 = 0; m2 < L2; m2++) X[(L2 * k1 + m2) * B + c] = b[m2];
    }
    __syncthreads();
    // step A' (inverse), output * chirp (conjugated for the forward transform) on rows < n
    for (int idx = threadIdx.x; idx < B * L2; idx += blockDim.x) {
        const int c = idx & (B - 1), m2 = idx >> lgB;
        C2<T> a[L1];
#pragma unroll
        for (int k1 = 0; k1 < L1; k1++) a[k1] = X[(L2 * k1 + m2) * B + c];
        if constexpr (PFA) dft_pfa<T, L1, +1>(a); else dft_reg<T, L1, +1>(a);
#pragma unroll
        for (int m1 = 0; m1 < kH; m1++) {
            const int pos = m2 + L2 * m1;
            if (pos < n) {
                C2<T> o = cmul(a[m1], __ldg(chirp + pos));
                o.y *= cs;
                X[pos * B + c] = o;
            }
        }
    }
    __syncthreads();
}

template <typename T, int L1, int L2, bool PFA = true>
__device__ __forceinline__ void fft4_bluestein_body(C2<T> *X, int B, const FFT4Desc &d, int sign) {
    if (B == 8) fft4_bluestein_impl<T, L1, L2, 8, PFA>(X, 8, d, sign);
    else if (B == 16) fft4_bluestein_impl<T, L1, L2, 16, PFA>(X, 16, d, sign);
    else fft4_bluestein_impl<T, L1, L2, 0, PFA>(X, B, d, sign);
}

template <typename T, int L1, int L2, int SIGN>
__device__ __forceinline__ void fft4_bluestein(C2<T> *X, int B, const FFT4Desc &d) {
    fft4_bluestein_body<T, L1, L2>(X, B, d, SIGN);
}

// Out-of-line copies for kernels that transform at many call sites (the fused column kernels):
// one body in the instruction stream instead of one per call site.
template <typename T, int L1, int L2>
__device__ __noinline__ void fft4_bluestein_ni(C2<T> *X, int B, const FFT4Desc &d, int sign) {
    fft4_bluestein_body<T, L1, L2, false>(X, B, d, sign);
}
template <typename T, int L1, int L2, int SIGN>
__device__ __noinline__ void fft4_np_ni(C2<T> *X, int B, const FFT4Desc &d) {
    fft4_np_impl<T, L1, L2, SIGN, false>(X, B, d);
}

}  // namespace sg
