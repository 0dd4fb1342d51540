// FP32 register four-step passes for the production grid lengths (see fast.h).
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "fast_launch.cuh"

namespace sg {

bool fast_pair(int axis, int L, int *L1, int *L2) {
#define SG_PAIR_CASE(A, B) if (L == (A) * (B)) { *L1 = A; *L2 = B; return true; }
    if (axis == kFastZ) { SG_FAST_PAIRS_Z(SG_PAIR_CASE) }
    if (axis == kFastY) { SG_FAST_PAIRS_Y(SG_PAIR_CASE) }
    if (axis == kFastX) { SG_FAST_PAIRS_X(SG_PAIR_CASE) }
#undef SG_PAIR_CASE
    return false;
}

static bool smooth235(int m) {
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    return m == 1;
}

typedef std::complex<long double> cld;
static cld root(long t, long n) {
    const long double pi = 3.14159265358979323846264338327950288L;
    long double a = -2.0L * pi * (long double)(t % n) / (long double)n;
    return cld(cosl(a), sinl(a));
}

// The register-DFT constant tables are per translation unit: upload those of the z (this
// file), x and y units.
int fast_init_device() {
    if (fft4_ensure_tables() != cudaSuccess || fast_x_init() != cudaSuccess || fast_y_init() != cudaSuccess) {
        set_error("constant table upload failed");
        return ERR_CUDA;
    }
    return OK;
}

// Tables of the four-step engine for an axis of length n: the length itself when it has a
// compiled split, else (z only) Bluestein over the smallest compiled length L >= 2n - 1.  The
// Bluestein body skips the zero half of step A and the unused half of step A' (fft4.cuh), which
// needs n <= L/2 and an even L1.  No table (t.ok = 0): the generic engine serves the axis.
int build_fft4_table(FFT4Table &t, int n, int axis) {
    t = FFT4Table{};
    int L1 = 0, L2 = 0, L = n, blue = 0;
    if (!fast_pair(axis, n, &L1, &L2)) {
        if (axis != kFastZ) return OK;
        L = 0;
        for (int m = 2 * n - 1; m <= 4 * n && !L; m++)
            if (smooth235(m) && 2 * n <= m && fast_pair(axis, m, &L1, &L2) && L1 % 2 == 0) L = m;
        if (!L) return OK;
        blue = 1;
    }
    int st = fast_init_device();
    if (st) return st;
    const size_t ntot = (size_t)L + (blue ? (size_t)n + (size_t)L : 0);
    std::vector<float2> h(ntot);
    for (int n2 = 0; n2 < L2; n2++)
        for (int k1 = 0; k1 < L1; k1++) {
            cld w = root((long)n2 * k1, L);
            h[(size_t)n2 * L1 + k1] = make_float2((float)w.real(), (float)w.imag());
        }
    if (blue) {
        const long double pi = 3.14159265358979323846264338327950288L;
        // chirp of the inverse transform, exp(+i pi k^2 / n); the filter is the length-L DFT of
        // its conjugate extended periodically over k = -(n-1)..n-1
        std::vector<cld> chirp(n), bb(L, cld(0)), w(L);
        for (long k = 0; k < n; k++) {
            long double a = -pi * (long double)((k * k) % (2L * n)) / (long double)n;
            chirp[k] = cld(cosl(a), sinl(a));
            h[(size_t)L + k] = make_float2((float)chirp[k].real(), (float)-chirp[k].imag());
        }
        for (int k = 0; k < n; k++) {
            bb[k] = chirp[k];
            if (k) bb[L - k] = chirp[k];
        }
        for (int k = 0; k < L; k++) w[k] = root(k, L);
        for (int j = 0; j < L; j++) {
            cld sb(0);
            for (int m = 0; m < L; m++) {
                if (bb[m] == cld(0)) continue;
                sb += bb[m] * w[((long)j * m) % L];
            }
            sb /= (long double)L;
            const int k1 = j % L1, k2 = j / L1;  // frequency j = k1 + L1*k2 -> slot k1*L2 + k2
            h[(size_t)L + n + (size_t)k1 * L2 + k2] = make_float2((float)sb.real(), (float)sb.imag());
        }
    }
    if (cudaMalloc(&t.mem, h.size() * sizeof(float2)) != cudaSuccess) { set_error("cudaMalloc failed"); return ERR_OOM; }
    cudaMemcpy(t.mem, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice);
    float2 *b = (float2 *)t.mem;
    t.d.n = n; t.d.L = L; t.d.L1 = L1; t.d.L2 = L2; t.d.blue = blue;
    t.d.tw4 = b;
    if (blue) { t.d.chirp = b + L; t.d.filtb = b + L + n; }
    t.ok = 1;
    return OK;
}

void free_fft4_table(FFT4Table &t) {
    if (t.mem) cudaFree(t.mem);
    t = FFT4Table{};
}

int fast_z_inverse(Plan &P, const ZInvArgs &a, int nf, double bytes) {
    return dispatch_z(P, P.tz4, [&](auto l1, auto l2) { return zinv<decltype(l1)::value, decltype(l2)::value>(P, a, nf, bytes); });
}
int fast_z_forward(Plan &P, const ZFwdArgs &a, int nf, double bytes) {
    return dispatch_z(P, P.tz4, [&](auto l1, auto l2) { return zfwd<decltype(l1)::value, decltype(l2)::value>(P, a, nf, bytes); });
}

}  // namespace sg
