// Float-float column kernels of the precision form on the three-step Bluestein engine
// (ffblue.cuh), and that engine's tables.
#include <cmath>
#include <complex>
#include <vector>

#include "fused_launch.cuh"
#include "ops.h"

namespace sg {

namespace {
typedef std::complex<long double> cld;
const long double kPi = 3.14159265358979323846264338327950288L;
cld root_l(long t, long n) {  // exp(-2 pi i t / n)
    const long double a = -2.0L * kPi * (long double)(t % n) / (long double)n;
    return cld(cosl(a), sinl(a));
}
ffc to_ffc(const cld &v) {
    ffc q;
    q.x = ff_split(v.real());
    q.y = ff_split(v.imag());
    return q;
}
}  // namespace

// Tables in the FFBTab layout, computed in long double: the step twiddles w_120^(n2 k1) and
// w_1080^(n3 j), the inverse transform's chirp exp(+i pi k^2 / n), and the filter: the length-L
// DFT of exp(-i pi m^2 / n), m = -(n-1) .. n-1 (wrapped), times 1/L, at frequency
// f = k1 + 8 k2 + 120 k3 stored in slot (k1 * 15 + k2) * 9 + k3 (the order step C reads).
int build_ffb_table(FFBTable &t, int n, int j0, int win) {
    using T = FFBTab;
    t = FFBTable{};
    if (n > T::kMaxN || 4 * n <= T::L) return OK;
    std::vector<ffc> h(T::kLen);
    for (auto &q : h) q.x = q.y = ff(0.f, 0.f);
    for (int n2 = 0; n2 < T::L2; n2++)
        for (int k1 = 0; k1 < T::L1; k1++) h[T::kOffTw1 + n2 * T::kTw1S + k1] = to_ffc(root_l((long)n2 * k1, T::J));
    for (int n3 = 0; n3 < T::L3; n3++)
        for (int j = 0; j < T::J; j++) h[T::kOffTw2 + n3 * T::kTw2S + j] = to_ffc(root_l((long)n3 * j, T::L));
    const int L = T::L;
    std::vector<cld> chirp(n), bb(L, cld(0)), w(L);
    for (long k = 0; k < n; k++) {
        const long double a = -kPi * (long double)((k * k) % (2L * n)) / (long double)n;
        chirp[k] = cld(cosl(a), sinl(a));
        h[T::kOffChirp + k] = to_ffc(std::conj(chirp[k]));
    }
    for (int k = 0; k < n; k++) {
        bb[k] = chirp[k];
        if (k) bb[L - k] = chirp[k];
    }
    for (int k = 0; k < L; k++) w[k] = root_l(k, L);
    for (int f = 0; f < L; f++) {
        cld s(0);
        for (int m = 0; m < L; m++) {
            if (bb[m] == cld(0)) continue;
            s += bb[m] * w[((long)f * m) % L];
        }
        s /= (long double)L;
        const int k1 = f % T::L1, k2 = (f / T::L1) % T::L2, k3 = f / T::J;
        h[T::kOffFilt + (k1 * T::L2 + k2) * T::L3 + k3] = to_ffc(s);
    }
    if (cudaMalloc(&t.mem, (size_t)T::kBytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc failed (float-float z tables)");
        return ERR_OOM;
    }
    if (cudaMemcpy(t.mem, h.data(), (size_t)T::kBytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(t.mem);
        t.mem = nullptr;
        return check_launch("float-float z tables");
    }
    t.d.n = n;
    t.d.L = L;
    t.d.blue = 1;
    t.d.tab = (const ffc *)t.mem;
    t.ok = 1;
    // the wall round trips as window corrections: C + 2d = 35 window rows and n + 34 <= 576
    if (win == FFZTab::kWin) {
        const std::vector<ffc> z = ffz_table_host(n, j0);
        if (!z.empty()) {
            if (cudaMalloc(&t.zmem, z.size() * sizeof(ffc)) != cudaSuccess) {
                cudaGetLastError();
                free_ffb_table(t);
                set_error("cudaMalloc failed (float-float window tables)");
                return ERR_OOM;
            }
            if (cudaMemcpy(t.zmem, z.data(), z.size() * sizeof(ffc), cudaMemcpyHostToDevice) != cudaSuccess) {
                free_ffb_table(t);
                return check_launch("float-float window tables");
            }
            t.d.ztab = (const ffc *)t.zmem;
            t.d.zj0 = j0;
            // the kernels' FFT buffer also holds the window scratch after the spectrum
            const int rows = n + FFZTab::L + 2 * FFZTab::kWin;
            if (rows > t.d.L) t.d.L = rows;
        }
    }
    return OK;
}

// The window-correction table (ffzoom.cuh) for z length n and window start j0, in long double.
// Chirp c_k = exp(+i pi k^2 / n); filters G = FFT_L(g) / L with g[s] = conj(c_{j0+s}),
// s = -(n-1) .. kWin-1, and H = FFT_L(h) / L with h[s] = c_{s-j0}, s = -(kWin-1) .. n-1, both
// stored at s mod L (disjoint for n + kWin - 1 <= L), at frequency f = k1 + 8 k2 + 64 k3 in slot
// (k1 * 8 + k2) * 9 + k3.  Empty when n is odd or too long.
namespace {
cld chirp_l(long k, long n) {  // exp(+i pi k^2 / n), period n for even n
    k = ((k % n) + n) % n;
    const long double a = kPi * (long double)((k * k) % (2L * n)) / (long double)n;
    return cld(cosl(a), sinl(a));
}
}  // namespace

std::vector<ffc> ffz_table_host(int n, int j0) {
    using T = FFZTab;
    if (n % 2 || n > T::kMaxN || j0 < 0 || j0 >= n) return {};
    std::vector<ffc> h(T::kLen);
    for (auto &e : h) e.x = e.y = ff(0.f, 0.f);
    for (int n2 = 0; n2 < T::L2; n2++)
        for (int k1 = 0; k1 < T::L1; k1++) h[T::kOffTw1 + n2 * T::kTw1S + k1] = to_ffc(root_l((long)n2 * k1, T::J));
    for (int n3 = 0; n3 < T::L3; n3++)
        for (int j = 0; j < T::J; j++) h[T::kOffTw2 + n3 * T::kTw2S + j] = to_ffc(root_l((long)n3 * j, T::L));
    for (int k = 0; k < n; k++) h[T::kOffChirp + k] = to_ffc(chirp_l(k, n));
    std::vector<cld> g(T::L, cld(0)), hh(T::L, cld(0)), w(T::L);
    for (int s = -(n - 1); s <= T::kWin - 1; s++) g[(s + T::L) % T::L] = std::conj(chirp_l(j0 + s, n));
    for (int s = -(T::kWin - 1); s <= n - 1; s++) hh[(s + T::L) % T::L] = chirp_l(s - j0, n);
    for (int k = 0; k < T::L; k++) w[k] = root_l(k, T::L);
    for (int f = 0; f < T::L; f++) {
        cld sg(0), sh(0);
        for (int m = 0; m < T::L; m++) {
            const cld r = w[((long)f * m) % T::L];
            sg += g[m] * r;
            sh += hh[m] * r;
        }
        const int k1 = f % T::L1, k2 = (f / T::L1) % T::L2, k3 = f / T::J;
        h[T::kOffG + (k1 * T::L2 + k2) * T::L3 + k3] = to_ffc(sg / (long double)T::L);
        h[T::kOffH + (k1 * T::L2 + k2) * T::L3 + k3] = to_ffc(sh / (long double)T::L);
    }
    return h;
}

void free_ffb_table(FFBTable &t) {
    if (t.mem) cudaFree(t.mem);
    if (t.zmem) cudaFree(t.zmem);
    t = FFBTable{};
}

// Two block shapes, chosen per kernel family by the plan (the autotuner tries both):
//   one block of 576 threads per SM at a tile width of 8: the three transform steps have 1080,
//   576 and 960 items (two rounds, one, two); alone the transform is fastest so (26 ns a column
//   against 29 ns for the pair below);
//   two blocks of 288 threads per SM at a width of 4: the same items per thread, and one block's
//   global loads and barriers overlap the other's arithmetic.
// Copies of the column kernels with the width fixed carry one transform body each.
int ffb_fused(Plan &P, const FFBDesc &d, const FusedArgs &a, int which, double bytes) {
    // the projection's FP32 pressure transform uses this translation unit's constant twiddles
    if (fft4_ensure_tables() != cudaSuccess) { set_error("constant table upload failed"); return ERR_CUDA; }
    const bool pair = which == kFusedVProj ? P.ff_pair_proj : P.ff_pair_cols;
    if (pair) return ffb_fused_pair(P, d, a, which, bytes);
    return launch_fused<ff, FFBlue<576>, 8>(P, d, a, which, bytes);
}

}  // namespace sg
