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
int build_ffb_table(FFBTable &t, int n) {
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
    return OK;
}

void free_ffb_table(FFBTable &t) {
    if (t.mem) cudaFree(t.mem);
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
    if (pair) return launch_fused<ff, FFBlue<288, 2>, 4>(P, d, a, which, bytes);
    return launch_fused<ff, FFBlue<576>, 8>(P, d, a, which, bytes);
}

}  // namespace sg
