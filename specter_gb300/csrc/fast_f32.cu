// FP32 register four-step passes for the production grid lengths (see fast.h).
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "fast.h"

namespace sg {

// Compiled splits L = L1 * L2: z (Bluestein lengths of nz = 538 and 282), y (512, 256) and
// x (H = 256, 128) of the 512^3- and 256^3-class grids.
bool fast_pair(int L, int *L1, int *L2) {
    switch (L) {
    case 1080: *L1 = 36; *L2 = 30; return true;
    case 576: *L1 = 24; *L2 = 24; return true;
    case 512: *L1 = 32; *L2 = 16; return true;
    case 256: *L1 = 16; *L2 = 16; return true;
    case 128: *L1 = 16; *L2 = 8; return true;
    default: return false;
    }
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

int fast_init_device() {
    if (fft4_ensure_tables() != cudaSuccess) { set_error("constant table upload failed"); return ERR_CUDA; }
    return OK;
}

int build_fft4_table(FFT4Table &t, int n) {
    t = FFT4Table{};
    int L1 = 0, L2 = 0, L = n, blue = 0;
    if (!fast_pair(n, &L1, &L2)) {
        L = 2 * n - 1;
        while (!smooth235(L)) L++;
        if (!fast_pair(L, &L1, &L2)) return OK;  // no compiled four-step kernel: generic engine
        // the Bluestein body skips the zero half of step A and the unused half of step A'
        // (fft4.cuh), which needs n <= L/2 and an even L1
        if (2 * n > L || L1 % 2) return OK;
        blue = 1;
    }
    int st = fast_init_device();
    if (st) return st;
    const size_t ntot = (size_t)L + (blue ? (size_t)n + 2 * (size_t)L : 0);
    std::vector<float2> h(ntot);
    for (int n2 = 0; n2 < L2; n2++)
        for (int k1 = 0; k1 < L1; k1++) {
            cld w = root((long)n2 * k1, L);
            h[(size_t)n2 * L1 + k1] = make_float2((float)w.real(), (float)w.imag());
        }
    if (blue) {
        const long double pi = 3.14159265358979323846264338327950288L;
        std::vector<cld> chirp(n), bf(L, cld(0)), bb(L, cld(0)), w(L);
        for (long k = 0; k < n; k++) {
            long double a = -pi * (long double)((k * k) % (2L * n)) / (long double)n;
            chirp[k] = cld(cosl(a), sinl(a));
            h[(size_t)L + k] = make_float2((float)chirp[k].real(), (float)chirp[k].imag());
        }
        for (int k = 0; k < n; k++) {
            bf[k] = std::conj(chirp[k]);
            bb[k] = chirp[k];
            if (k) { bf[L - k] = std::conj(chirp[k]); bb[L - k] = chirp[k]; }
        }
        for (int k = 0; k < L; k++) w[k] = root(k, L);
        for (int j = 0; j < L; j++) {
            cld sf(0), sb(0);
            for (int m = 0; m < L; m++) {
                if (bf[m] == cld(0)) continue;
                const cld ww = w[((long)j * m) % L];
                sf += bf[m] * ww;
                sb += bb[m] * ww;
            }
            sf /= (long double)L;
            sb /= (long double)L;
            const int k1 = j % L1, k2 = j / L1;  // frequency j = k1 + L1*k2 -> slot k1*L2 + k2
            h[(size_t)L + n + (size_t)k1 * L2 + k2] = make_float2((float)sf.real(), (float)sf.imag());
            h[(size_t)L + n + L + (size_t)k1 * L2 + k2] = make_float2((float)sb.real(), (float)sb.imag());
        }
    }
    if (cudaMalloc(&t.mem, h.size() * sizeof(float2)) != cudaSuccess) { set_error("cudaMalloc failed"); return ERR_OOM; }
    cudaMemcpy(t.mem, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice);
    float2 *b = (float2 *)t.mem;
    t.d.n = n; t.d.L = L; t.d.L1 = L1; t.d.L2 = L2; t.d.blue = blue;
    t.d.tw4 = b;
    if (blue) { t.d.chirp = b + L; t.d.filtf = b + L + n; t.d.filtb = b + L + n + L; }
    t.ok = 1;
    return OK;
}

void free_fft4_table(FFT4Table &t) {
    if (t.mem) cudaFree(t.mem);
    t = FFT4Table{};
}

// ------------------------------------------------------------------ launches

namespace {
constexpr size_t kFastBudget = 110 * 1024;  // two resident blocks per SM
constexpr size_t kMaxSmem = 227 * 1024;     // one block per SM (largest dynamic allocation)

int pick(size_t per, size_t budget = kFastBudget) {
    for (int t : {16, 8, 4, 2, 1})
        if (per * t <= budget) return t;
    return 0;
}

// Stage the input tile once (two-output passes) only when that keeps the tile width; otherwise
// the second output re-reads the tile, which is then still in L2.
int stage_tile(void *const out0[], void *const out1[], int nf, int L, int n) {
    int two = 0;
    for (int f = 0; f < nf; f++) two |= (out0[f] && out1[f]) ? 1 : 0;
    if (!two) return 0;
    return pick((size_t)L * sizeof(float2)) == pick(((size_t)L + n) * sizeof(float2)) ? 1 : 0;
}

template <typename K>
void smem_attr(K kern, size_t bytes) {
    if (bytes > 40 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct Scope {
    Plan &P;
    Scope(Plan &p, const char *n, double b) : P(p) { P.prof_begin(n, b); }
    ~Scope() { P.prof_end(); }
};

int done(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string(what) + ": " + cudaGetErrorString(e)); return ERR_CUDA; }
    return OK;
}

template <int L1, int L2>
int zinv(Plan &P, const ZInvArgs &a0, int nf, double bytes) {
    using E = FourStep<float, L1, L2>;
    ZInvArgs a = a0;
    a.staged = stage_tile(a.out0, a.out1, nf, P.tz4.d.L, P.nz);
    const size_t per = ((size_t)P.tz4.d.L + (a.staged ? P.nz : 0)) * sizeof(float2);
    const int tk = P.capped(pick(per), Plan::kTileZ);
    const size_t sm = per * tk;
    smem_attr(k_z_inverse<float, E>, sm);
    Scope s(P, "z_inverse", bytes);
    k_z_inverse<float, E><<<dim3(cdiv(P.nxh, tk), P.ny, nf), kThreads, sm, P.stream>>>(P.geo, P.tz4.d, a.prepared(), tk);
    return done("z_inverse");
}

template <int L1, int L2>
int zfwd(Plan &P, const ZFwdArgs &a, int nf, double bytes) {
    using E = FourStep<float, L1, L2>;
    const int tk = P.capped(pick((size_t)P.tz4.d.L * sizeof(float2)), Plan::kTileZ);
    const size_t sm = (size_t)P.tz4.d.L * tk * sizeof(float2);
    smem_attr(k_z_forward<float, E>, sm);
    Scope s(P, "z_forward", bytes);
    k_z_forward<float, E><<<dim3(cdiv(P.nxh, tk), P.ny, nf), kThreads, sm, P.stream>>>(P.geo, P.tz4.d, a.prepared(), tk);
    return done("z_forward");
}

template <int L1, int L2>
int ypass(Plan &P, const YArgs &a0, int nf, int nplanes, double bytes) {
    using E = FourStep<float, L1, L2>;
    YArgs a = a0;
    a.staged = stage_tile(a.out0, a.out1, nf, P.ty4.d.L, P.ny);
    const size_t per = ((size_t)P.ty4.d.L + (a.staged ? P.ny : 0)) * sizeof(float2);
    const int tk = P.capped(pick(per), Plan::kTileY);
    const size_t sm = per * tk;
    smem_attr(k_y_pass<float, E>, sm);
    Scope s(P, a.sign < 0 ? "y_forward" : "y_inverse", bytes);
    k_y_pass<float, E><<<dim3(cdiv(P.nxh, tk), nplanes, nf), kThreads, sm, P.stream>>>(P.geo, P.ty4.d, a.prepared(), tk);
    return done("y_pass");
}

template <int L1, int L2>
int xpass(Plan &P, const XArgs &a, int nf, bool r2c, double bytes) {
    using E = FourStep<float, L1, L2>;
    int rb = 0;
    for (int t : {16, 8, 4, 2, 1})
        if (t <= P.tile_cap[Plan::kTileX] && x_pass_elems<E>(P.tx4.d, P.nxh, t) * sizeof(float2) <= kFastBudget) { rb = t; break; }
    if (!rb) return kNoFast;
    const size_t sm = x_pass_elems<E>(P.tx4.d, P.nxh, rb) * sizeof(float2);
    const dim3 grid(cdiv(a.nrows * P.ny, rb), 1, nf);
    if (r2c) {
        smem_attr(k_x_r2c<float, E>, sm);
        Scope s(P, "x_r2c", bytes);
        k_x_r2c<float, E><<<grid, kThreads, sm, P.stream>>>(P.geo, P.tx4.d, a.prepared(), rb);
    } else {
        smem_attr(k_x_c2r<float, E>, sm);
        Scope s(P, "x_c2r", bytes);
        k_x_c2r<float, E><<<grid, kThreads, sm, P.stream>>>(P.geo, P.tx4.d, a.prepared(), rb);
    }
    return done(r2c ? "x_r2c" : "x_c2r");
}

template <int L1, int L2>
int xnl(Plan &P, const XNLArgs &a, double bytes) {
    using E = FourStep<float, L1, L2>;
    int rb = 0;
    for (int t : {16, 8, 4, 2, 1})
        if (t <= P.tile_cap[Plan::kTileX] && x_nl_elems<E>(P.tx4.d, P.nxh, P.H, t) * sizeof(float2) <= kMaxSmem) { rb = t; break; }
    if (!rb) return kNoFast;
    const size_t sm = x_nl_elems<E>(P.tx4.d, P.nxh, P.H, rb) * sizeof(float2);
    smem_attr(k_x_nonlinear<float, E>, sm);
    Scope s(P, "x_nonlinear", bytes);
    k_x_nonlinear<float, E><<<dim3(cdiv(a.nrows * P.ny, rb)), kThreads, sm, P.stream>>>(P.geo, P.tx4.d, a.prepared(), rb);
    return done("x_nonlinear");
}
}  // namespace

template <int V> using IC = std::integral_constant<int, V>;

// calls fn(IC<L1>, IC<L2>) for the compiled split of the table's length
template <typename Fn>
static int dispatch(const Plan &P, const FFT4Table &t, Fn &&fn) {
    if (P.prec != FP32 || !t.ok) return kNoFast;
    const int l1 = t.d.L1, l2 = t.d.L2;
    if (l1 == 36 && l2 == 30) return fn(IC<36>{}, IC<30>{});
    if (l1 == 24 && l2 == 24) return fn(IC<24>{}, IC<24>{});
    if (l1 == 32 && l2 == 16) return fn(IC<32>{}, IC<16>{});
    if (l1 == 16 && l2 == 16) return fn(IC<16>{}, IC<16>{});
    if (l1 == 16 && l2 == 8) return fn(IC<16>{}, IC<8>{});
    return kNoFast;
}

int fast_z_inverse(Plan &P, const ZInvArgs &a, int nf, double bytes) {
    return dispatch(P, P.tz4, [&](auto l1, auto l2) { return zinv<decltype(l1)::value, decltype(l2)::value>(P, a, nf, bytes); });
}
int fast_z_forward(Plan &P, const ZFwdArgs &a, int nf, double bytes) {
    return dispatch(P, P.tz4, [&](auto l1, auto l2) { return zfwd<decltype(l1)::value, decltype(l2)::value>(P, a, nf, bytes); });
}
int fast_y(Plan &P, const YArgs &a, int nf, int nplanes, double bytes) {
    return dispatch(P, P.ty4, [&](auto l1, auto l2) { return ypass<decltype(l1)::value, decltype(l2)::value>(P, a, nf, nplanes, bytes); });
}
int fast_x(Plan &P, const XArgs &a, int nf, bool r2c, double bytes) {
    return dispatch(P, P.tx4, [&](auto l1, auto l2) { return xpass<decltype(l1)::value, decltype(l2)::value>(P, a, nf, r2c, bytes); });
}
int fast_x_nl(Plan &P, const XNLArgs &a, double bytes) {
    return dispatch(P, P.tx4, [&](auto l1, auto l2) { return xnl<decltype(l1)::value, decltype(l2)::value>(P, a, bytes); });
}

}  // namespace sg
