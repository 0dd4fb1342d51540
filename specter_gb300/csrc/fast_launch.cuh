// Launch helpers of the FP32 four-step passes, shared by the translation units that
// instantiate them (fast_f32.cu: z passes; fast_x_f32.cu: x passes; fast_y_f32.cu: y passes).
#pragma once

#include <string>
#include <type_traits>

#include "fast.h"

namespace sg {
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
    // the production z lengths (Bluestein 1080, 576) at tile width 8 run a copy with the width fixed
    constexpr bool kFixed = (L1 == 36 && L2 == 30) || (L1 == 24 && L2 == 24);
    if (P.batch) {  // record for a batched launch (batch.h)
        using R = PassRec<E, ZInvArgs>;
        const R r{{0, cdiv(P.nxh, tk), P.ny, nf}, P.geo, P.tz4.d, a.prepared(), tk};
        batch_add(*P.batch, r, (const void *)k_z_inverse_batch<float, E>, &batch_launch<R, k_z_inverse_batch<float, E>, kThreads>,
                  sm, "z_inverse", bytes);
        return OK;
    }
    auto k = (kFixed && tk == 8) ? k_z_inverse<float, E, kFixed ? 8 : 0> : k_z_inverse<float, E>;
    smem_attr(k, sm);
    Scope s(P, "z_inverse", bytes);
    k<<<dim3(cdiv(P.nxh, tk), P.ny, nf), kThreads, sm, P.stream>>>(P.geo, P.tz4.d, a.prepared(), tk);
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
    // the production y lengths (512, 256) at tile width 16 run a copy with the width fixed
    constexpr bool kFixed = L2 == 16 && (L1 == 32 || L1 == 16);
    if (P.batch) {  // record for a batched launch (batch.h)
        using R = PassRec<E, YArgs>;
        const R r{{0, cdiv(P.nxh, tk), nplanes, nf}, P.geo, P.ty4.d, a.prepared(), tk};
        batch_add(*P.batch, r, (const void *)k_y_pass_batch<float, E>, &batch_launch<R, k_y_pass_batch<float, E>, kThreads>,
                  sm, a.sign < 0 ? "y_forward" : "y_inverse", bytes);
        return OK;
    }
    auto k = (kFixed && tk == 16) ? k_y_pass_t<float, E, kFixed ? 16 : 0> : k_y_pass_t<float, E, 0>;
    smem_attr(k, sm);
    Scope s(P, a.sign < 0 ? "y_forward" : "y_inverse", bytes);
    k<<<dim3(cdiv(P.nxh, tk), nplanes, nf), kThreads, sm, P.stream>>>(P.geo, P.ty4.d, a.prepared(), tk);
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
    // the production x lengths (H = 256, 128) at 8 rows run a copy with the row count fixed,
    // which takes the pipelined form (two FFT buffers, row-major staging: x_nl_pipe_elems)
    constexpr bool kFixed = L1 == 16 && (L2 == 16 || L2 == 8);
    const bool fixed = kFixed && rb == 8;
    if (P.batch) {  // record for a batched launch (batch.h): the plain body
        const size_t smb = x_nl_elems<E>(P.tx4.d, P.nxh, P.H, rb) * sizeof(float2);
        using R = PassRec<E, XNLArgs>;
        const R r{{0, cdiv(a.nrows * P.ny, rb), 1, 1}, P.geo, P.tx4.d, a.prepared(), rb};
        batch_add(*P.batch, r, (const void *)k_x_nonlinear_batch<float, E>,
                  &batch_launch<R, k_x_nonlinear_batch<float, E>, kThreads>, smb, "x_nonlinear", bytes);
        return OK;
    }
    const size_t sm = (fixed ? x_nl_pipe_elems(P.nxh, P.H, rb) : x_nl_elems<E>(P.tx4.d, P.nxh, P.H, rb)) * sizeof(float2);
    auto k = fixed ? k_x_nonlinear<float, E, kFixed ? 8 : 0> : k_x_nonlinear<float, E>;
    smem_attr(k, sm);
    Scope s(P, "x_nonlinear", bytes);
    k<<<dim3(cdiv(a.nrows * P.ny, rb)), kThreads, sm, P.stream>>>(P.geo, P.tx4.d, a.prepared(), rb);
    return done("x_nonlinear");
}
}  // namespace

template <int V> using IC = std::integral_constant<int, V>;

// calls fn(IC<L1>, IC<L2>) for the compiled split of the table's length on that axis
#define SG_DISPATCH_CASE(A, B) if (l1 == (A) && l2 == (B)) return fn(IC<A>{}, IC<B>{});
#define SG_DEFINE_DISPATCH(NAME, LIST)                                      \
    template <typename Fn>                                                  \
    static int NAME(const Plan &P, const FFT4Table &t, Fn &&fn) {           \
        if (P.prec != FP32 || !t.ok) return kNoFast;                        \
        const int l1 = t.d.L1, l2 = t.d.L2;                                 \
        LIST(SG_DISPATCH_CASE)                                              \
        return kNoFast;                                                     \
    }
SG_DEFINE_DISPATCH(dispatch_x, SG_FAST_PAIRS_X)
SG_DEFINE_DISPATCH(dispatch_y, SG_FAST_PAIRS_Y)
SG_DEFINE_DISPATCH(dispatch_z, SG_FAST_PAIRS_Z)

}  // namespace sg
