// Launch helpers of the fused column kernels, shared by the generic and the four-step TUs.
#pragma once

#include <string>

#include "ffzoom.cuh"
#include "fused_kernels.cuh"

namespace sg {

enum FusedKernel { kFusedVelocity = 0, kFusedTheta = 1, kFusedHerm = 2, kFusedVComp = 3, kFusedVProj = 4 };

// FIX: a tile width with its own compiled copy of the column kernels (0: none)
template <typename T, class E, int FIX = 0>
int launch_fused(Plan &P, const typename E::Desc &fd, const FusedArgs &a, int which, double bytes) {
    const size_t es = sizeof(C2<T>);
    const size_t L = (size_t)fd.L;
    auto smem = [&](int tk) -> size_t {
        if (which == kFusedVProj && E::kStreamProj)  // vel_project_streamed: X, d, per-warp wall sums (two
                                                     // sets), coefficients, the pressure's wall rows
            return ((size_t)E::kProjRows + (size_t)P.nz) * tk * es + (4 * ((size_t)E::kColThreads / 32) * tk + (size_t)tk * 2) * 16 +
                   (size_t)tk * 2 * es + (size_t)tk * sizeof(LapCol<T>);
        if (which == kFusedVelocity || which == kFusedVProj) {
            const size_t thr = which == kFusedVelocity ? (size_t)E::wide_threads(tk) : (size_t)E::kColThreads;
            return (3 * (size_t)P.nz + E::kBuffers * L) * tk * es + (2 * thr + (size_t)tk * 2) * 16 +
                   (size_t)tk * sizeof(LapCol<T>);
        }
        if (which == kFusedTheta || which == kFusedVComp) {
            if constexpr (E::kZoom)  // update_direct: the FFT buffer only
                if (fd.ztab && a.nl_spec) return E::kBuffers * L * tk * es;
            return ((size_t)P.nz + E::kBuffers * L) * tk * es;
        }
        return E::kBuffers * L * 2 * es;
    };
    int tk = 2;
    if (which != kFusedHerm) {
        tk = 0;
        // the one-kernel velocity stage needs all three components: one block per SM; the others
        // (including the projection, which holds the three components but transforms once) keep
        // two blocks per SM
        // (float-float kernels run one block per SM anyway, their registers allow no more: they
        // may use most of the SM's shared memory)
        const size_t budget = which == kFusedVelocity ? 200 * 1024
                              : is_ff<T>              ? (E::kMinBlocks > 1 ? 110 : 220) * 1024
                                                      : 110 * 1024;
        for (int t : {16, 8, 4, 2, 1})
            if (t <= P.tile_cap[Plan::kTileFused] && smem(t) <= budget) { tk = t; break; }
        if (!tk) { set_error("z length too large for the fused column kernels"); return ERR_SHAPE; }
    }
    const size_t sm = smem(tk);
    const char *name = which == kFusedVelocity ? "fused_velocity"
                       : which == kFusedTheta  ? "fused_theta"
                       : which == kFusedVComp  ? "fused_vcomp"
                       : which == kFusedVProj  ? "fused_vproj"
                                               : "theta_herm";
    if constexpr (is_ff<T>) {  // float-float solvers are not batched (specter_batch_create)
        if (P.batch) { set_error("float-float column kernels have no batched form"); return ERR_STATE; }
    } else if (P.batch && (which == kFusedVComp || which == kFusedVProj)) {  // record (batch.h)
        using R = PassRec<E, FusedArgs>;
        const R r{{0, cdiv(P.nxh, tk), P.ny, which == kFusedVComp ? 3 : 1}, P.geo, fd, a.prepared(), tk};
        if (which == kFusedVComp)
            batch_add(*P.batch, r, (const void *)k_fused_vcomp_batch<T, E>,
                      &batch_launch<R, k_fused_vcomp_batch<T, E>, E::kColThreads>, sm, name, bytes);
        else
            batch_add(*P.batch, r, (const void *)k_fused_vproj_batch<T, E>,
                      &batch_launch<R, k_fused_vproj_batch<T, E>, E::kColThreads>, sm, name, bytes);
        return OK;
    }
    P.prof_begin(name, bytes);
    if (which == kFusedVelocity) {
        auto k = k_fused_velocity<T, E>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(cdiv(P.nxh, tk), P.ny), E::wide_threads(tk), sm, P.stream>>>(P.geo, fd, a.prepared(), tk);
    } else if (which == kFusedVComp) {
        auto k = (FIX && tk == FIX) ? k_fused_vcomp<T, E, FIX> : k_fused_vcomp<T, E>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(cdiv(P.nxh, tk), P.ny, 3), E::kColThreads, sm, P.stream>>>(P.geo, fd, a.prepared(), tk);
    } else if (which == kFusedVProj) {
        // the projection holds three components, so at the same cap it runs half the width of
        // the other column kernels: its own fixed-width copy at FIX / 2
        auto k = (FIX && tk == FIX) ? k_fused_vproj<T, E, FIX> : (FIX && tk == FIX / 2) ? k_fused_vproj<T, E, FIX / 2> : k_fused_vproj<T, E>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(cdiv(P.nxh, tk), P.ny), E::kColThreads, sm, P.stream>>>(P.geo, fd, a.prepared(), tk);
    } else if (which == kFusedTheta) {
        auto k = (FIX && tk == FIX) ? k_fused_theta<T, E, FIX> : k_fused_theta<T, E>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(cdiv(P.nxh, tk), P.ny), E::kColThreads, sm, P.stream>>>(P.geo, fd, a.prepared(), tk);
    } else {
        auto k = k_theta_herm<T, E>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(P.ny, 2), E::kColThreads, sm, P.stream>>>(P.geo, fd, a.prepared());
    }
    P.prof_end();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string(name) + ": " + cudaGetErrorString(e)); return ERR_CUDA; }
    return OK;
}

// four-step variant (fused_fast_f32.cu); kNoFast (-1) when the plan has no four-step z table
int fast_fused(Plan &P, const FusedArgs &a, int which, double bytes);

// tables of the float-float three-step Bluestein engine (ffblue.cuh) for one z length;
// ok == 0 when the length is outside (L/4, L/2] and the generic engine serves it (fused_ffb.cu)
struct FFBTable {
    FFBDesc d{};
    void *mem = nullptr;
    void *zmem = nullptr;  // window-correction tables (ffzoom.cuh), when the window fits
    int ok = 0;
};
// n = nz + C; window: first row j0 = nzp - d and win = C + 2d rows
int build_ffb_table(FFBTable &t, int n, int j0, int win);
void free_ffb_table(FFBTable &t);
// the float-float column kernels on that engine: one 576-thread block per SM (fused_ffb.cu) or two
// 288-thread blocks (fused_ffb_pair.cu)
int ffb_fused(Plan &P, const FFBDesc &d, const FusedArgs &a, int which, double bytes);
int ffb_fused_pair(Plan &P, const FFBDesc &d, const FusedArgs &a, int which, double bytes);
// the float-float column kernels on the generic Stockham engine, P.ff_threads threads a block
// (fused_ff_generic.cu)
int ff_generic_fused(Plan &P, const FFTDesc &d, const FusedArgs &a, int which, double bytes);

}  // namespace sg
