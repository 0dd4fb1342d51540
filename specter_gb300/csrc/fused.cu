// Host orchestration of the fused RK stage (generic-engine instantiations live here too).
#include <cstring>

#include "fused.h"
#include "fast.h"
#include "fused_launch.cuh"

namespace sg {

struct FusedState {
    StageParams sp;
    void *X1[4] = {nullptr, nullptr, nullptr, nullptr};
    void *X2[4] = {nullptr, nullptr, nullptr, nullptr};
    void *side = nullptr;  // theta rows of the kx = 0 and kx = nx/2 columns [2][ny][nzp]
    int nc = 3;
};

int fused_create(Plan &P, const StageParams &sp, FusedState **out) {
    *out = nullptr;
    FusedState *fs = new FusedState();
    fs->sp = sp;
    fs->nc = sp.solver == 1 ? 4 : 3;
    bool ok = true;
    for (int i = 0; i < fs->nc; i++) {
        ok = ok && cudaMalloc(&fs->X1[i], P.field_bytes()) == cudaSuccess;
        if (sp.ord >= 3) ok = ok && cudaMalloc(&fs->X2[i], P.field_bytes()) == cudaSuccess;
    }
    if (sp.solver == 1) ok = ok && cudaMalloc(&fs->side, 2 * (size_t)P.ny * P.nzp * P.elt()) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fused_destroy(fs);
        set_error("out of device memory (fused stage buffers)");
        return ERR_OOM;
    }
    *out = fs;
    return OK;
}

void fused_destroy(FusedState *fs) {
    if (!fs) return;
    for (int i = 0; i < 4; i++) {
        if (fs->X1[i]) cudaFree(fs->X1[i]);
        if (fs->X2[i]) cudaFree(fs->X2[i]);
    }
    if (fs->side) cudaFree(fs->side);
    delete fs;
}

template <typename T>
static int launch(Plan &P, const FusedArgs &a, int which, double bytes) {
    const int st = fast_fused(P, a, which, bytes);
    if (st != kNoFast) return st;
    return launch_fused<T, GenericFFT<T>>(P, P.tz.d, a, which, bytes);
}

template <typename T>
static int run_stage(Plan &P, FusedState *fs, int o, const void *const vin[4], const void *const cold[4],
                     void *const vout[4], void *pr) {
    const StageParams &sp = fs->sp;
    const bool bouss = sp.solver == 1;
    const void *nl[4] = {nullptr, nullptr, nullptr, nullptr};
    const void *v3[3] = {vin[0], vin[1], vin[2]};
    int st = Ops<T>::nonlinear(P, v3, bouss ? vin[3] : nullptr, nullptr, 0, bouss ? 4 : 3, nl);
    if (st) return st;
    FusedArgs a{};
    for (int i = 0; i < 4; i++) {
        a.nl[i] = nl[i];
        a.vin[i] = vin[i];
        a.cold[i] = cold[i];
        a.vout[i] = vout[i];
    }
    a.pr = pr;
    a.side = fs->side;
    a.dt = sp.dt; a.nu = sp.nu; a.kappa = sp.kappa; a.rmp = 1 / (double)o;
    a.xmom = sp.xmom; a.xtemp = sp.xtemp;
    double tmp = 1 / (double)o;
    if (o != sp.ord) tmp = (double)(o + 1) * tmp;
    a.wall_tmp = tmp;
    a.vb[0] = sp.vzsta[0]; a.vb[1] = sp.vzsta[1]; a.vb[2] = sp.vzend[0]; a.vb[3] = sp.vzend[1];
    a.bouss = bouss ? 1 : 0;
    const double row = (double)P.ny * P.nxh * P.elt();
    // reads: NL (physical rows), vin, cold (+ theta for buoyancy); writes: vout and pr rows
    const double bv = row * (3.0 * P.nzp + (6.0 + (bouss ? 1 : 0)) * P.nz + 3.0 * P.nz + P.nzp);
    if ((st = launch<T>(P, a, kFusedVelocity, bv))) return st;
    if (bouss) {
        const double bt = row * (1.0 * P.nzp + 3.0 * P.nz + 1.0 * P.nz);
        if ((st = launch<T>(P, a, kFusedTheta, bt))) return st;
        if ((st = launch<T>(P, a, kFusedHerm, 4.0 * P.ny * P.nz * P.elt()))) return st;
    }
    return OK;
}

template <typename T>
static int step_impl(Plan &P, FusedState *fs, void *const v[4], void *pr) {
    const int ord = fs->sp.ord;
    void *const *cur = v;
    for (int o = ord; o >= 1; o--) {
        void *const *out;
        if (o == 1 && ord > 1) out = v;
        else out = ((ord - o) % 2 == 0) ? fs->X1 : fs->X2;
        int st = run_stage<T>(P, fs, o, (const void *const *)cur, (const void *const *)v, out, pr);
        if (st) return st;
        cur = out;
    }
    if (ord == 1)
        for (int i = 0; i < fs->nc; i++) cudaMemcpyAsync(v[i], fs->X1[i], P.field_bytes(), cudaMemcpyDeviceToDevice, P.stream);
    return check_launch("fused step");
}

int fused_step(Plan &P, FusedState *fs, void *const v[4], void *pr) {
    return P.prec == FP64 ? step_impl<double>(P, fs, v, pr) : step_impl<float>(P, fs, v, pr);
}

int fused_stage(Plan &P, FusedState *fs, int o, void *const v[4], void *pr, const void *const Cold[4]) {
    const void *vin[4] = {v[0], v[1], v[2], v[3]};
    int st = P.prec == FP64 ? run_stage<double>(P, fs, o, vin, Cold, fs->X1, pr)
                            : run_stage<float>(P, fs, o, vin, Cold, fs->X1, pr);
    if (st) return st;
    for (int i = 0; i < fs->nc; i++) cudaMemcpyAsync(v[i], fs->X1[i], P.field_bytes(), cudaMemcpyDeviceToDevice, P.stream);
    return check_launch("fused stage");
}

}  // namespace sg
