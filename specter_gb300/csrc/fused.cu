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
    void *E[2] = {nullptr, nullptr};  // z spectra of the unit laplace_z profiles, per column
    void *W[3] = {nullptr, nullptr, nullptr};  // split velocity form: updated components
    int nc = 3;
    // nl_fp32 (FP64 plans): the FP32 companion plan of the nonlinear term and the FP32 copy of
    // the stage input it reads
    Plan *nlp = nullptr;
    void *v32[4] = {nullptr, nullptr, nullptr, nullptr};
    // the column kernels of that form compute in float-float: their z FFT tables, and the state
    // (vq, prq) held in float-float inside the RK loop (converted from and to the FP64 fields at
    // the ends of fused_step / fused_stage; cq: the RK step start for fused_stage)
    FFTTable tzq;
    FFBTable ffb;  // the three-step float-float engine's tables, when the z length has them
    void *vq[4] = {nullptr, nullptr, nullptr, nullptr};
    void *cq[4] = {nullptr, nullptr, nullptr, nullptr};
    void *prq = nullptr;
};

// Unit laplace_z profiles on the physical rows (boundary_mod.fpp:635-675 with c1 = 1, c2 = 0
// and c1 = 0, c2 = 1): p1 = exp(kh (z - Lz)), p2 = exp(-kh z); for kx = ky = 0, p1 = z, p2 = 1.
// Rows z >= nzp are zero (the continuation rebuilds them).  FP64.
__global__ void k_unit_profiles(Geo g, double2 *p1, double2 *p2) {
    const size_t n = (size_t)g.nz * g.ny * g.ldx;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int kx = (int)(q % g.ldx), ky = (int)((q / g.ldx) % g.ny), z = (int)(q / ((size_t)g.ldx * g.ny));
        double a = 0, b = 0;
        if (z < g.nzp && kx < g.nxh) {
            const double zz = g.z[z];
            if (kx == 0 && ky == 0) {
                a = zz;
                b = 1.0;
            } else {
                const double kh = sqrt(g.kx[kx] * g.kx[kx] + g.ky[ky] * g.ky[ky]);
                a = exp(kh * (zz - g.Lz));
                b = exp(-(kh * zz));
            }
        }
        p1[q] = make_double2(a, 0.0);
        p2[q] = make_double2(b, 0.0);
    }
}

__global__ void k_narrow(const double2 *src, float2 *dst, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        dst[q] = make_float2((float)src[q].x, (float)src[q].y);
}

// float-float <-> FP64 fields of the nl_fp32 form (in place allowed: both are 16 bytes a
// complex element), once per field per fused_step call, on the FP64 pipe (1.07 and 0.80 ms a
// 512^2 x 538 field; splits by integer operations on the bit patterns measured no faster, their
// fallback for magnitudes outside the float range diverging within warps).
__global__ void k_d2q(const double2 *src, ffc *dst, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double2 v = src[q];
        ffc r;
        r.x = ff_from_double(v.x);
        r.y = ff_from_double(v.y);
        dst[q] = r;
    }
}
__global__ void k_q2d(const ffc *src, double2 *dst, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const ffc v = src[q];
        dst[q] = make_double2(ff_to_double(v.x), ff_to_double(v.y));
    }
}

static int convert(Plan &P, const void *src, void *dst, bool to_ff, const char *what) {
    const size_t n = P.field_elems();
    {
        Launch L_(P, what, 32.0 * n);
        if (to_ff) k_d2q<<<152 * 8, 256, 0, P.stream>>>((const double2 *)src, (ffc *)dst, n);
        else k_q2d<<<152 * 8, 256, 0, P.stream>>>((const ffc *)src, (double2 *)dst, n);
    }
    return check_launch(what);
}

// The harmonic correction of sol_project forward-transforms a(z) = c1 p1 + c2 p2 and
// b(z) = da/dz with FC-Gram continuation.  Continuation and transform are linear, so
// FFT(cont(a)) = c1 E1 + c2 E2 with E_i = FFT(cont(p_i)) fixed by the grid: E1, E2 are computed
// once here, in FP64 (continuation and transform), and stored in the plan's precision; the
// column kernel then forms the corrections without transforming.
static int harmonic_spectra(Plan &P, void *E1, void *E2) {
    FFTTable t64;
    const FFTTable *t = &P.tz;
    if (P.prec != FP64) {
        if (build_fft_table(t64, P.nz, FP64)) { set_error("FFT table construction failed"); return ERR_CUDA; }
        t = &t64;
    }
    const size_t n = P.field_elems();
    double2 *buf = nullptr;
    if (P.prec == FP64) buf = nullptr;
    else if (cudaMalloc(&buf, 2 * n * sizeof(double2)) != cudaSuccess) {
        cudaGetLastError();
        free_fft_table(t64);
        set_error("out of device memory (harmonic spectra)");
        return ERR_OOM;
    }
    double2 *p1 = P.prec == FP64 ? (double2 *)E1 : buf, *p2 = P.prec == FP64 ? (double2 *)E2 : buf + n;
    k_unit_profiles<<<152 * 8, 256, 0, P.stream>>>(P.geo, p1, p2);
    ZFwdArgs a{};
    a.in[0] = p1; a.in[1] = p2; a.out[0] = p1; a.out[1] = p2;
    a.in_scale = 1.0;
    const size_t es = sizeof(double2);
    int tk = 0;
    for (int c : {16, 8, 4, 2, 1})
        if (2 * (size_t)t->d.L * c * es <= 200 * 1024) { tk = c; break; }
    int st = OK;
    if (!tk) { set_error("z length too large for shared memory"); st = ERR_SHAPE; }
    else {
        const size_t sm = 2 * (size_t)t->d.L * tk * es;
        auto k = k_z_forward<double, GenericFFT<double>>;
        if (sm > 40 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k<<<dim3(cdiv(P.nxh, tk), P.ny, 2), kThreads, sm, P.stream>>>(P.geo, t->d, a, tk);
        if (P.prec != FP64) {
            k_narrow<<<152 * 8, 256, 0, P.stream>>>(p1, (float2 *)E1, n);
            k_narrow<<<152 * 8, 256, 0, P.stream>>>(p2, (float2 *)E2, n);
        }
        if (cudaStreamSynchronize(P.stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            set_error("harmonic spectra: CUDA error");
            st = ERR_CUDA;
        }
    }
    if (buf) cudaFree(buf);
    if (P.prec != FP64) free_fft_table(t64);
    return st;
}

int fused_create(Plan &P, const StageParams &sp, FusedState **out) {
    *out = nullptr;
    FusedState *fs = new FusedState();
    fs->sp = sp;
    fs->nc = sp.solver >= 1 ? 4 : 3;
    bool ok = true;
    for (int i = 0; i < fs->nc; i++) {
        ok = ok && cudaMalloc(&fs->X1[i], P.field_bytes()) == cudaSuccess;
        if (sp.ord >= 3) ok = ok && cudaMalloc(&fs->X2[i], P.field_bytes()) == cudaSuccess;
    }
    if (sp.solver == 1) ok = ok && cudaMalloc(&fs->side, 2 * (size_t)P.ny * P.nzp * P.elt()) == cudaSuccess;  // BOUSS only
    for (int i = 0; i < 2; i++) ok = ok && cudaMalloc(&fs->E[i], P.field_bytes()) == cudaSuccess;
    for (int i = 0; i < 3; i++) ok = ok && cudaMalloc(&fs->W[i], P.field_bytes()) == cudaSuccess;
    if (ok && sp.nl_fp32) {
        if (P.prec != FP64) {
            fused_destroy(fs);
            set_error("nl_fp32 needs an FP64 plan");
            return ERR_ARG;
        }
        const int n[3] = {P.nx, P.ny, P.nz}, c[3] = {0, 0, P.cz}, o[3] = {0, 0, P.oz};
        const double len[3] = {P.Lx, P.Ly, P.Lz};
        const int st = plan_create(&fs->nlp, n, c, o, len, P.tdir.c_str(), FP32);
        if (st) {
            fs->nlp = nullptr;
            fused_destroy(fs);
            return st;
        }
        // the companion runs on the owner's stream, so its launches are ordered with the FP64
        // column kernels, captured with them and profiled with them
        cudaStreamSynchronize(fs->nlp->stream);
        cudaStreamDestroy(fs->nlp->stream);
        fs->nlp->stream = P.stream;
        fs->nlp->owner = &P;
        for (int i = 0; i < fs->nc; i++) {
            ok = ok && cudaMalloc(&fs->v32[i], fs->nlp->field_bytes()) == cudaSuccess;
            ok = ok && cudaMalloc(&fs->vq[i], P.field_bytes()) == cudaSuccess;
            ok = ok && cudaMalloc(&fs->cq[i], P.field_bytes()) == cudaSuccess;
        }
        ok = ok && cudaMalloc(&fs->prq, P.field_bytes()) == cudaSuccess;
        if (ok) {
            if (const int st2 = build_ffb_table(fs->ffb, P.nz, P.nzp - P.oz, P.cz + 2 * P.oz)) {
                fused_destroy(fs);
                return st2;
            }
            if (build_fft_table(fs->tzq, P.nz, FF)) {
                fused_destroy(fs);
                set_error("float-float FFT table construction failed");
                return ERR_CUDA;
            }
        }
    }
    if (!ok) {
        cudaGetLastError();
        fused_destroy(fs);
        set_error("out of device memory (fused stage buffers)");
        return ERR_OOM;
    }
    int st = harmonic_spectra(P, fs->E[0], fs->E[1]);
    // the float-float column kernels read the unit-profile spectra in float-float
    for (int i = 0; i < 2 && !st && fs->nlp; i++) st = convert(P, fs->E[i], fs->E[i], true, "spectra_to_ff");
    if (!st && cudaStreamSynchronize(P.stream) != cudaSuccess) st = check_launch("fused stage setup");
    if (st) {
        fused_destroy(fs);
        return st;
    }
    *out = fs;
    return OK;
}

unsigned long long fused_bytes(const Plan &P, const FusedState *fs) {
    if (!fs) return 0;
    unsigned long long b = 0;
    for (int i = 0; i < 4; i++) b += (fs->X1[i] ? P.field_bytes() : 0) + (fs->X2[i] ? P.field_bytes() : 0);
    b += fs->side ? 2ull * P.ny * P.nzp * P.elt() : 0;
    b += (fs->E[0] ? P.field_bytes() : 0) + (fs->E[1] ? P.field_bytes() : 0);
    for (int i = 0; i < 3; i++) b += fs->W[i] ? P.field_bytes() : 0;
    if (fs->nlp) {
        b += plan_bytes(*fs->nlp);
        for (int i = 0; i < 4; i++) {
            b += fs->v32[i] ? fs->nlp->field_bytes() : 0;
            b += (fs->vq[i] ? P.field_bytes() : 0) + (fs->cq[i] ? P.field_bytes() : 0);
        }
        b += fs->prq ? P.field_bytes() : 0;
    }
    return b;
}

void fused_destroy(FusedState *fs) {
    if (!fs) return;
    for (int i = 0; i < 4; i++) {
        if (fs->X1[i]) cudaFree(fs->X1[i]);
        if (fs->X2[i]) cudaFree(fs->X2[i]);
    }
    if (fs->side) cudaFree(fs->side);
    for (int i = 0; i < 2; i++)
        if (fs->E[i]) cudaFree(fs->E[i]);
    for (int i = 0; i < 3; i++)
        if (fs->W[i]) cudaFree(fs->W[i]);
    for (int i = 0; i < 4; i++) {
        if (fs->v32[i]) cudaFree(fs->v32[i]);
        if (fs->vq[i]) cudaFree(fs->vq[i]);
        if (fs->cq[i]) cudaFree(fs->cq[i]);
    }
    if (fs->prq) cudaFree(fs->prq);
    free_fft_table(fs->tzq);
    free_ffb_table(fs->ffb);
    if (fs->nlp) plan_destroy(fs->nlp);
    delete fs;
}

template <typename T>
static int launch(Plan &P, const FusedState *fs, const FusedArgs &a, int which, double bytes) {
    if constexpr (is_ff<T>) {
        // the three-step register engine where the z length has its tables (2.6x the generic
        // engine's transform rate at n = 538), else the generic Stockham engine
        if (fs->ffb.ok && P.ff_engine) {
            FFBDesc d = fs->ffb.d;
            if (!P.ff_zoom) {  // plain round trips (two transforms each)
                d.ztab = nullptr;
                d.L = FFBTab::L;
            }
            return ffb_fused(P, d, a, which, bytes);
        }
        return ff_generic_fused(P, fs->tzq.d, a, which, bytes);
    } else {
        const int st = fast_fused(P, a, which, bytes);
        if (st != kNoFast) return st;
        return launch_fused<T, GenericFFT<T>>(P, P.tz.d, a, which, bytes);
    }
}

template <typename T>
static int run_stage(Plan &P, FusedState *fs, int o, const void *const vin[4], const void *const cold[4],
                     void *const vout[4], void *pr) {
    const StageParams &sp = fs->sp;
    const bool bouss = sp.solver >= 1, rot = sp.solver == 2;
    const void *nl[4] = {nullptr, nullptr, nullptr, nullptr};
    int st = OK;
    if (fs->nlp) {
        // nl_fp32: the nonlinear term in FP32 from an FP32 copy of the stage input
        Plan &Q = *fs->nlp;
        for (int k = 0; k < 3; k++) Q.tile_cap[k] = P.tile_cap[k];  // the autotuned z, y, x caps
        const size_t n = P.field_elems();
        // float-float state: the FP32 z-inverse of the nonlinear term reads it directly (the rounded
        // sum of each pair); an FP64 state is narrowed into the FP32 copies first
        const void *in32[4] = {fs->v32[0], fs->v32[1], fs->v32[2], fs->v32[3]};
        if constexpr (is_ff<T>) {
            Q.nl_input_ff = 1;
            for (int i = 0; i < 4; i++) in32[i] = vin[i];
        } else {
            Q.nl_input_ff = 0;
            for (int i = 0; i < fs->nc; i++) {
                Launch L_(P, "narrow_state", 24.0 * n);
                k_narrow<<<152 * 8, 256, 0, P.stream>>>((const double2 *)vin[i], (float2 *)fs->v32[i], n);
            }
            if ((st = check_launch("narrow_state"))) return st;
        }
        const void *v3[3] = {in32[0], in32[1], in32[2]};
        // the FP32 pipeline finishes the nonlinear term with its forward z transform (with
        // continuation): the FP64 column kernels read spectra and transform only the state
        void *spec[4] = {nullptr, nullptr, nullptr, nullptr};
        for (int c = 0; c < fs->nc; c++)
            if (!(spec[c] = Q.scratch_field(16 + c))) { set_error("out of device memory (NL spectra)"); return ERR_OOM; }
        st = Ops<float>::nonlinear(Q, v3, bouss ? in32[3] : nullptr, spec, 0, bouss ? 4 : 3, nullptr);
        for (int c = 0; c < 4; c++) nl[c] = spec[c];
    } else if constexpr (!is_ff<T>) {
        const void *v3[3] = {vin[0], vin[1], vin[2]};
        st = Ops<T>::nonlinear(P, v3, bouss ? vin[3] : nullptr, nullptr, 0, bouss ? 4 : 3, nl);
    } else {
        set_error("float-float stages need the FP32 companion plan");
        return ERR_STATE;
    }
    if (st) return st;
    FusedArgs a{};
    a.nl32 = fs->nlp ? 1 : 0;
    a.nl_spec = a.nl32;
    for (int i = 0; i < 4; i++) {
        a.nl[i] = nl[i];
        a.vin[i] = vin[i];
        a.cold[i] = cold[i];
        a.vout[i] = vout[i];
    }
    a.pr = pr;
    if constexpr (is_ff<T>)
        if (fs->nlp && fs->nlp->tz4.ok && fs->ffb.ok && P.ff_engine) a.z32 = fs->nlp->tz4.d;
    a.side = fs->side;
    a.hspec[0] = fs->E[0];
    a.hspec[1] = fs->E[1];
    for (int i = 0; i < 3; i++) a.work[i] = fs->W[i];
    a.dt = sp.dt; a.nu = sp.nu; a.kappa = sp.kappa; a.rmp = 1 / (double)o;
    a.xmom = sp.xmom; a.xtemp = sp.xtemp;
    double tmp = 1 / (double)o;
    if (o != sp.ord) tmp = (double)(o + 1) * tmp;
    a.wall_tmp = tmp;
    a.vb[0] = sp.vzsta[0]; a.vb[1] = sp.vzsta[1]; a.vb[2] = sp.vzend[0]; a.vb[3] = sp.vzend[1];
    a.bouss = bouss ? 1 : 0;
    a.rot = rot ? 1 : 0;
    for (int i = 0; i < 3; i++) a.omega[i] = sp.omega[i];
    const double row = (double)P.ny * P.nxh * P.elt();
    // NL rows read per column, in units of plan-precision rows: mixed-domain physical rows, or
    // (nl_fp32) FP32 spectra of all nz rows
    const double nlr = fs->nlp ? 0.5 * P.nz : (double)P.nzp;
    // reads: NL (physical rows), vin, cold (+ theta for buoyancy), the two unit-profile
    // spectra; writes: vout and pr rows
    const double bv = row * (3.0 * nlr + (6.0 + (bouss ? 1 : 0) + 2.0) * P.nz + 3.0 * P.nz + P.nzp);
    if (P.velocity_split) {
        // part 1: NL, vin, cold (+ theta) in, the three updated components out; part 2: those
        // and the unit-profile spectra in, vout and pr rows out
        const double bc = row * (3.0 * nlr + (6.0 + (bouss ? 1 : 0)) * P.nz + 3.0 * P.nz);
        const double bp = row * ((3.0 + 2.0) * P.nz + 3.0 * P.nz + P.nzp);
        if ((st = launch<T>(P, fs, a, kFusedVComp, bc))) return st;
        if ((st = launch<T>(P, fs, a, kFusedVProj, bp))) return st;
    } else if ((st = launch<T>(P, fs, a, kFusedVelocity, bv))) {
        return st;
    }
    if (bouss) {
        const double bt = row * (1.0 * nlr + 3.0 * P.nz + 1.0 * P.nz);
        if ((st = launch<T>(P, fs, a, kFusedTheta, bt))) return st;
        if (!rot && (st = launch<T>(P, fs, a, kFusedHerm, 4.0 * P.ny * P.nz * P.elt()))) return st;
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

int fused_step(Plan &P, FusedState *fs, void *const v[4], void *pr, int nsteps) {
    if (fs->nlp) {
        // nl_fp32: the state in float-float for the whole call
        int st = OK;
        for (int i = 0; i < fs->nc && !st; i++) st = convert(P, v[i], fs->vq[i], true, "state_to_ff");
        if (!st) st = convert(P, pr, fs->prq, true, "state_to_ff");
        for (int t = 0; t < nsteps && !st; t++) st = step_impl<ff>(P, fs, fs->vq, fs->prq);
        for (int i = 0; i < fs->nc && !st; i++) st = convert(P, fs->vq[i], v[i], false, "state_from_ff");
        if (!st) st = convert(P, fs->prq, pr, false, "state_from_ff");
        return st;
    }
    for (int t = 0; t < nsteps; t++) {
        const int st = P.prec == FP64 ? step_impl<double>(P, fs, v, pr) : step_impl<float>(P, fs, v, pr);
        if (st) return st;
    }
    return OK;
}

int fused_stage(Plan &P, FusedState *fs, int o, void *const v[4], void *pr, const void *const Cold[4]) {
    const void *vin[4] = {v[0], v[1], v[2], v[3]};
    int st;
    if (fs->nlp) {
        st = OK;
        for (int i = 0; i < fs->nc && !st; i++) st = convert(P, v[i], fs->vq[i], true, "state_to_ff");
        for (int i = 0; i < fs->nc && !st; i++) st = convert(P, Cold[i], fs->cq[i], true, "state_to_ff");
        if (!st) st = convert(P, pr, fs->prq, true, "state_to_ff");
        const void *vq[4] = {fs->vq[0], fs->vq[1], fs->vq[2], fs->vq[3]};
        const void *cq[4] = {fs->cq[0], fs->cq[1], fs->cq[2], fs->cq[3]};
        if (!st) st = run_stage<ff>(P, fs, o, vq, cq, fs->X1, fs->prq);
        for (int i = 0; i < fs->nc && !st; i++) st = convert(P, fs->X1[i], v[i], false, "state_from_ff");
        if (!st) st = convert(P, fs->prq, pr, false, "state_from_ff");
        return st;
    }
    st = P.prec == FP64 ? run_stage<double>(P, fs, o, vin, Cold, fs->X1, pr)
                        : run_stage<float>(P, fs, o, vin, Cold, fs->X1, pr);
    if (st) return st;
    for (int i = 0; i < fs->nc; i++) cudaMemcpyAsync(v[i], fs->X1[i], P.field_bytes(), cudaMemcpyDeviceToDevice, P.stream);
    return check_launch("fused stage");
}

}  // namespace sg
