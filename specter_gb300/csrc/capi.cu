// C ABI (include/specter_gpu.h): handles, reference-layout conversion, dispatch on precision.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/specter_gpu.h"
#include "batch.h"
#include "fused.h"
#include "handles.h"
#include "ops.h"

using namespace sg;

namespace sg {
const char *last_error();
}

static void plan_release(specter_plan *pl) {
    if (--pl->refs == 0) {
        plan_destroy(pl->p);
        delete pl;
    }
}

struct specter_solver {
    specter_plan *plan;
    StageParams sp;
    int fused;
    specter_field *v[4];   // vx, vy, vz, th
    specter_field *pr;
    void *cold[4];         // RK storage C1, C2, C3, C7
    FusedState *fs;
};

#define CHECK_PLAN(pl)                                                         \
    do {                                                                       \
        if (!(pl) || !(pl)->p) { set_error("null plan"); return SPECTER_ERR_ARG; } \
    } while (0)

static int need(const specter_field *f, const specter_plan *pl, int kind) {
    if (!f || !f->d) { set_error("null field"); return SPECTER_ERR_ARG; }
    if (f->plan != pl) { set_error("field belongs to a different plan"); return SPECTER_ERR_STATE; }
    if (f->kind != kind) { set_error(kind == SPECTER_COMPLEX ? "expected a complex field" : "expected a real field"); return SPECTER_ERR_ARG; }
    return SPECTER_OK;
}
#define NEED(f, k)                                  \
    do {                                            \
        int _s = need((f), plan, (k));              \
        if (_s) return _s;                          \
    } while (0)

#define DISPATCH(plan, call) ((plan)->p->prec == FP64 ? Ops<double>::call : Ops<float>::call)

extern "C" {

const char *specter_last_error(void) { return sg::last_error(); }
int specter_version(void) { return 100; }

int specter_set_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return SPECTER_ERR_CUDA; }
    return SPECTER_OK;
}

int specter_device_count(int *count) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) { *count = 0; set_error(cudaGetErrorString(e)); return SPECTER_ERR_CUDA; }
    *count = n;
    return SPECTER_OK;
}

int specter_table_check(const char *tdir, int C, int d, double out[3]) {
    if (!out) { set_error("null argument"); return SPECTER_ERR_ARG; }
    return table_check(tdir, C, d, out);
}

int specter_device_memory(unsigned long long *free_bytes, unsigned long long *total_bytes) {
    if (!free_bytes || !total_bytes) { set_error("null argument"); return SPECTER_ERR_ARG; }
    size_t f = 0, t = 0;
    cudaError_t e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return SPECTER_ERR_CUDA; }
    *free_bytes = f;
    *total_bytes = t;
    return SPECTER_OK;
}

int specter_plan_create(const int n[3], const int c[3], const int o[3], const double len[3],
                        const char *tdir, int precision, specter_plan **out) {
    if (!n || !c || !o || !len || !out) { set_error("null argument"); return SPECTER_ERR_ARG; }
    *out = nullptr;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev < 1) {
        set_error("no CUDA device: the GB300 path has no CPU fallback");
        return SPECTER_ERR_CUDA;
    }
    Plan *p = nullptr;
    int st = plan_create(&p, n, c, o, len, tdir, precision);
    if (st) return st;
    specter_plan *h = new (std::nothrow) specter_plan{p, 1};
    *out = h;
    return SPECTER_OK;
}

int specter_plan_destroy(specter_plan *plan) {
    if (!plan) return SPECTER_OK;
    plan_release(plan);
    return SPECTER_OK;
}

int specter_plan_info(const specter_plan *plan, int info[8]) {
    CHECK_PLAN(plan);
    const Plan &P = *plan->p;
    int v[8] = {P.nx, P.ny, P.nz, P.cz, P.oz, P.nxh, P.ldx, (int)P.prec};
    memcpy(info, v, sizeof v);
    return SPECTER_OK;
}

int specter_plan_engines(const specter_plan *plan, int out[12]) {
    CHECK_PLAN(plan);
    if (!out) { set_error("null argument"); return SPECTER_ERR_ARG; }
    const Plan &P = *plan->p;
    const FFTTable *gen[3] = {&P.tx, &P.ty, &P.tz};
    const FFT4Table *four[3] = {&P.tx4, &P.ty4, &P.tz4};
    for (int a = 0; a < 3; a++) {
        const bool f = four[a]->ok;
        out[4 * a + 0] = f ? four[a]->d.L : gen[a]->d.L;
        out[4 * a + 1] = f ? four[a]->d.L1 : 0;
        out[4 * a + 2] = f ? four[a]->d.L2 : 0;
        out[4 * a + 3] = f ? four[a]->d.blue : gen[a]->d.blue;
    }
    return SPECTER_OK;
}

int specter_plan_arrays(const specter_plan *plan, double *kx, double *ky, double *kz, double *z, double *dir) {
    CHECK_PLAN(plan);
    const Plan &P = *plan->p;
    if (kx) memcpy(kx, P.kx.data(), sizeof(double) * P.nxh);
    if (ky) memcpy(ky, P.ky.data(), sizeof(double) * P.ny);
    if (kz) memcpy(kz, P.kz.data(), sizeof(double) * P.nz);
    if (z) memcpy(z, P.z.data(), sizeof(double) * P.nz);
    if (dir) memcpy(dir, P.dir.data(), sizeof(double) * P.dir.size());
    return SPECTER_OK;
}

int specter_plan_synchronize(specter_plan *plan) {
    CHECK_PLAN(plan);
    cudaError_t e = cudaStreamSynchronize(plan->p->stream);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return SPECTER_ERR_CUDA; }
    return SPECTER_OK;
}

int specter_plan_stream(specter_plan *plan, void **stream) {
    CHECK_PLAN(plan);
    *stream = (void *)plan->p->stream;
    return SPECTER_OK;
}

// ------------------------------------------------------------------ fields

int specter_field_create(specter_plan *plan, int kind, specter_field **out) {
    CHECK_PLAN(plan);
    if (kind != SPECTER_COMPLEX && kind != SPECTER_REAL) { set_error("bad field kind"); return SPECTER_ERR_ARG; }
    const Plan &P = *plan->p;
    size_t bytes = kind == SPECTER_COMPLEX ? P.field_bytes() : P.real_elems() * P.rel();
    void *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) { cudaGetLastError(); set_error("cudaMalloc failed for a field"); return SPECTER_ERR_OOM; }
    cudaMemsetAsync(d, 0, bytes, P.stream);
    *out = new specter_field{plan, kind, d, bytes};
    plan->refs++;
    return SPECTER_OK;
}

int specter_field_destroy(specter_field *f) {
    if (!f) return SPECTER_OK;
    cudaStreamSynchronize(f->plan->p->stream);
    if (f->d) cudaFree(f->d);
    specter_plan *pl = f->plan;
    delete f;
    plan_release(pl);
    return SPECTER_OK;
}

}  // extern "C"

// reference C(nz, ny, nxh) [z fastest]  <->  device [(z*ny + ky)*ldx + kx]
template <typename V>
__global__ void k_ref_to_dev(const V *__restrict__ h, V *__restrict__ d, int nz, int ny, int nxh, int ldx) {
    __shared__ V tile[32][33];
    const int ky = blockIdx.z;
    const int z0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // r indexes kx, threadIdx.x indexes z
        const int kx = k0 + r, z = z0 + threadIdx.x;
        if (kx < nxh && z < nz) tile[r][threadIdx.x] = h[((size_t)kx * ny + ky) * nz + z];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // r indexes z, threadIdx.x indexes kx
        const int z = z0 + r, kx = k0 + threadIdx.x;
        if (kx < nxh && z < nz) d[((size_t)z * ny + ky) * ldx + kx] = tile[threadIdx.x][r];
    }
}

template <typename V>
__global__ void k_dev_to_ref(const V *__restrict__ d, V *__restrict__ h, int nz, int ny, int nxh, int ldx) {
    __shared__ V tile[32][33];
    const int ky = blockIdx.z;
    const int z0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // r indexes z, threadIdx.x indexes kx
        const int z = z0 + r, kx = k0 + threadIdx.x;
        if (kx < nxh && z < nz) tile[r][threadIdx.x] = d[((size_t)z * ny + ky) * ldx + kx];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // r indexes kx, threadIdx.x indexes z
        const int kx = k0 + r, z = z0 + threadIdx.x;
        if (kx < nxh && z < nz) h[((size_t)kx * ny + ky) * nz + z] = tile[threadIdx.x][r];
    }
}

static constexpr int kStageSlot = 23;  // scratch slots 23, 24: reference-layout staging

static int staging(Plan &P, void **buf, int which = 0) {
    *buf = P.scratch_field(kStageSlot + which);
    if (!*buf) { set_error("out of device memory (staging)"); return SPECTER_ERR_OOM; }
    return SPECTER_OK;
}

static int xfer_init(Plan &P) {
    if (P.copy_stream) return SPECTER_OK;
    if (cudaStreamCreateWithFlags(&P.copy_stream, cudaStreamNonBlocking) != cudaSuccess) return check_launch("copy stream");
    for (cudaEvent_t &e : P.xfer_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return check_launch("copy events");
    return SPECTER_OK;
}

static int convert(Plan &P, const void *src, void *dst, bool to_dev) {
    dim3 grid(cdiv(P.nz, 32), cdiv(P.nxh, 32), P.ny), block(32, 8);
    P.prof_begin(to_dev ? "layout_to_device" : "layout_to_reference", 2.0 * P.nz * P.ny * P.nxh * P.elt());
    struct End { Plan &P; ~End() { P.prof_end(); } } end{P};
    if (P.prec == FP64) {
        if (to_dev) k_ref_to_dev<double2><<<grid, block, 0, P.stream>>>((const double2 *)src, (double2 *)dst, P.nz, P.ny, P.nxh, P.ldx);
        else k_dev_to_ref<double2><<<grid, block, 0, P.stream>>>((const double2 *)src, (double2 *)dst, P.nz, P.ny, P.nxh, P.ldx);
    } else {
        if (to_dev) k_ref_to_dev<float2><<<grid, block, 0, P.stream>>>((const float2 *)src, (float2 *)dst, P.nz, P.ny, P.nxh, P.ldx);
        else k_dev_to_ref<float2><<<grid, block, 0, P.stream>>>((const float2 *)src, (float2 *)dst, P.nz, P.ny, P.nxh, P.ldx);
    }
    return check_launch("layout conversion");
}

extern "C" {

int specter_field_upload(specter_field *f, const void *host) {
    if (!f || !host) { set_error("null argument"); return SPECTER_ERR_ARG; }
    Plan &P = *f->plan->p;
    if (f->kind == SPECTER_REAL) {
        if (cudaMemcpyAsync(f->d, host, f->bytes, cudaMemcpyHostToDevice, P.stream) != cudaSuccess) return check_launch("upload");
        return SPECTER_OK;
    }
    void *stg;
    int st = staging(P, &stg);
    if (st) return st;
    const size_t nbytes = (size_t)P.nz * P.ny * P.nxh * P.elt();
    if (cudaMemcpyAsync(stg, host, nbytes, cudaMemcpyHostToDevice, P.stream) != cudaSuccess) return check_launch("upload");
    return convert(P, stg, f->d, true);
}

// Several fields of one plan: host copies on the plan's copy stream overlap the layout
// conversions on the plan stream, through two staging buffers (xfer_ev[b]: copy into / out of
// buffer b done; xfer_ev[2 + b]: conversion from / into buffer b done).
int specter_fields_upload(int n, specter_field *const *fields, const void *const *hosts) {
    if (n < 1 || !fields || !hosts) { set_error("bad arguments"); return SPECTER_ERR_ARG; }
    for (int i = 0; i < n; i++)
        if (!fields[i] || !hosts[i] || fields[i]->plan != fields[0]->plan) { set_error("fields must share one plan"); return SPECTER_ERR_ARG; }
    Plan &P = *fields[0]->plan->p;
    int st = xfer_init(P);
    if (st) return st;
    cudaEventRecord(P.xfer_ev[2], P.stream);  // earlier work on the plan stream is ordered first
    cudaStreamWaitEvent(P.copy_stream, P.xfer_ev[2], 0);
    for (int i = 0; i < n; i++) {
        specter_field *f = fields[i];
        if (f->kind == SPECTER_REAL) {
            if (cudaMemcpyAsync(f->d, hosts[i], f->bytes, cudaMemcpyHostToDevice, P.copy_stream) != cudaSuccess) return check_launch("upload");
            cudaEventRecord(P.xfer_ev[0], P.copy_stream);
            cudaStreamWaitEvent(P.stream, P.xfer_ev[0], 0);
            continue;
        }
        const int b = i & 1;
        void *stg;
        if ((st = staging(P, &stg, b))) return st;
        if (i >= 2) cudaStreamWaitEvent(P.copy_stream, P.xfer_ev[2 + b], 0);  // conversion i-2 left buffer b
        const size_t nbytes = (size_t)P.nz * P.ny * P.nxh * P.elt();
        if (cudaMemcpyAsync(stg, hosts[i], nbytes, cudaMemcpyHostToDevice, P.copy_stream) != cudaSuccess) return check_launch("upload");
        cudaEventRecord(P.xfer_ev[b], P.copy_stream);
        cudaStreamWaitEvent(P.stream, P.xfer_ev[b], 0);
        if ((st = convert(P, stg, f->d, true))) return st;
        cudaEventRecord(P.xfer_ev[2 + b], P.stream);
    }
    return check_launch("upload");
}

int specter_fields_download(int n, specter_field *const *fields, void *const *hosts) {
    if (n < 1 || !fields || !hosts) { set_error("bad arguments"); return SPECTER_ERR_ARG; }
    for (int i = 0; i < n; i++)
        if (!fields[i] || !hosts[i] || fields[i]->plan != fields[0]->plan) { set_error("fields must share one plan"); return SPECTER_ERR_ARG; }
    Plan &P = *fields[0]->plan->p;
    int st = xfer_init(P);
    if (st) return st;
    for (int i = 0; i < n; i++) {
        specter_field *f = fields[i];
        const int b = i & 1;
        if (f->kind == SPECTER_REAL) {
            cudaEventRecord(P.xfer_ev[2 + b], P.stream);
            cudaStreamWaitEvent(P.copy_stream, P.xfer_ev[2 + b], 0);
            if (cudaMemcpyAsync(hosts[i], f->d, f->bytes, cudaMemcpyDeviceToHost, P.copy_stream) != cudaSuccess) return check_launch("download");
            continue;
        }
        void *stg;
        if ((st = staging(P, &stg, b))) return st;
        if (i >= 2) cudaStreamWaitEvent(P.stream, P.xfer_ev[b], 0);  // copy-out i-2 left buffer b
        if ((st = convert(P, f->d, stg, false))) return st;
        cudaEventRecord(P.xfer_ev[2 + b], P.stream);
        cudaStreamWaitEvent(P.copy_stream, P.xfer_ev[2 + b], 0);
        const size_t nbytes = (size_t)P.nz * P.ny * P.nxh * P.elt();
        if (cudaMemcpyAsync(hosts[i], stg, nbytes, cudaMemcpyDeviceToHost, P.copy_stream) != cudaSuccess) return check_launch("download");
        cudaEventRecord(P.xfer_ev[b], P.copy_stream);
    }
    if (cudaStreamSynchronize(P.copy_stream) != cudaSuccess) return check_launch("download");
    return SPECTER_OK;
}

int specter_field_download(const specter_field *f, void *host) {
    if (!f || !host) { set_error("null argument"); return SPECTER_ERR_ARG; }
    Plan &P = *f->plan->p;
    if (f->kind == SPECTER_REAL) {
        if (cudaMemcpyAsync(host, f->d, f->bytes, cudaMemcpyDeviceToHost, P.stream) != cudaSuccess) return check_launch("download");
    } else {
        void *stg;
        int st = staging(P, &stg);
        if (st) return st;
        if ((st = convert(P, f->d, stg, false))) return st;
        const size_t nbytes = (size_t)P.nz * P.ny * P.nxh * P.elt();
        if (cudaMemcpyAsync(host, stg, nbytes, cudaMemcpyDeviceToHost, P.stream) != cudaSuccess) return check_launch("download");
    }
    if (cudaStreamSynchronize(P.stream) != cudaSuccess) return check_launch("download");
    return SPECTER_OK;
}

int specter_field_copy(specter_field *dst, const specter_field *src) {
    if (!dst || !src || dst->plan != src->plan || dst->kind != src->kind) { set_error("incompatible fields"); return SPECTER_ERR_ARG; }
    cudaMemcpyAsync(dst->d, src->d, dst->bytes, cudaMemcpyDeviceToDevice, dst->plan->p->stream);
    return check_launch("field copy");
}

int specter_field_zero(specter_field *f) {
    if (!f) { set_error("null field"); return SPECTER_ERR_ARG; }
    cudaMemsetAsync(f->d, 0, f->bytes, f->plan->p->stream);
    return check_launch("field zero");
}

int specter_field_device_ptr(specter_field *f, void **ptr, long long *bytes) {
    if (!f) { set_error("null field"); return SPECTER_ERR_ARG; }
    *ptr = f->d;
    if (bytes) *bytes = (long long)f->bytes;
    return SPECTER_OK;
}

// ------------------------------------------------------------------ fftp

int specter_fftp3d_real_to_complex(specter_plan *plan, const specter_field *in, specter_field *out) {
    CHECK_PLAN(plan); NEED(in, SPECTER_REAL); NEED(out, SPECTER_COMPLEX);
    return DISPATCH(plan, fftp3d_r2c(*plan->p, in->d, out->d));
}
int specter_fftp3d_complex_to_real(specter_plan *plan, specter_field *in, specter_field *out) {
    CHECK_PLAN(plan); NEED(in, SPECTER_COMPLEX); NEED(out, SPECTER_REAL);
    return DISPATCH(plan, fftp3d_c2r(*plan->p, in->d, out->d));
}
int specter_fftp2d_real_to_complex_xy(specter_plan *plan, const specter_field *in, specter_field *out) {
    CHECK_PLAN(plan); NEED(in, SPECTER_REAL); NEED(out, SPECTER_COMPLEX);
    return DISPATCH(plan, fftp2d_r2c_xy(*plan->p, in->d, out->d));
}
int specter_fftp2d_complex_to_real_xy(specter_plan *plan, const specter_field *in, specter_field *out) {
    CHECK_PLAN(plan); NEED(in, SPECTER_COMPLEX); NEED(out, SPECTER_REAL);
    return DISPATCH(plan, fftp2d_c2r_xy(*plan->p, in->d, out->d));
}
int specter_fftp1d_real_to_complex_z(specter_plan *plan, specter_field *inout) {
    CHECK_PLAN(plan); NEED(inout, SPECTER_COMPLEX);
    return DISPATCH(plan, fftp1d_r2c_z(*plan->p, inout->d));
}
int specter_fftp1d_complex_to_real_z(specter_plan *plan, specter_field *inout) {
    CHECK_PLAN(plan); NEED(inout, SPECTER_COMPLEX);
    return DISPATCH(plan, fftp1d_c2r_z(*plan->p, inout->d));
}

// ------------------------------------------------------------------ pseudo

int specter_derivk(specter_plan *plan, const specter_field *a, specter_field *b, int dir) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX);
    return DISPATCH(plan, derivk(*plan->p, a->d, b->d, dir));
}
int specter_laplak(specter_plan *plan, const specter_field *a, specter_field *b) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX);
    return DISPATCH(plan, laplak(*plan->p, a->d, b->d));
}
int specter_curlk(specter_plan *plan, const specter_field *a, const specter_field *b, specter_field *c, int dir) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    return DISPATCH(plan, curlk(*plan->p, a->d, b->d, c->d, dir));
}
int specter_gradre(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                   specter_field *d, specter_field *e, specter_field *f) {
    CHECK_PLAN(plan);
    NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    NEED(d, SPECTER_COMPLEX); NEED(e, SPECTER_COMPLEX); NEED(f, SPECTER_COMPLEX);
    const void *v[3] = {a->d, b->d, c->d};
    void *out[4] = {d->d, e->d, f->d, nullptr};
    return DISPATCH(plan, nonlinear(*plan->p, v, nullptr, out, 0, 3));
}
int specter_advect(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                   const specter_field *d, specter_field *e) {
    CHECK_PLAN(plan);
    NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    NEED(d, SPECTER_COMPLEX); NEED(e, SPECTER_COMPLEX);
    const void *v[3] = {a->d, b->d, c->d};
    void *out[4] = {nullptr, nullptr, nullptr, e->d};
    return DISPATCH(plan, nonlinear(*plan->p, v, d->d, out, 3, 4));
}
int specter_fc_filter(specter_plan *plan, specter_field *a) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX);
    return DISPATCH(plan, fc_filter(*plan->p, a->d));
}
int specter_energy(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                   int kin, double *out) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    return DISPATCH(plan, energy(*plan->p, a->d, b->d, c->d, kin, out));
}
int specter_helicity(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                     double *out) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    return DISPATCH(plan, helicity(*plan->p, a->d, b->d, c->d, out));
}
int specter_cross(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                  const specter_field *d, const specter_field *e, const specter_field *f, int kin, double *out) {
    CHECK_PLAN(plan);
    NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    NEED(d, SPECTER_COMPLEX); NEED(e, SPECTER_COMPLEX); NEED(f, SPECTER_COMPLEX);
    const void *A[3] = {a->d, b->d, c->d}, *B[3] = {d->d, e->d, f->d};
    return DISPATCH(plan, cross(*plan->p, A, B, kin, out));
}
int specter_divergence(specter_plan *plan, const specter_field *a, const specter_field *b, const specter_field *c,
                       double *out) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX);
    return DISPATCH(plan, divergence(*plan->p, a->d, b->d, c->d, out));
}
int specter_variance(specter_plan *plan, const specter_field *a, int kin, double *out) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX);
    return DISPATCH(plan, variance(*plan->p, a->d, kin, out));
}
int specter_product(specter_plan *plan, const specter_field *a, const specter_field *b, double *out) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX);
    return DISPATCH(plan, product(*plan->p, a->d, b->d, out));
}

// ------------------------------------------------------------------ boundary

int specter_bouncheck_z(specter_plan *plan, const specter_field *a, const specter_field *b, double *bot, double *top) {
    CHECK_PLAN(plan); NEED(a, SPECTER_COMPLEX);
    if (b) NEED(b, SPECTER_COMPLEX);
    return DISPATCH(plan, bouncheck_z(*plan->p, a->d, b ? b->d : nullptr, bot, top));
}
int specter_sol_project(specter_plan *plan, specter_field *a, specter_field *b, specter_field *c, specter_field *d,
                        int bctarget, int bczsta, int bczend) {
    CHECK_PLAN(plan);
    NEED(a, SPECTER_COMPLEX); NEED(b, SPECTER_COMPLEX); NEED(c, SPECTER_COMPLEX); NEED(d, SPECTER_COMPLEX);
    if (bczsta != 0 || bczend != 0) {
        set_error("[ERROR] Unsupported BC kind in call to sol_project (only homogeneous Dirichlet walls)");
        return SPECTER_ERR_BC;
    }
    return DISPATCH(plan, sol_project(*plan->p, a->d, b->d, c->d, d->d, bctarget));
}
int specter_v_imposebc_and_project(specter_plan *plan, specter_field *vx, specter_field *vy, specter_field *vz,
                                   specter_field *pr, int rki, int ord, const double v_zsta[2], const double v_zend[2]) {
    CHECK_PLAN(plan);
    NEED(vx, SPECTER_COMPLEX); NEED(vy, SPECTER_COMPLEX); NEED(vz, SPECTER_COMPLEX); NEED(pr, SPECTER_COMPLEX);
    const double zero[2] = {0.0, 0.0};
    return DISPATCH(plan, v_imposebc_and_project(*plan->p, vx->d, vy->d, vz->d, pr->d, rki, ord,
                                                 v_zsta ? v_zsta : zero, v_zend ? v_zend : zero));
}
int specter_s_imposebc(specter_plan *plan, specter_field *th) {
    CHECK_PLAN(plan); NEED(th, SPECTER_COMPLEX);
    return DISPATCH(plan, s_imposebc(*plan->p, th->d));
}

// ------------------------------------------------------------------ solver

int specter_solver_create(specter_plan *plan, const specter_solver_params *p, specter_solver **out) {
    CHECK_PLAN(plan);
    if (!p || !out) { set_error("null argument"); return SPECTER_ERR_ARG; }
    if ((p->solver != SPECTER_HD && p->solver != SPECTER_BOUSS && p->solver != SPECTER_ROTBOUSS) || p->ord < 1) {
        set_error("bad solver parameters");
        return SPECTER_ERR_ARG;
    }
    specter_solver *s = new specter_solver();  // value-initialised: all handles null
    s->plan = plan;
    plan->refs++;
    s->sp.solver = p->solver;
    s->sp.ord = p->ord;
    s->sp.dt = p->dt; s->sp.nu = p->nu; s->sp.kappa = p->kappa;
    s->sp.xmom = p->xmom * p->gama; s->sp.xtemp = p->xtemp * p->gama;
    s->sp.vzsta[0] = p->v_zsta[0]; s->sp.vzsta[1] = p->v_zsta[1];
    s->sp.vzend[0] = p->v_zend[0]; s->sp.vzend[1] = p->v_zend[1];
    for (int i = 0; i < 3; i++) s->sp.omega[i] = p->solver == SPECTER_ROTBOUSS ? p->omega[i] : 0.0;
    s->fused = p->fused;
    s->sp.nl_fp32 = p->nl_fp32 ? 1 : 0;
    if (s->sp.nl_fp32 && (!p->fused || plan->p->prec != FP64)) {
        set_error("nl_fp32 needs a fused solver on an FP64 plan");
        delete s;
        plan_release(plan);
        return SPECTER_ERR_ARG;
    }
    const int nc = p->solver == SPECTER_HD ? 3 : 4;
    int st = SPECTER_OK;
    for (int i = 0; i < 4 && !st; i++) {
        s->v[i] = nullptr;
        if (i < nc) st = specter_field_create(plan, SPECTER_COMPLEX, &s->v[i]);
    }
    if (!st) st = specter_field_create(plan, SPECTER_COMPLEX, &s->pr);
    for (int i = 0; i < 4 && !st; i++) {
        s->cold[i] = nullptr;
        if (i < nc && cudaMalloc(&s->cold[i], plan->p->field_bytes()) != cudaSuccess) { set_error("cudaMalloc failed"); st = SPECTER_ERR_OOM; }
    }
    s->fs = nullptr;
    if (!st && s->fused) st = fused_create(*plan->p, s->sp, &s->fs);
    if (st) { specter_solver_destroy(s); return st; }
    *out = s;
    return SPECTER_OK;
}

int specter_solver_destroy(specter_solver *s) {
    if (!s) return SPECTER_OK;
    cudaStreamSynchronize(s->plan->p->stream);
    for (int i = 0; i < 4; i++) { specter_field_destroy(s->v[i]); if (s->cold[i]) cudaFree(s->cold[i]); }
    specter_field_destroy(s->pr);
    if (s->fs) fused_destroy(s->fs);
    specter_plan *pl = s->plan;
    delete s;
    plan_release(pl);
    return SPECTER_OK;
}

int specter_solver_fields(specter_solver *s, specter_field **vx, specter_field **vy, specter_field **vz,
                          specter_field **th, specter_field **pr) {
    if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
    if (vx) *vx = s->v[0];
    if (vy) *vy = s->v[1];
    if (vz) *vz = s->v[2];
    if (th) *th = s->v[3];
    if (pr) *pr = s->pr;
    return SPECTER_OK;
}

}  // extern "C"

static int stage_ref(specter_solver *s, int o) {
    Plan &P = *s->plan->p;
    void *v[4] = {s->v[0]->d, s->v[1]->d, s->v[2]->d, s->v[3] ? s->v[3]->d : nullptr};
    const void *C[4] = {s->cold[0], s->cold[1], s->cold[2], s->cold[3]};
    return P.prec == FP64 ? Ops<double>::stage(P, s->sp, o, v, s->pr->d, C) : Ops<float>::stage(P, s->sp, o, v, s->pr->d, C);
}

extern "C" {

int specter_solver_stage(specter_solver *s, int o) {
    if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
    if (o < 1 || o > s->sp.ord) { set_error("stage index o must be in [1, ord]"); return SPECTER_ERR_ARG; }
    if (s->fused) {
        void *v[4] = {s->v[0]->d, s->v[1]->d, s->v[2]->d, s->v[3] ? s->v[3]->d : nullptr};
        const void *C[4] = {s->cold[0], s->cold[1], s->cold[2], s->cold[3]};
        return fused_stage(*s->plan->p, s->fs, o, v, s->pr->d, C);
    }
    return stage_ref(s, o);
}

int specter_solver_step(specter_solver *s, int nsteps) {
    if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
    Plan &P = *s->plan->p;
    const int nc = s->sp.solver == SPECTER_HD ? 3 : 4;
    if (s->fused) {
        void *v[4] = {s->v[0]->d, s->v[1]->d, s->v[2]->d, s->v[3] ? s->v[3]->d : nullptr};
        return fused_step(P, s->fs, v, s->pr->d, nsteps);
    }
    for (int t = 0; t < nsteps; t++) {
        // rkstep1: C_i = v_i (hd_rkstep1.f90:4-6, bouss_rkstep1.f90:4-7)
        for (int i = 0; i < nc; i++)
            cudaMemcpyAsync(s->cold[i], s->v[i]->d, P.field_bytes(), cudaMemcpyDeviceToDevice, P.stream);
        int st = check_launch("rkstep1");
        if (st) return st;
        for (int o = s->sp.ord; o >= 1; o--) {
            st = specter_solver_stage(s, o);
            if (st) return st;
        }
    }
    return SPECTER_OK;
}

int specter_solver_check(specter_solver *s) {
    if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
    Plan &P = *s->plan->p;
    const int nc = s->sp.solver == SPECTER_HD ? 3 : 4;
    for (int i = 0; i < nc; i++) {
        double e = 0.0;
        int st = P.prec == FP64 ? Ops<double>::variance(P, s->v[i]->d, 1, &e) : Ops<float>::variance(P, s->v[i]->d, 1, &e);
        if (st) return st;
        if (!(e == e) || e > 1e300) { set_error("non-finite value in the solver state"); return SPECTER_ERR_NONFINITE; }
    }
    return SPECTER_OK;
}

// ------------------------------------------------------------------ autotuning, graphs

}  // extern "C"

// Device copies of a solver's state (velocity, theta, pressure) around trial steps.
struct StateCopy {
    std::vector<std::pair<void *, void *>> pairs;  // (state field, copy)
    int take(specter_solver *s) {
        Plan &P = *s->plan->p;
        specter_field *f[5] = {s->v[0], s->v[1], s->v[2], s->v[3], s->pr};
        for (specter_field *x : f) {
            if (!x) continue;
            void *c = nullptr;
            if (cudaMalloc(&c, x->bytes) != cudaSuccess) { cudaGetLastError(); release(); set_error("cudaMalloc failed"); return SPECTER_ERR_OOM; }
            cudaMemcpyAsync(c, x->d, x->bytes, cudaMemcpyDeviceToDevice, P.stream);
            pairs.push_back({x->d, c});
        }
        return check_launch("state copy");
    }
    int put_back(specter_solver *s) {
        Plan &P = *s->plan->p;
        size_t i = 0;
        specter_field *f[5] = {s->v[0], s->v[1], s->v[2], s->v[3], s->pr};
        for (specter_field *x : f) {
            if (!x) continue;
            cudaMemcpyAsync(pairs[i].first, pairs[i].second, x->bytes, cudaMemcpyDeviceToDevice, P.stream);
            i++;
        }
        cudaStreamSynchronize(P.stream);
        return check_launch("state restore");
    }
    void release() {
        for (auto &p : pairs) cudaFree(p.second);
        pairs.clear();
    }
};

extern "C" {

int specter_plan_tile_caps(specter_plan *plan, const int caps[4]) {
    CHECK_PLAN(plan);
    if (!caps) { set_error("null argument"); return SPECTER_ERR_ARG; }
    for (int i = 0; i < 4; i++)
        if (caps[i] > 0) plan->p->tile_cap[i] = caps[i];
    return SPECTER_OK;
}

int specter_plan_set_option(specter_plan *plan, const char *name, int value) {
    CHECK_PLAN(plan);
    if (!name) { set_error("null option name"); return SPECTER_ERR_ARG; }
    Plan &P = *plan->p;
    if (!strcmp(name, "velocity_split")) { P.velocity_split = value ? 1 : 0; return SPECTER_OK; }
    if (!strcmp(name, "ff_engine")) { P.ff_engine = value ? 1 : 0; return SPECTER_OK; }
    if (!strcmp(name, "ff_pair_proj")) { P.ff_pair_proj = value ? 1 : 0; return SPECTER_OK; }
    if (!strcmp(name, "ff_pair_cols")) { P.ff_pair_cols = value ? 1 : 0; return SPECTER_OK; }
    if (!strcmp(name, "ff_zoom")) { P.ff_zoom = value ? 1 : 0; return SPECTER_OK; }
    if (!strcmp(name, "ff_threads")) {
        if (value != 256 && value != 384) { set_error("ff_threads is 256 or 384"); return SPECTER_ERR_ARG; }
        P.ff_threads = value;
        return SPECTER_OK;
    }
    const char *caps[4] = {"tile_cap_z", "tile_cap_y", "tile_cap_x", "tile_cap_fused"};
    for (int i = 0; i < 4; i++)
        if (!strcmp(name, caps[i])) {
            if (value < 1 || value > 16 || (value & (value - 1))) { set_error("tile caps are powers of two in [1, 16]"); return SPECTER_ERR_ARG; }
            P.tile_cap[i] = value;
            return SPECTER_OK;
        }
    set_error(std::string("unknown plan option ") + name);
    return SPECTER_ERR_ARG;
}

int specter_plan_get_option(specter_plan *plan, const char *name, int *value) {
    CHECK_PLAN(plan);
    if (!name || !value) { set_error("null argument"); return SPECTER_ERR_ARG; }
    const Plan &P = *plan->p;
    const struct { const char *n; int v; } opts[] = {
        {"velocity_split", P.velocity_split}, {"ff_threads", P.ff_threads}, {"ff_engine", P.ff_engine},
        {"ff_pair_proj", P.ff_pair_proj},     {"ff_pair_cols", P.ff_pair_cols}, {"ff_zoom", P.ff_zoom},
        {"tile_cap_z", P.tile_cap[0]},
        {"tile_cap_y", P.tile_cap[1]},        {"tile_cap_x", P.tile_cap[2]},   {"tile_cap_fused", P.tile_cap[3]}};
    for (const auto &o : opts)
        if (!strcmp(name, o.n)) { *value = o.v; return SPECTER_OK; }
    set_error(std::string("unknown plan option ") + name);
    return SPECTER_ERR_ARG;
}

int specter_solver_autotune(specter_solver *s, int caps[5]) {
    if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
    Plan &P = *s->plan->p;
    if (P.profile) { set_error("autotune with profiling enabled"); return SPECTER_ERR_STATE; }
    StateCopy snap;
    int st = snap.take(s);
    if (st) return st;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // time of two RK steps after one warm-up step at the current caps (infinite on error)
    auto trial = [&]() -> float {
        if (specter_solver_step(s, 1)) { cudaGetLastError(); return 1e30f; }
        cudaEventRecord(e0, P.stream);
        if (specter_solver_step(s, 2)) { cudaGetLastError(); return 1e30f; }
        cudaEventRecord(e1, P.stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) { cudaGetLastError(); return 1e30f; }
        float ms = 1e30f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    for (int kind = 0; kind < 4; kind++) {
        int best = P.tile_cap[kind];
        float best_ms = trial();
        for (int cap : {16, 8, 4, 2}) {
            if (cap == best) continue;
            P.tile_cap[kind] = cap;
            const float ms = trial();
            if (ms < best_ms) { best_ms = ms; best = cap; }
        }
        P.tile_cap[kind] = best;
        // the state was advanced by the trials: bring it back before the next family
        if ((st = snap.put_back(s))) break;
    }
    if (!st && s->fused) {  // fused velocity stage: two kernels or one
        const int keep = P.velocity_split;
        const float ms_keep = trial();
        P.velocity_split = !keep;
        const float ms_other = trial();
        if (!(ms_other < ms_keep)) P.velocity_split = keep;
        st = snap.put_back(s);
    }
    if (!st && s->fused && s->sp.nl_fp32) {  // block shapes of the float-float column kernels
        int *opt[3] = {&P.ff_threads, &P.ff_pair_proj, &P.ff_pair_cols};
        for (int i = 0; i < 3 && !st; i++) {
            const int keep = *opt[i];
            const float ms_keep = trial();
            *opt[i] = i == 0 ? (keep == 384 ? 256 : 384) : !keep;
            const float ms_other = trial();
            if (!(ms_other < ms_keep)) *opt[i] = keep;
            st = snap.put_back(s);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!st) st = snap.put_back(s);
    snap.release();
    if (!st && caps) {
        for (int i = 0; i < 4; i++) caps[i] = P.tile_cap[i];
        caps[4] = P.velocity_split;
    }
    return st;
}

}  // extern "C"

struct specter_graph {
    cudaStream_t root = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> streams;  // distinct plan streams of the captured solvers
    std::vector<cudaEvent_t> ev;        // one per stream (join at capture, entry at launch)
    cudaEvent_t fork = nullptr, done = nullptr;
    long long kernels = 0;
};

extern "C" {

int specter_graph_destroy(specter_graph *g) {
    if (!g) return SPECTER_OK;
    if (g->root) cudaStreamSynchronize(g->root);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    for (cudaEvent_t e : g->ev) cudaEventDestroy(e);
    if (g->fork) cudaEventDestroy(g->fork);
    if (g->done) cudaEventDestroy(g->done);
    if (g->root) cudaStreamDestroy(g->root);
    delete g;
    return SPECTER_OK;
}

int specter_graph_create(specter_solver *const *solvers, int n, int nsteps, specter_graph **out) {
    if (!solvers || n < 1 || nsteps < 1 || !out) { set_error("bad graph arguments"); return SPECTER_ERR_ARG; }
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!solvers[i]) { set_error("null solver"); return SPECTER_ERR_ARG; }
        if (solvers[i]->plan->p->profile) { set_error("graph capture with profiling enabled"); return SPECTER_ERR_STATE; }
    }
    // one trial step per solver (state restored) creates every lazily allocated buffer and
    // uploads every table, so that the capture records kernels and copies only
    for (int i = 0; i < n; i++) {
        StateCopy snap;
        int st = snap.take(solvers[i]);
        if (!st) st = specter_solver_step(solvers[i], 1);
        if (!st) st = snap.put_back(solvers[i]);
        snap.release();
        if (st) return st;
    }
    specter_graph *g = new specter_graph();
    for (int i = 0; i < n; i++) {
        cudaStream_t s = solvers[i]->plan->p->stream;
        bool seen = false;
        for (cudaStream_t t : g->streams) seen = seen || t == s;
        if (!seen) g->streams.push_back(s);
    }
    cudaStreamCreateWithFlags(&g->root, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
    g->ev.resize(g->streams.size());
    for (auto &e : g->ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    int st = SPECTER_OK;
    if (cudaStreamBeginCapture(g->root, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        st = check_launch("graph capture");
        specter_graph_destroy(g);
        return st ? st : SPECTER_ERR_CUDA;
    }
    cudaEventRecord(g->fork, g->root);
    for (cudaStream_t s : g->streams) cudaStreamWaitEvent(s, g->fork, 0);
    for (int i = 0; i < n && !st; i++) {
        Plan &P = *solvers[i]->plan->p;
        const long long l0 = P.launches;
        st = specter_solver_step(solvers[i], nsteps);
        g->kernels += P.launches - l0;
    }
    for (size_t j = 0; j < g->streams.size(); j++) {
        cudaEventRecord(g->ev[j], g->streams[j]);
        cudaStreamWaitEvent(g->root, g->ev[j], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(g->root, &graph);
    g->graph = graph;
    if (!st && ec != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(ec)); st = SPECTER_ERR_CUDA; }
    if (!st && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) {
        set_error("graph instantiation failed");
        st = SPECTER_ERR_CUDA;
    }
    cudaGetLastError();
    if (st) { specter_graph_destroy(g); return st; }
    *out = g;
    return SPECTER_OK;
}

int specter_graph_launch(specter_graph *g) {
    if (!g || !g->exec) { set_error("null graph"); return SPECTER_ERR_ARG; }
    for (size_t j = 0; j < g->streams.size(); j++) {
        cudaEventRecord(g->ev[j], g->streams[j]);
        cudaStreamWaitEvent(g->root, g->ev[j], 0);
    }
    if (cudaGraphLaunch(g->exec, g->root) != cudaSuccess) return check_launch("graph launch");
    cudaEventRecord(g->done, g->root);
    for (cudaStream_t s : g->streams) cudaStreamWaitEvent(s, g->done, 0);
    return check_launch("graph launch");
}

int specter_graph_synchronize(specter_graph *g) {
    if (!g) { set_error("null graph"); return SPECTER_ERR_ARG; }
    if (cudaStreamSynchronize(g->root) != cudaSuccess) return check_launch("graph synchronize");
    return SPECTER_OK;
}

int specter_graph_query(specter_graph *g, int *done) {
    if (!g || !done) { set_error("null argument"); return SPECTER_ERR_ARG; }
    const cudaError_t e = cudaStreamQuery(g->root);
    if (e == cudaSuccess) { *done = 1; return SPECTER_OK; }
    if (e == cudaErrorNotReady) { cudaGetLastError(); *done = 0; return SPECTER_OK; }
    return check_launch("graph query");
}

int specter_solver_memory(specter_solver *s, unsigned long long *bytes) {
    if (!s || !bytes) { set_error("null argument"); return SPECTER_ERR_ARG; }
    const Plan &P = *s->plan->p;
    const int nc = s->sp.solver == SPECTER_HD ? 3 : 4;
    unsigned long long b = 0;
    b += (unsigned long long)(2 * nc + 1) * P.field_bytes();  // state, pr, RK start
    b += fused_bytes(P, s->fs);
    b += plan_bytes(P);
    *bytes = b;
    return SPECTER_OK;
}

int specter_graph_kernels(specter_graph *g, long long *kernels) {
    if (!g || !kernels) { set_error("null argument"); return SPECTER_ERR_ARG; }
    *kernels = g->kernels;
    return SPECTER_OK;
}

int specter_timers(specter_plan *plan, double out[6]) {
    CHECK_PLAN(plan);
    for (int i = 0; i < 6; i++) out[i] = plan->p->timers[i];
    return SPECTER_OK;
}

int specter_timers_reset(specter_plan *plan) {
    CHECK_PLAN(plan);
    for (int i = 0; i < 6; i++) plan->p->timers[i] = 0.0;
    return SPECTER_OK;
}

int specter_profile(specter_plan *plan, int enable) {
    CHECK_PLAN(plan);
    Plan &P = *plan->p;
    P.prof_flush();
    P.agg.clear();
    P.profile = enable != 0;
    return SPECTER_OK;
}

int specter_profile_report(specter_plan *plan, char *buf, int buflen) {
    CHECK_PLAN(plan);
    Plan &P = *plan->p;
    P.prof_flush();
    std::string out;
    char line[256];
    for (const Plan::Agg &g : P.agg) {
        snprintf(line, sizeof line, "%s %lld %.6f %.0f\n", g.name.c_str(), g.n, g.ms, g.bytes);
        out += line;
    }
    if (!buf || buflen <= (int)out.size()) { set_error("report buffer too small"); return SPECTER_ERR_ARG; }
    memcpy(buf, out.c_str(), out.size() + 1);
    return SPECTER_OK;
}

int specter_launch_count(specter_plan *plan, long long *count) {
    CHECK_PLAN(plan);
    *count = plan->p->launches;
    return SPECTER_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batched ensembles

// One RK step of several solvers as a sequence of batched launches (batch.h), captured once as a
// CUDA graph: position i of the sequence is the i-th kernel of every solver's step, launched once
// per distinct kernel (template instance and shared memory) over all the solvers that use it.
struct specter_batch {
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *recs = nullptr;  // every record, device
    long long kernels = 0;
    std::vector<specter_solver *> solvers;
};

extern "C" {

int specter_batch_destroy(specter_batch *b) {
    if (!b) return SPECTER_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->recs) cudaFree(b->recs);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SPECTER_OK;
}

int specter_batch_create(specter_solver *const *solvers, int n, specter_batch **out) {
    if (!solvers || n < 1 || !out) { set_error("bad batch arguments"); return SPECTER_ERR_ARG; }
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        specter_solver *s = solvers[i];
        if (!s) { set_error("null solver"); return SPECTER_ERR_ARG; }
        const Plan &P = *s->plan->p;
        if (!s->fused || P.prec != FP32 || s->sp.solver != SPECTER_HD || s->sp.ord < 2 || s->sp.nl_fp32) {
            set_error("batched ensembles take fused FP32 HD solvers of RK order >= 2");
            return SPECTER_ERR_ARG;
        }
        if (P.profile) { set_error("batch with profiling enabled"); return SPECTER_ERR_STATE; }
        for (int j = 0; j < i; j++)
            if (solvers[j]->plan == s->plan) {  // their scratch fields would be shared within a launch
                set_error("batched solvers need plans of their own");
                return SPECTER_ERR_ARG;
            }
    }
    // record one RK step of every solver (the split velocity form: its two kernels batch)
    std::vector<Batch> rec(n);
    int st = SPECTER_OK;
    for (int i = 0; i < n && !st; i++) {
        Plan &P = *solvers[i]->plan->p;
        cudaStreamSynchronize(P.stream);
        P.velocity_split = 1;
        P.batch = &rec[i];
        void *v[4] = {solvers[i]->v[0]->d, solvers[i]->v[1]->d, solvers[i]->v[2]->d, nullptr};
        st = fused_step(P, solvers[i]->fs, v, solvers[i]->pr->d, 1);
        P.batch = nullptr;
        if (!st && rec[i].unbatchable) {
            set_error(std::string("batch: launch without a batched form: ") + rec[i].unbatchable);
            st = SPECTER_ERR_STATE;
        }
        if (!st && (rec[i].entries.size() != rec[0].entries.size())) {
            set_error("batch: the solvers' steps have different kernel sequences");
            st = SPECTER_ERR_STATE;
        }
        for (size_t k = 0; !st && k < rec[i].entries.size(); k++)
            if (strcmp(rec[i].entries[k].name, rec[0].entries[k].name)) {
                set_error("batch: the solvers' steps have different kernel sequences");
                st = SPECTER_ERR_STATE;
            }
    }
    if (st) return st;
    // group each position by (kernel, shared memory); lay every group's records out contiguously
    struct Group { const BatchEntry *proto; size_t off; int n, blocks; };
    std::vector<Group> seq;
    std::vector<unsigned char> host;
    const size_t npos = rec[0].entries.size();
    for (size_t k = 0; k < npos; k++) {
        std::vector<int> used(n, 0);
        for (int i = 0; i < n; i++) {
            if (used[i]) continue;
            const BatchEntry &e0 = rec[i].entries[k];
            Group g{&e0, 0, 0, 0};
            const size_t rsz = e0.rec.size();
            host.resize((host.size() + 255) / 256 * 256);  // 256-byte aligned group start
            g.off = host.size();
            for (int j = i; j < n; j++) {
                const BatchEntry &e = rec[j].entries[k];
                if (used[j] || e.key != e0.key || e.smem != e0.smem || e.rec.size() != rsz) continue;
                used[j] = 1;
                const size_t at = host.size();
                host.insert(host.end(), e.rec.begin(), e.rec.end());
                BatchGrid *gr = (BatchGrid *)(host.data() + at);
                gr->block0 = g.blocks;
                g.blocks += e.blocks;
                g.n++;
            }
            seq.push_back(g);
        }
    }
    specter_batch *b = new specter_batch();
    b->solvers.assign(solvers, solvers + n);
    if (cudaMalloc(&b->recs, host.size()) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        set_error("out of device memory (batch records)");
        return SPECTER_ERR_OOM;
    }
    cudaMemcpy(b->recs, host.data(), host.size(), cudaMemcpyHostToDevice);
    cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    // the shared-memory limit is a per-kernel attribute: set each kernel's largest use once (a
    // kernel appears at several positions with different tile sizes)
    std::vector<std::pair<const BatchEntry *, size_t>> limits;
    for (const Group &g : seq) {
        bool found = false;
        for (auto &l : limits)
            if (l.first->key == g.proto->key) { l.second = std::max(l.second, g.proto->smem); found = true; }
        if (!found) limits.push_back({g.proto, g.proto->smem});
    }
    for (auto &l : limits) l.first->launch(nullptr, 0, 0, l.second, b->stream, true);
    if ((st = check_launch("batch kernel attributes"))) {
        specter_batch_destroy(b);
        return st;
    }
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        st = check_launch("batch capture");
        specter_batch_destroy(b);
        return st ? st : SPECTER_ERR_CUDA;
    }
    for (const Group &g : seq) {
        g.proto->launch((const unsigned char *)b->recs + g.off, g.n, g.blocks, g.proto->smem, b->stream, false);
        b->kernels++;
        const cudaError_t el = cudaPeekAtLastError();
        if (el != cudaSuccess && !st) {
            set_error(std::string("batch capture: ") + g.proto->name + " (" + std::to_string(g.n) + " instances, " +
                      std::to_string(g.blocks) + " blocks, " + std::to_string(g.proto->smem) + " B smem): " +
                      cudaGetErrorString(el));
            st = SPECTER_ERR_CUDA;
        }
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
    b->graph = graph;
    if (ec != cudaSuccess && !st) { set_error(std::string("batch capture: ") + cudaGetErrorString(ec)); st = SPECTER_ERR_CUDA; }
    if (!st && cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
        set_error("batch graph instantiation failed");
        st = SPECTER_ERR_CUDA;
    }
    cudaGetLastError();
    if (st) { specter_batch_destroy(b); return st; }
    *out = b;
    return SPECTER_OK;
}

int specter_batch_step(specter_batch *b, int nsteps) {
    if (!b || nsteps < 0) { set_error("bad batch arguments"); return SPECTER_ERR_ARG; }
    // work queued on the solvers' own streams (initial fields, earlier steps) comes first
    for (specter_solver *s : b->solvers) cudaStreamSynchronize(s->plan->p->stream);
    for (int t = 0; t < nsteps; t++)
        if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) return check_launch("batch launch");
    return check_launch("batch launch");
}

int specter_batch_synchronize(specter_batch *b) {
    if (!b) { set_error("null batch"); return SPECTER_ERR_ARG; }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return check_launch("batch synchronize");
    return SPECTER_OK;
}

int specter_batch_kernels(specter_batch *b, long long *kernels) {
    if (!b || !kernels) { set_error("null argument"); return SPECTER_ERR_ARG; }
    *kernels = b->kernels;
    return SPECTER_OK;
}

}  // extern "C"
