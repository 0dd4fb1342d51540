// Host orchestration of the reference routines on device fields (both precisions).
#include <cstdio>
#include <string>
#include <vector>

#include "fast.h"
#include "kernels.cuh"
#include "kernels_elem.cuh"
#include "ops.h"

namespace sg {

#ifdef SG_PREC_DOUBLE
int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return ERR_CUDA;
    }
    return OK;
}
#endif

#define SG_TRY(x)                  \
    do {                           \
        int _st = (x);             \
        if (_st != OK) return _st; \
    } while (0)

static constexpr size_t kSmemBudget = 200 * 1024;

// scratch field slots of a plan
enum { kScrNL = 0 /* 16 slots */, kScrBC = 16 /* 2 */, kScrN = 18 /* 4 */, kScrR = 22 };

static int pick_tile(size_t per_col_bytes) {
    for (int t : {16, 8, 4, 2, 1})
        if (per_col_bytes * t <= kSmemBudget) return t;
    return 0;
}

// Opt in to more than the default 48 KB per block early: kernels that run the FC-Gram
// continuation also hold a small static array (fc_continuation), which counts against it.
template <typename K>
static void set_smem(K kern, size_t bytes) {
    if (bytes > 40 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

static int elem_blocks(const Plan &P, int rows) {
    long long n = (long long)rows * P.ny * P.nxh;
    long long b = (n + kThreads - 1) / kThreads;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b < 1 ? 1 : b);
}

// Launch (plan.h) brackets each kernel launch; `bytes` is the launch's algorithmic traffic:
// each input element read once and each output element written once.
static double cplx_rows(const Plan &P, double rows) { return rows * P.ny * P.nxh * (double)P.elt(); }

// ------------------------------------------------------------------------- launchers
// Tile widths (kx columns per block for the y/z passes, rows per block for the x pass) are
// runtime values: the largest power of two whose ping-pong buffers fit the smem budget.

// 1 when some field of a two-output pass writes both outputs: its input tile is then read
// from HBM once into a staging buffer instead of once per output.
static int two_outputs(void *const out0[], void *const out1[], int nf) {
    for (int f = 0; f < nf; f++)
        if (out0[f] && out1[f]) return 1;
    return 0;
}

template <typename T>
static int launch_z_inverse(Plan &P, const ZInvArgs &a0, int nf) {
    const size_t es = sizeof(C2<T>);
    ZInvArgs a = a0;
    a.staged = two_outputs(a.out0, a.out1, nf);
    const int tk = P.capped(pick_tile((2 * (size_t)P.tz.d.L + (a.staged ? P.nz : 0)) * es), Plan::kTileZ);
    if (!tk) { set_error("z length too large for shared memory"); return ERR_SHAPE; }
    const size_t sm = (2 * (size_t)P.tz.d.L + (a.staged ? P.nz : 0)) * tk * es;
    double bytes = 0;
    for (int f = 0; f < nf; f++)
        bytes += cplx_rows(P, P.nz) + cplx_rows(P, a.nrows) * ((a.out0[f] ? 1 : 0) + (a.out1[f] ? 1 : 0) + (a.add[f] ? 1 : 0));
    const int fst = fast_z_inverse(P, a, nf, bytes);
    if (fst != kNoFast) return fst;
    set_smem(k_z_inverse<T, GenericFFT<T>>, sm);
    Launch L(P, "z_inverse", bytes);
    k_z_inverse<T, GenericFFT<T>><<<dim3(cdiv(P.nxh, tk), P.ny, nf), kThreads, sm, P.stream>>>(P.geo, P.tz.d, a.prepared(), tk);
    return check_launch("z_inverse");
}

template <typename T>
static int launch_z_forward(Plan &P, const ZFwdArgs &a, int nf) {
    const size_t es = sizeof(C2<T>);
    const int tk = P.capped(pick_tile(2 * (size_t)P.tz.d.L * es), Plan::kTileZ);
    if (!tk) { set_error("z length too large for shared memory"); return ERR_SHAPE; }
    const size_t sm = 2 * (size_t)P.tz.d.L * tk * es;
    const double bytes = nf * (cplx_rows(P, P.nzp) + cplx_rows(P, P.nz));
    const int fst = fast_z_forward(P, a, nf, bytes);
    if (fst != kNoFast) return fst;
    set_smem(k_z_forward<T, GenericFFT<T>>, sm);
    Launch L(P, "z_forward", bytes);
    k_z_forward<T, GenericFFT<T>><<<dim3(cdiv(P.nxh, tk), P.ny, nf), kThreads, sm, P.stream>>>(P.geo, P.tz.d, a.prepared(), tk);
    return check_launch("z_forward");
}

template <typename T>
static int launch_y(Plan &P, const YArgs &a0, int nf, int nplanes) {
    const size_t es = sizeof(C2<T>);
    YArgs a = a0;
    a.staged = two_outputs(a.out0, a.out1, nf);
    const int tk = P.capped(pick_tile((2 * (size_t)P.ty.d.L + (a.staged ? P.ny : 0)) * es), Plan::kTileY);
    if (!tk) { set_error("y length too large for shared memory"); return ERR_SHAPE; }
    const size_t sm = (2 * (size_t)P.ty.d.L + (a.staged ? P.ny : 0)) * tk * es;
    double bytes = 0;
    for (int f = 0; f < nf; f++) bytes += cplx_rows(P, nplanes) * (1 + (a.out0[f] ? 1 : 0) + (a.out1[f] ? 1 : 0));
    const int fst = fast_y(P, a, nf, nplanes, bytes);
    if (fst != kNoFast) return fst;
    set_smem(k_y_pass_t<T, GenericFFT<T>, 0>, sm);
    Launch L(P, a.sign < 0 ? "y_forward" : "y_inverse", bytes);
    k_y_pass_t<T, GenericFFT<T>, 0><<<dim3(cdiv(P.nxh, tk), nplanes, nf), kThreads, sm, P.stream>>>(P.geo, P.ty.d, a.prepared(), tk);
    return check_launch("y_pass");
}

template <typename T>
static int launch_x(Plan &P, const XArgs &a, int nf, bool r2c) {
    const size_t es = sizeof(C2<T>);
    int rb = 0;
    for (int t : {16, 8, 4, 2, 1})
        if (t <= P.tile_cap[Plan::kTileX] && x_pass_elems<GenericFFT<T>>(P.tx.d, P.nxh, t) * es <= kSmemBudget) { rb = t; break; }
    if (!rb) { set_error("x length too large for shared memory"); return ERR_SHAPE; }
    const size_t sm = x_pass_elems<GenericFFT<T>>(P.tx.d, P.nxh, rb) * es;
    const dim3 grid(cdiv(a.nrows * P.ny, rb), 1, nf);
    const double rows = (double)a.nrows * P.ny;
    const double bytes = nf * rows * ((double)P.nxh * P.elt() + (double)P.nx * P.rel());
    const int fst = fast_x(P, a, nf, r2c, bytes);
    if (fst != kNoFast) return fst;
    if (r2c) {
        set_smem(k_x_r2c<T, GenericFFT<T>>, sm);
        Launch L(P, "x_r2c", bytes);
        k_x_r2c<T, GenericFFT<T>><<<grid, kThreads, sm, P.stream>>>(P.geo, P.tx.d, a.prepared(), rb);
    } else {
        set_smem(k_x_c2r<T, GenericFFT<T>>, sm);
        Launch L(P, "x_c2r", bytes);
        k_x_c2r<T, GenericFFT<T>><<<grid, kThreads, sm, P.stream>>>(P.geo, P.tx.d, a.prepared(), rb);
    }
    return check_launch(r2c ? "x_r2c" : "x_c2r");
}

template <typename T>
static int launch_x_nl(Plan &P, const XNLArgs &a) {
    const size_t es = sizeof(C2<T>);
    int rb = 0;
    for (int t : {16, 8, 4, 2, 1})
        if (t <= P.tile_cap[Plan::kTileX] && x_nl_elems<GenericFFT<T>>(P.tx.d, P.nxh, P.H, t) * es <= kSmemBudget) { rb = t; break; }
    if (!rb) { set_error("x length too large for shared memory"); return ERR_SHAPE; }
    const size_t sm = x_nl_elems<GenericFFT<T>>(P.tx.d, P.nxh, P.H, rb) * es;
    const int nc = a.c1 - a.c0;
    // rows read: 3 velocity rows (+ theta), d/dy and d/dz rows of each component; written: NL rows
    const double nin = 3 + (a.c1 == 4 ? 1 : 0) + 2 * nc;
    const double bytes = cplx_rows(P, a.nrows) * (nin + nc);
    const int fst = fast_x_nl(P, a, bytes);
    if (fst != kNoFast) return fst;
    set_smem(k_x_nonlinear<T, GenericFFT<T>>, sm);
    Launch L(P, "x_nonlinear", bytes);
    k_x_nonlinear<T, GenericFFT<T>><<<dim3(cdiv(a.nrows * P.ny, rb)), kThreads, sm, P.stream>>>(P.geo, P.tx.d, a.prepared(), rb);
    return check_launch("x_nonlinear");
}

template <typename T> static inline C2<T> *F(void *p) { return (C2<T> *)p; }
template <typename T> static inline const C2<T> *F(const void *p) { return (const C2<T> *)p; }

static int scratch(Plan &P, int n, void **out) {
    for (int i = 0; i < n; i++) {
        out[i] = P.scratch_field(i);
        if (!out[i]) { set_error("out of device memory (scratch fields)"); return ERR_OOM; }
    }
    return OK;
}

// sum block partials on the host in a fixed order (deterministic)
static int finish_reduce(Plan &P, int nblocks, int per, double *out) {
    std::vector<double> h((size_t)nblocks * per);
    if (cudaMemcpyAsync(h.data(), P.dred, h.size() * sizeof(double), cudaMemcpyDeviceToHost, P.stream) != cudaSuccess ||
        cudaStreamSynchronize(P.stream) != cudaSuccess)
        return check_launch("reduce");
    for (int j = 0; j < per; j++) {
        double s = 0.0;
        for (int b = 0; b < nblocks; b++) s += h[(size_t)b * per + j];
        out[j] = s;
    }
    return OK;
}

template <typename T>
static int reduce(Plan &P, const RedArgs &a, double *out) {
    const int nb = 304;
    { Launch L_(P, "reduce", a.nf * cplx_rows(P, a.z1)); k_reduce<T><<<nb, kThreads, 0, P.stream>>>(P.geo, a, P.dred); }
    SG_TRY(check_launch("reduce"));
    return finish_reduce(P, nb, 1, out);
}

static double inv_n2(const Plan &P) {
    const double t = (double)P.nx * (double)P.ny * (double)P.nz;
    return 1.0 / (t * t);
}

// ------------------------------------------------------------------------- fftp

// fftp1d_real_to_complex_z, src/fftp/fftp.fpp:720-786
template <typename T> int Ops<T>::fftp1d_r2c_z(Plan &P, void *inout) {
    ZFwdArgs a{};
    a.in[0] = inout; a.out[0] = inout; a.in_scale = 1.0;
    return launch_z_forward<T>(P, a, 1);
}

// fftp1d_complex_to_real_z, src/fftp/fftp.fpp:1060-1094
template <typename T> int Ops<T>::fftp1d_c2r_z(Plan &P, void *inout) {
    ZInvArgs a{};
    a.in[0] = inout; a.out0[0] = inout; a.nrows = P.nz; a.scale_rows = 0; a.scale = 1.0;
    return launch_z_inverse<T>(P, a, 1);
}

// fftp2d_real_to_complex_xy, src/fftp/fftp.fpp:428-524 (R2C over x, FFT over y per z plane)
template <typename T> int Ops<T>::fftp2d_r2c_xy(Plan &P, const void *rin, void *cout) {
    void *S[1];
    SG_TRY(scratch(P, 1, S));
    XArgs x{};
    x.in[0] = rin; x.out[0] = S[0]; x.nrows = P.nz; x.scale = 1.0;
    SG_TRY(launch_x<T>(P, x, 1, true));
    YArgs y{};
    y.in[0] = S[0]; y.out0[0] = cout; y.sign = -1; y.scale = 1.0;
    return launch_y<T>(P, y, 1, P.nz);
}

// fftp2d_complex_to_real_xy, src/fftp/fftp.fpp:824-919 (input left intact)
template <typename T> int Ops<T>::fftp2d_c2r_xy(Plan &P, const void *cin, void *rout) {
    void *S[1];
    SG_TRY(scratch(P, 1, S));
    YArgs y{};
    y.in[0] = cin; y.out0[0] = S[0]; y.sign = +1; y.scale = 1.0;
    SG_TRY(launch_y<T>(P, y, 1, P.nz));
    XArgs x{};
    x.in[0] = S[0]; x.out[0] = rout; x.nrows = P.nz; x.scale = 1.0;
    return launch_x<T>(P, x, 1, false);
}

// fftp3d_real_to_complex, src/fftp/fftp.fpp:388-425
template <typename T> int Ops<T>::fftp3d_r2c(Plan &P, const void *rin, void *cout) {
    SG_TRY(fftp2d_r2c_xy(P, rin, cout));
    return fftp1d_r2c_z(P, cout);
}

// fftp3d_complex_to_real, src/fftp/fftp.fpp:789-821 (input destroyed, :812)
template <typename T> int Ops<T>::fftp3d_c2r(Plan &P, void *cin, void *rout) {
    SG_TRY(fftp1d_c2r_z(P, cin));
    return fftp2d_c2r_xy(P, cin, rout);
}

// ------------------------------------------------------------------------- pseudo

template <typename T> int Ops<T>::derivk(Plan &P, const void *a, void *b, int dir) {
    if (dir < 1 || dir > 3) { set_error("derivk: dir must be 1, 2 or 3"); return ERR_ARG; }
    { Launch L_(P, "derivk", 2.0 * cplx_rows(P, P.nz)); k_derivk<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b), dir); }
    return check_launch("derivk");
}

template <typename T> int Ops<T>::laplak(Plan &P, const void *a, void *b) {
    { Launch L_(P, "laplak", 2.0 * cplx_rows(P, P.nz)); k_laplak<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b)); }
    return check_launch("laplak");
}

template <typename T> int Ops<T>::curlk(Plan &P, const void *a, const void *b, void *c, int dir) {
    if (dir < 1 || dir > 3) { set_error("curlk: dir must be 1, 2 or 3"); return ERR_ARG; }
    { Launch L_(P, "curlk", 3.0 * cplx_rows(P, P.nz)); k_curlk<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b), F<T>(c), dir); }
    return check_launch("curlk");
}

template <typename T> int Ops<T>::fc_filter(Plan &P, void *a) {
    { Launch L_(P, "filter", 2.0 * cplx_rows(P, P.nz)); k_filter<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a)); }
    return check_launch("fc_filter");
}

// gradre (pseudospec_hd.f90:209-319) for components [c0,c1) = [0,3); advect
// (pseudospec_phd.f90:23-113) for [3,4); both at once for [0,4).  Pipeline:
//   z inverse (v, d/dz v) -> y inverse (v, d/dy v, d/dz v) -> x: C2R, products, R2C
//   -> y forward -> z forward with FC-Gram continuation.
// Products are formed on the physical rows z < nz - Cz only; rows above are rebuilt
// by the continuation, exactly as in the reference.
template <typename T>
int Ops<T>::nonlinear(Plan &P, const void *const v[3], const void *th, void *const out[4], int c0, int c1,
                      const void **mixed) {
    void *S[16];
    SG_TRY(scratch(P, 16, S));
    const int nzp = P.nzp;
    const bool has_th = c1 == 4;
    auto want_d = [&](int c) { return c >= c0 && c < c1; };
    // z inverse: zS[c] = IFFT_z(v_c), zS[4+c] = IFFT_z(i kz v_c) (derivative only if needed)
    ZInvArgs z{};
    int nf = 0;
    for (int c = 0; c < (has_th ? 4 : 3); c++) {
        z.in[nf] = c < 3 ? v[c] : th;
        z.out0[nf] = S[c];
        z.out1[nf] = want_d(c) ? S[4 + c] : nullptr;
        nf++;
    }
    z.nrows = nzp; z.scale_rows = 0; z.scale = 1.0;
    z.in_ff = P.nl_input_ff;
    SG_TRY(launch_z_inverse<T>(P, z, nf));
    // y inverse A: U_c = S[8+c], DY_c = S[12+c]
    YArgs y{};
    nf = 0;
    for (int c = 0; c < (has_th ? 4 : 3); c++) {
        y.in[nf] = S[c];
        y.out0[nf] = S[8 + c];
        y.out1[nf] = want_d(c) ? S[12 + c] : nullptr;
        nf++;
    }
    y.sign = +1; y.scale = 1.0;
    SG_TRY(launch_y<T>(P, y, nf, nzp));
    // y inverse B: DZ_c in place
    YArgs y2{};
    nf = 0;
    for (int c = c0; c < c1; c++) { y2.in[nf] = S[4 + c]; y2.out0[nf] = S[4 + c]; y2.out1[nf] = nullptr; nf++; }
    y2.sign = +1; y2.scale = 1.0;
    SG_TRY(launch_y<T>(P, y2, nf, nzp));
    // x: products
    XNLArgs x{};
    for (int c = 0; c < 4; c++) {
        x.u[c] = S[8 + c];
        x.dy[c] = S[12 + c];
        x.dz[c] = S[4 + c];
        x.out[c] = S[c];
    }
    x.c0 = c0; x.c1 = c1; x.nrows = nzp; x.tmp = inv_n2(P);
    SG_TRY(launch_x_nl<T>(P, x));
    // y forward in place, then z forward with continuation into the outputs
    YArgs y3{};
    ZFwdArgs zf{};
    nf = 0;
    for (int c = c0; c < c1; c++) {
        y3.in[nf] = S[c]; y3.out0[nf] = S[c]; y3.out1[nf] = nullptr;
        zf.in[nf] = S[c]; zf.out[nf] = out ? out[c] : nullptr;
        nf++;
    }
    y3.sign = -1; y3.scale = 1.0;
    SG_TRY(launch_y<T>(P, y3, nf, nzp));
    if (mixed) {  // the caller finishes the z direction itself (fused stage kernels)
        for (int c = 0; c < 4; c++) mixed[c] = S[c];
        return OK;
    }
    zf.in_scale = 1.0;
    return launch_z_forward<T>(P, zf, nf);
}

// z inverse of up to 4 fields into scratch slots [s0, s0+n), physical rows only
template <typename T>
static int zinv_scratch(Plan &P, const void *const in[], int n, void *const dst[]) {
    ZInvArgs z{};
    for (int i = 0; i < n; i++) { z.in[i] = in[i]; z.out0[i] = dst[i]; z.out1[i] = nullptr; }
    z.nrows = P.nzp; z.scale_rows = 0; z.scale = 1.0;
    return launch_z_inverse<T>(P, z, n);
}

// energy, pseudospec_hd.f90:405-635 (kin=0 keeps the reference's y-curl-twice quirk)
template <typename T> int Ops<T>::energy(Plan &P, const void *a, const void *b, const void *c, int kin, double *out) {
    void *S[6];
    SG_TRY(scratch(P, 6, S));
    RedArgs r{};
    r.mode = 0; r.z1 = P.nzp;
    if (kin == 1) {
        const void *in[3] = {a, b, c};
        SG_TRY(zinv_scratch<T>(P, in, 3, S));
        r.nf = 3;
    } else if (kin == 0) {
        SG_TRY(curlk(P, b, c, S[3], 1));
        SG_TRY(curlk(P, a, c, S[4], 2));
        const void *in[3] = {S[3], S[4], S[4]};
        SG_TRY(zinv_scratch<T>(P, in, 3, S));
        r.nf = 3;
    } else if (kin == 2) {
        SG_TRY(curlk(P, b, c, S[3], 1));
        SG_TRY(curlk(P, a, c, S[4], 2));
        SG_TRY(curlk(P, a, b, S[5], 3));
        SG_TRY(curlk(P, S[4], S[5], S[0], 1));
        SG_TRY(curlk(P, S[3], S[5], S[1], 2));
        SG_TRY(curlk(P, S[3], S[4], S[2], 3));
        const void *in[3] = {S[0], S[1], S[2]};
        SG_TRY(zinv_scratch<T>(P, in, 3, S));
        r.nf = 3;
    } else {
        set_error("energy: kin must be 0, 1 or 2");
        return ERR_ARG;
    }
    for (int i = 0; i < 3; i++) r.f[i] = S[i];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// helicity, pseudospec_hd.f90:638-775
template <typename T> int Ops<T>::helicity(Plan &P, const void *a, const void *b, const void *c, double *out) {
    void *S[6];
    SG_TRY(scratch(P, 6, S));
    SG_TRY(curlk(P, b, c, S[3], 1));
    SG_TRY(curlk(P, a, c, S[4], 2));
    SG_TRY(curlk(P, a, b, S[5], 3));
    const void *in1[3] = {a, b, c};
    SG_TRY(zinv_scratch<T>(P, in1, 3, S));
    const void *in2[3] = {S[3], S[4], S[5]};
    SG_TRY(zinv_scratch<T>(P, in2, 3, S + 3));
    RedArgs r{};
    r.mode = 1; r.z1 = P.nzp; r.nf = 6;
    for (int i = 0; i < 6; i++) r.f[i] = S[i];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// cross, pseudospec_hd.f90:778-940
template <typename T> int Ops<T>::cross(Plan &P, const void *const A[3], const void *const B[3], int kin, double *out) {
    void *S[12];
    SG_TRY(scratch(P, 12, S));
    const void *ia[3], *ib[3];
    if (kin == 1) {
        for (int i = 0; i < 3; i++) { ia[i] = A[i]; ib[i] = B[i]; }
    } else {
        SG_TRY(curlk(P, A[1], A[2], S[6], 1)); SG_TRY(curlk(P, B[1], B[2], S[9], 1));
        SG_TRY(curlk(P, A[0], A[2], S[7], 2)); SG_TRY(curlk(P, B[0], B[2], S[10], 2));
        SG_TRY(curlk(P, A[0], A[1], S[8], 3)); SG_TRY(curlk(P, B[0], B[1], S[11], 3));
        for (int i = 0; i < 3; i++) { ia[i] = S[6 + i]; ib[i] = S[9 + i]; }
    }
    SG_TRY(zinv_scratch<T>(P, ia, 3, S));
    SG_TRY(zinv_scratch<T>(P, ib, 3, S + 3));
    RedArgs r{};
    r.mode = 1; r.z1 = P.nzp; r.nf = 6;
    for (int i = 0; i < 6; i++) r.f[i] = S[i];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// divergence, pseudospec_hd.f90:1118-1235
template <typename T> int Ops<T>::divergence(Plan &P, const void *a, const void *b, const void *c, double *out) {
    void *S[2];
    SG_TRY(scratch(P, 2, S));
    { Launch L_(P, "div", 4.0 * cplx_rows(P, P.nz)); k_div<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b), F<T>(c), F<T>(S[1])); }
    SG_TRY(check_launch("divergence"));
    const void *in[1] = {S[1]};
    SG_TRY(zinv_scratch<T>(P, in, 1, S));
    RedArgs r{};
    r.mode = 0; r.z1 = P.nzp; r.nf = 1; r.f[0] = S[0];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// variance, pseudospec_phd.f90:116-196
template <typename T> int Ops<T>::variance(Plan &P, const void *a, int kin, double *out) {
    void *S[2];
    SG_TRY(scratch(P, 2, S));
    const void *src = a;
    if (kin == 0) {
        { Launch L_(P, "kk2_mul", 2.0 * cplx_rows(P, P.nz)); k_kk2_mul<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(S[1])); }
        SG_TRY(check_launch("variance"));
        src = S[1];
    }
    const void *in[1] = {src};
    SG_TRY(zinv_scratch<T>(P, in, 1, S));
    RedArgs r{};
    r.mode = 0; r.z1 = P.nzp; r.nf = 1; r.f[0] = S[0];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// product, pseudospec_phd.f90:199-272
template <typename T> int Ops<T>::product(Plan &P, const void *a, const void *b, double *out) {
    void *S[2];
    SG_TRY(scratch(P, 2, S));
    const void *in[2] = {a, b};
    SG_TRY(zinv_scratch<T>(P, in, 2, S));
    RedArgs r{};
    r.mode = 1; r.z1 = P.nzp; r.nf = 2;
    r.f[0] = S[0]; r.f[1] = S[1];
    double s;
    SG_TRY(reduce<T>(P, r, &s));
    *out = s * (inv_n2(P) / (double)(P.nz - P.cz));
    return OK;
}

// ------------------------------------------------------------------------- boundary

static double2 *plan_wtw(Plan &P) { return (double2 *)P.dwtw; }
static double2 *plan_bc(Plan &P, int i) { return (double2 *)P.scratch_field(kScrBC + i); }

template <typename T>
static int wall_eval(Plan &P, const void *in, double scale, double2 *bc, int neg) {
    { Launch L_(P, "wall_eval", cplx_rows(P, P.nz)); k_wall_eval<T><<<dim3(cdiv(P.nxh, 64), P.ny), 64, 0, P.stream>>>(P.geo, F<T>(in), scale, plan_wtw(P), bc, neg); }
    return check_launch("wall_eval");
}

// bouncheck_z, boundary_mod.fpp:681-801
template <typename T> int Ops<T>::bouncheck_z(Plan &P, const void *a, const void *b, double *bot, double *top) {
    double2 *bcA = plan_bc(P, 0), *bcB = plan_bc(P, 1);
    if (!bcA || !bcB) { set_error("out of device memory"); return ERR_OOM; }
    SG_TRY(wall_eval<T>(P, a, 1.0, bcA, 0));
    if (b) SG_TRY(wall_eval<T>(P, b, 1.0, bcB, 0));
    const int nb = 152;
    { Launch L_(P, "reduce_walls", 64.0 * P.nxh * P.ny); k_reduce_walls<<<nb, kThreads, 0, P.stream>>>(P.geo, bcA, b ? bcB : nullptr, P.dred); }
    SG_TRY(check_launch("bouncheck_z"));
    double r[2];
    SG_TRY(finish_reduce(P, nb, 2, r));
    const double inv = 1.0 / (double)((long long)P.nx * P.ny * P.nz);
    *bot = r[0] * inv * inv;
    *top = r[1] * inv * inv;
    return OK;
}

// sol_project, boundary_mod.fpp:197-402, with poisson_inhomogeneous (:405-448) and the
// Dirichlet / Neumann branches of laplace_z (:451-678); bczsta = bczend = 0.
template <typename T> int Ops<T>::sol_project(Plan &P, void *a, void *b, void *c, void *d, int bctarget) {
    if (bctarget != 0 && bctarget != 1) { set_error("sol_project: bctarget must be 0 or 1"); return ERR_BC; }
    void *S[3];
    SG_TRY(scratch(P, 3, S));
    double2 *bc = plan_bc(P, 0), *coef = plan_bc(P, 1);
    if (!bc || !coef) { set_error("out of device memory"); return ERR_OOM; }
    { Launch L_(P, "poisson", 8.0 * cplx_rows(P, P.nz)); k_poisson<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b), F<T>(c), F<T>(d), F<T>(S[0]), bctarget); }
    SG_TRY(check_launch("poisson"));
    SG_TRY(wall_eval<T>(P, S[0], 1.0, bc, bctarget == 0));
    { Launch L_(P, "laplace_coef", 64.0 * P.nxh * P.ny); k_laplace_coef<<<dim3(cdiv(P.nxh, 64), P.ny), 64, 0, P.stream>>>(P.geo, bc, coef, bctarget); }
    SG_TRY(check_launch("laplace_coef"));
    { Launch L_(P, "laplace_profile", 2.0 * cplx_rows(P, P.nz)); k_laplace_profile<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, coef, F<T>(S[1]), F<T>(S[2])); }
    SG_TRY(check_launch("laplace_profile"));
    ZInvArgs z{};
    if (bctarget == 0) {
        // d = IFFT_z(d/nz) + C2
        z.in[0] = S[0]; z.out0[0] = d; z.add[0] = S[1];
        z.nrows = P.nz; z.scale_rows = 0; z.scale = 1.0;
    } else {
        // d = IFFT_z(d)/nz + C2
        z.in[0] = d; z.out0[0] = d; z.add[0] = S[1];
        z.nrows = P.nz; z.scale_rows = P.nz; z.scale = 1.0 / (double)P.nz;
    }
    SG_TRY(launch_z_inverse<T>(P, z, 1));
    ZFwdArgs f{};
    f.in[0] = S[1]; f.out[0] = S[1]; f.in[1] = S[2]; f.out[1] = S[2]; f.in_scale = 1.0;
    SG_TRY(launch_z_forward<T>(P, f, 2));
    { Launch L_(P, "proj_sub", 8.0 * cplx_rows(P, P.nz)); k_proj_sub<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(a), F<T>(b), F<T>(c), F<T>(S[1]), F<T>(S[2])); }
    return check_launch("proj_sub");
}

// v_imposebc_and_project, vboundary.f90:67-151 (no-slip walls, noslip_z :154-211)
template <typename T>
int Ops<T>::v_imposebc_and_project(Plan &P, void *vx, void *vy, void *vz, void *pr, int rki, int ord,
                                   const double vzsta[2], const double vzend[2]) {
    if (rki < 1) { set_error("v_imposebc_and_project: rki must be >= 1"); return ERR_ARG; }
    // goto_domain_w_boundaries (boundary_mod.fpp:72-150): IFFT_z, 1/nz on the physical rows
    ZInvArgs z{};
    // rows >= nzp are rebuilt by the continuation in goto_3d_fourier, so only the
    // physical rows are written back
    z.in[0] = vx; z.out0[0] = vx; z.in[1] = vy; z.out0[1] = vy;
    z.nrows = P.nzp; z.scale_rows = P.nzp; z.scale = 1.0 / (double)P.nz;
    SG_TRY(launch_z_inverse<T>(P, z, 2));
    double tmp = 1 / (double)rki;
    if (rki != ord) tmp = (double)(rki + 1) * tmp;
    WallVel vb{vzsta[0], vzsta[1], vzend[0], vzend[1]};
    { Launch L_(P, "noslip", cplx_rows(P, 6)); k_noslip<T><<<dim3(cdiv(P.nxh, 64), P.ny), 64, 0, P.stream>>>(P.geo, F<T>(vx), F<T>(vy), F<T>(pr), tmp, vb); }
    SG_TRY(check_launch("noslip"));
    // goto_3d_fourier (boundary_mod.fpp:153-194)
    ZFwdArgs f{};
    f.in[0] = vx; f.out[0] = vx; f.in[1] = vy; f.out[1] = vy; f.in_scale = 1.0;
    SG_TRY(launch_z_forward<T>(P, f, 2));
    return sol_project(P, vx, vy, vz, pr, 1);
}

// s_imposebc, sboundary.f90:67-165 (constant wall value 0)
template <typename T> int Ops<T>::s_imposebc(Plan &P, void *th) {
    ZInvArgs z{};
    z.in[0] = th; z.out0[0] = th;
    z.nrows = P.nzp; z.scale_rows = P.nzp; z.scale = 1.0 / (double)P.nz;
    SG_TRY(launch_z_inverse<T>(P, z, 1));
    { Launch L_(P, "zero_walls", cplx_rows(P, 2)); k_zero_walls<T><<<dim3(cdiv(P.nxh, 64), P.ny), 64, 0, P.stream>>>(P.geo, F<T>(th)); }
    SG_TRY(check_launch("zero_walls"));
    return fftp1d_r2c_z(P, th);
}

// ------------------------------------------------------------------------- stage

template <typename T> int Ops<T>::axpy_sub(Plan &P, void *y, const void *x, double s) {
    { Launch L_(P, "sub_scaled", 3.0 * cplx_rows(P, P.nz)); k_sub_scaled<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(y), F<T>(x), s); }
    return check_launch("sub_scaled");
}

template <typename T> int Ops<T>::rk_update(Plan &P, void *v, const void *Cold, const void *N, double dt, double nu, double rmp) {
    { Launch L_(P, "rk_update", 4.0 * cplx_rows(P, P.nz)); k_rk_update<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(P.geo, F<T>(v), F<T>(Cold), F<T>(N), dt, nu, rmp); }
    return check_launch("rk_update");
}

template <typename T>
static __global__ void k_scale_real(T *r, long long n, T s) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) r[i] *= s;
}

template <typename T> int Ops<T>::scale_real(Plan &P, void *r, double s) {
    { Launch L_(P, "scale_real", 2.0 * P.real_elems() * P.rel()); k_scale_real<T><<<152 * 8, kThreads, 0, P.stream>>>((T *)r, (long long)P.real_elems(), (T)s); }
    return check_launch("scale_real");
}

// One RK stage: hd_rkstep2.f90:1-36 (solver 0) or bouss_rkstep2.f90:1-59 (solver 1), executed
// as the reference's call sequence.  v = {vx, vy, vz, th}; Cold = {C1, C2, C3, C7}.
template <typename T>
int Ops<T>::coriolis(Plan &P, void *const N[3], const void *const v[3], const double omega[3]) {
    Launch L(P, "coriolis", 9.0 * cplx_rows(P, P.nz));
    k_coriolis<T><<<elem_blocks(P, P.nz), kThreads, 0, P.stream>>>(
        P.geo, (C2<T> *)N[0], (C2<T> *)N[1], (C2<T> *)N[2], (const C2<T> *)v[0], (const C2<T> *)v[1],
        (const C2<T> *)v[2], (T)omega[0], (T)omega[1], (T)omega[2]);
    return check_launch("coriolis");
}

template <typename T>
int Ops<T>::stage(Plan &P, const StageParams &sp, int o, void *const v[4], void *pr, const void *const Cold[4]) {
    void *N[4];
    for (int i = 0; i < 4; i++) {
        N[i] = P.scratch_field(kScrN + i);
        if (!N[i]) { set_error("out of device memory"); return ERR_OOM; }
    }
    const double rmp = 1 / (double)o;
    const bool bouss = sp.solver >= 1, rot = sp.solver == 2;
    const void *vv[3] = {v[0], v[1], v[2]};
    SG_TRY(nonlinear(P, vv, bouss ? v[3] : nullptr, N, 0, bouss ? 4 : 3));
    if (rot) SG_TRY(coriolis(P, N, vv, sp.omega));  // rotbouss_rkstep2.f90:13-17
    if (bouss) {
        SG_TRY(axpy_sub(P, N[2], v[3], sp.xmom));   // buoyancy
        SG_TRY(axpy_sub(P, N[3], v[2], sp.xtemp));  // heat current
    }
    for (int i = 0; i < (bouss ? 4 : 3); i++) SG_TRY(fc_filter(P, N[i]));
    for (int i = 0; i < 3; i++) SG_TRY(rk_update(P, v[i], Cold[i], N[i], sp.dt, sp.nu, rmp));
    if (bouss) SG_TRY(rk_update(P, v[3], Cold[3], N[3], sp.dt, sp.kappa, rmp));
    SG_TRY(v_imposebc_and_project(P, v[0], v[1], v[2], pr, o, sp.ord, sp.vzsta, sp.vzend));
    if (rot) return s_imposebc(P, v[3]);  // no theta filter / round trip in rotbouss_rkstep2.f90
    if (bouss) {
        SG_TRY(s_imposebc(P, v[3]));
        SG_TRY(fc_filter(P, v[3]));
        // c2r -> /nx/ny/nz -> r2c (bouss_rkstep2.f90:56-59)
        void *R = P.scratch_field(kScrR);  // a complex slot is large enough for nx*ny*nz reals
        if (!R) { set_error("out of device memory"); return ERR_OOM; }
        SG_TRY(fftp3d_c2r(P, v[3], R));
        SG_TRY(scale_real(P, R, 1.0 / ((double)P.nx * P.ny * P.nz)));
        SG_TRY(fftp3d_r2c(P, R, v[3]));
    }
    return OK;
}

#ifdef SG_PREC_DOUBLE
template struct Ops<double>;
#else
template struct Ops<float>;
#endif

}  // namespace sg
