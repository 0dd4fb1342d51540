// Plan construction: the GB300 counterpart of fcgram_create_plan (src/fftp/fcgram_mod.f90:49-144,
// tables :180-257) together with the grid / wavenumber setup the driver performs
// (src/specter.fpp:683-800, kes module src/pseudo/pseudospec_mod.fpp:84-91).
#include "batch.h"
#include "plan.h"

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace sg {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
const char *last_error() { return g_err.c_str(); }

static bool smooth235(int m) {
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    return m == 1;
}

static int factorize(int n, int *radix) {
    int nf = 0;
    const int pref[] = {8, 4, 2, 3, 5, 7, 11, 13};
    for (int r : pref)
        while (n % r == 0) {
            if (nf >= kMaxStages) return -1;
            radix[nf++] = r;
            n /= r;
        }
    return n == 1 ? nf : -1;
}

typedef std::complex<long double> cld;
static cld root(long t, long n) {  // exp(-2*pi*i*t/n)
    const long double pi = 3.14159265358979323846264338327950288L;
    long double a = -2.0L * pi * (long double)(t % n) / (long double)n;
    return cld(cosl(a), sinl(a));
}

template <typename T>
static void put(std::vector<char> &buf, size_t off, const cld &v) {
    T re = (T)v.real(), im = (T)v.imag();
    memcpy(buf.data() + off, &re, sizeof(T));
    memcpy(buf.data() + off + sizeof(T), &im, sizeof(T));
}

int build_fft_table(FFTTable &t, int n, Prec prec) {
    FFTDesc &d = t.d;
    memset(&d, 0, sizeof d);
    d.n = n;
    int nf = factorize(n, d.radix);
    int L = n;
    if (nf < 0) {
        L = 2 * n - 1;
        while (!smooth235(L)) L++;
        nf = factorize(L, d.radix);
        d.blue = 1;
    }
    if (nf < 0) return ERR_SHAPE;
    d.L = L;
    d.nst = nf;
    const size_t es = prec == FP32 ? 8 : 16;
    const size_t ntot = (size_t)L + (d.blue ? (size_t)n + 2 * (size_t)L : 0);
    std::vector<char> h(ntot * es);
    auto P = [&](size_t i, const cld &v) {
        if (prec == FP64) put<double>(h, i * es, v);
        else if (prec == FP32) put<float>(h, i * es, v);
        else {
            const ff q[2] = {ff_split(v.real()), ff_split(v.imag())};
            memcpy(h.data() + i * es, q, sizeof q);
        }
    };
    for (int k = 0; k < L; k++) P(k, root(k, L));
    if (d.blue) {
        const long double pi = 3.14159265358979323846264338327950288L;
        std::vector<cld> chirp(n), bf(L, cld(0)), bb(L, cld(0));
        for (long k = 0; k < n; k++) {
            long k2 = (k * k) % (2L * n);
            long double a = -pi * (long double)k2 / (long double)n;
            chirp[k] = cld(cosl(a), sinl(a));
        }
        for (int k = 0; k < n; k++) {
            bf[k] = std::conj(chirp[k]);
            bb[k] = chirp[k];
            if (k) { bf[L - k] = std::conj(chirp[k]); bb[L - k] = chirp[k]; }
        }
        // exact-index DFT in long double: F_j = sum_m b_m exp(-2 pi i j m / L), scaled by 1/L
        std::vector<cld> w(L);
        for (int k = 0; k < L; k++) w[k] = root(k, L);
        for (int j = 0; j < L; j++) {
            cld sf(0), sb(0);
            for (int m = 0; m < L; m++) {
                if (bf[m] == cld(0) && bb[m] == cld(0)) continue;
                const cld ww = w[((long)j * m) % L];
                sf += bf[m] * ww;
                sb += bb[m] * ww;
            }
            P((size_t)L + n + j, sf / (long double)L);
            P((size_t)L + n + L + j, sb / (long double)L);
        }
        for (int k = 0; k < n; k++) P((size_t)L + k, chirp[k]);
    }
    if (cudaMalloc(&t.mem, h.size()) != cudaSuccess) return ERR_OOM;
    cudaMemcpy(t.mem, h.data(), h.size(), cudaMemcpyHostToDevice);
    char *b = (char *)t.mem;
    d.tw = b;
    if (d.blue) {
        d.chirp = b + (size_t)L * es;
        d.filtf = b + ((size_t)L + n) * es;
        d.filtb = b + ((size_t)L + n + L) * es;
    }
    return OK;
}

void free_fft_table(FFTTable &t) {
    if (t.mem) cudaFree(t.mem);
    t.mem = nullptr;
}

// load_dirichlet_tables, src/fftp/fcgram_mod.f90:180-257: raw float64 streams in Fortran
// order, A(C,d) and Q(d,d); dir = A * transpose(Q).
static int read_tables(const char *tdir, int C, int d, std::vector<double> &A, std::vector<double> &Q) {
    A.assign((size_t)C * d, 0.0);
    Q.assign((size_t)d * d, 0.0);
    char path[4096];
    snprintf(path, sizeof path, "%s/A%d-%d.dat", tdir, C, d);
    FILE *f = fopen(path, "rb");
    if (!f || fread(A.data(), sizeof(double), A.size(), f) != A.size()) {
        if (f) fclose(f);
        set_error(std::string("Could not find table ") + path);
        return ERR_TABLE;
    }
    fclose(f);
    snprintf(path, sizeof path, "%s/Q%d.dat", tdir, d);
    f = fopen(path, "rb");
    if (!f || fread(Q.data(), sizeof(double), Q.size(), f) != Q.size()) {
        if (f) fclose(f);
        set_error(std::string("Could not find table ") + path);
        return ERR_TABLE;
    }
    fclose(f);
    return OK;
}

static std::vector<double> dir_from(const std::vector<double> &A, const std::vector<double> &Q, int C, int d) {
    std::vector<double> dir((size_t)C * d, 0.0);
    for (int i = 0; i < C; i++)
        for (int j = 0; j < d; j++) {
            double s = 0.0;
            for (int l = 0; l < d; l++) s += A[i + (size_t)C * l] * Q[j + (size_t)d * l];
            dir[i + (size_t)C * j] = s;
        }
    return dir;
}

static int load_tables(Plan *p, const char *tdir) {
    std::vector<double> A, Q;
    const int st = read_tables(tdir, p->cz, p->oz, A, Q);
    if (st) return st;
    p->dir = dir_from(A, Q, p->cz, p->oz);
    return OK;
}

int table_check(const char *tdir, int C, int d, double out[3]) {
    if (C < 1 || d < 1 || C > 4096 || d > 64) { set_error("bad table sizes"); return ERR_ARG; }
    std::vector<double> A, Q;
    const int st = read_tables(tdir ? tdir : ".", C, d, A, Q);
    if (st) return st;
    // orthonormality of the Gram basis: max |Q^T Q - I|
    double e = 0.0;
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++) {
            double s = 0.0;
            for (int l = 0; l < d; l++) s += Q[l + (size_t)d * i] * Q[l + (size_t)d * j];
            e = std::max(e, std::fabs(s - (i == j ? 1.0 : 0.0)));
        }
    const std::vector<double> dir = dir_from(A, Q, C, d);
    double mx = 0.0, rs = 0.0;
    for (int i = 0; i < C; i++) {
        double r = 0.0;
        for (int j = 0; j < d; j++) {
            mx = std::max(mx, std::fabs(dir[i + (size_t)C * j]));
            r += std::fabs(dir[i + (size_t)C * j]);
        }
        rs = std::max(rs, r);
    }
    out[0] = e;
    out[1] = mx;
    out[2] = rs;
    return OK;
}

int plan_create(Plan **out, const int n[3], const int c[3], const int o[3], const double len[3],
                const char *tdir, int prec) {
    *out = nullptr;
    if (prec != FP64 && prec != FP32) { set_error("precision must be 0 (FP64) or 1 (FP32)"); return ERR_ARG; }
    const int nx = n[0], ny = n[1], nz = n[2];
    // x and y periodic (C = o = 0), z non-periodic with FC-Gram (the reference's XY -> Z branch,
    // src/fftp/fftp.fpp:411-416 with plan%y%C = 0)
    if (c[0] != 0 || c[1] != 0 || o[0] != 0 || o[1] != 0) {
        set_error("only periodic x,y with an FC-Gram z direction is supported (Cx=Cy=ox=oy=0)");
        return ERR_SHAPE;
    }
    if (o[2] > 9) {  // the continuation kernels hold at most 2 * 9 wall-adjacent rows per column
        set_error("oz > 9 is not supported (the FC-Gram tables stop at d = 9)");
        return ERR_SHAPE;
    }
    if (nx < 4 || ny < 2 || nz < 4 || nx % 2 || ny % 2 || nz % 2 || c[2] <= 0 || o[2] <= 0 ||
        nz - c[2] < 2 * o[2] || nz - c[2] < 2) {
        set_error("bad grid shape: nx, ny, nz must be even, nz - Cz >= 2*oz");
        return ERR_SHAPE;
    }
    if (!(len[0] > 0 && len[1] > 0 && len[2] > 0)) { set_error("box lengths must be positive"); return ERR_ARG; }
    Plan *p = new Plan();
    p->prec = (Prec)prec;
    p->nx = nx; p->ny = ny; p->nz = nz; p->cz = c[2]; p->oz = o[2];
    p->nxh = nx / 2 + 1; p->nzp = nz - c[2]; p->H = nx / 2;
    p->ldx = (p->nxh + 7) / 8 * 8;
    p->Lx = len[0]; p->Ly = len[1]; p->Lz = len[2];
    // kernels index fields with 32-bit offsets
    if ((double)nz * ny * (((nx / 2 + 1) + 7) / 8 * 8) >= 4294967296.0 || (double)nx * ny * nz >= 4294967296.0) {
        set_error("grid too large: a field must hold fewer than 2^32 elements");
        delete p;
        return ERR_SHAPE;
    }
    p->tdir = tdir ? tdir : ".";
    int st = load_tables(p, p->tdir.c_str());
    if (st) { delete p; return st; }
    // grids and wavenumbers, src/specter.fpp:683-800
    const double pi = 3.14159265358979323846;
    p->Dkx = 1.0 / p->Lx;
    p->Dky = 1.0 / p->Ly;
    p->dz = p->Lz / (nz - p->cz - 1);
    p->Dkz = 2.0 * pi / (p->dz * nz);
    p->z.resize(nz);
    for (int k = 0; k < nz; k++) p->z[k] = p->dz * k;
    p->kx.resize(p->nxh); p->ky.resize(ny); p->kz.resize(nz);
    for (int i = 0; i < p->nxh; i++) p->kx[i] = (i < nx / 2 ? (double)i : (double)(i - nx)) * p->Dkx;
    for (int j = 0; j < ny; j++) p->ky[j] = (j < ny / 2 ? (double)j : (double)(j - ny)) * p->Dky;
    for (int k = 0; k < nz; k++) p->kz[k] = (k < nz / 2 ? (double)k : (double)(k - nz)) * p->Dkz;
    // fc_filter factors, src/pseudo/pseudospec_hd.f90:1082-1115 (alpha = 16 ln 10, p = 50)
    const double alpha = 16 * std::log(10.0), p2 = 100.0;
    p->fx.resize(p->nxh); p->fy.resize(ny); p->fz.resize(nz);
    for (int i = 0; i < p->nxh; i++) p->fx[i] = std::exp(-alpha * std::pow(2 * p->kx[i] / nx / p->Dkx, p2));
    for (int j = 0; j < ny; j++) p->fy[j] = std::exp(-alpha * std::pow(2 * p->ky[j] / ny / p->Dky, p2));
    for (int k = 0; k < nz; k++) p->fz[k] = std::exp(-alpha * std::pow(2 * p->kz[k] / nz / p->Dkz, p2));

    std::vector<double> g;
    auto app = [&](const std::vector<double> &v) { size_t o = g.size(); g.insert(g.end(), v.begin(), v.end()); return o; };
    size_t okx = app(p->kx), oky = app(p->ky), okz = app(p->kz), oz_ = app(p->z), odir = app(p->dir);
    size_t ofx = app(p->fx), ofy = app(p->fy), ofz = app(p->fz);
    if (cudaMalloc(&p->dgeo, g.size() * sizeof(double)) != cudaSuccess) { set_error("cudaMalloc failed"); delete p; return ERR_OOM; }
    cudaMemcpy(p->dgeo, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice);
    {
        std::vector<float> gf(g.begin(), g.end());
        if (cudaMalloc(&p->dgeof, gf.size() * sizeof(float)) != cudaSuccess) { set_error("cudaMalloc failed"); plan_destroy(p); return ERR_OOM; }
        cudaMemcpy(p->dgeof, gf.data(), gf.size() * sizeof(float), cudaMemcpyHostToDevice);
        std::vector<ff> gq(g.size());
        for (size_t i = 0; i < g.size(); i++) gq[i] = ff_split(g[i]);
        if (cudaMalloc(&p->dgeoq, gq.size() * sizeof(ff)) != cudaSuccess) { set_error("cudaMalloc failed"); plan_destroy(p); return ERR_OOM; }
        cudaMemcpy(p->dgeoq, gq.data(), gq.size() * sizeof(ff), cudaMemcpyHostToDevice);
    }
    // R2C / C2R post-processing twiddles exp(-2*pi*i*k/nx), k = 0..H
    {
        const size_t es = p->elt();
        std::vector<char> h((size_t)(p->H + 1) * es);
        for (int k = 0; k <= p->H; k++) {
            cld v = root(k, nx);
            if (p->prec == FP64) put<double>(h, k * es, v); else put<float>(h, k * es, v);
        }
        cudaMalloc(&p->dxtw, h.size());
        cudaMemcpy(p->dxtw, h.data(), h.size(), cudaMemcpyHostToDevice);
    }
    if ((st = build_fft_table(p->tx, p->H, p->prec)) || (st = build_fft_table(p->ty, ny, p->prec)) ||
        (st = build_fft_table(p->tz, nz, p->prec))) {
        set_error("FFT table construction failed");
        plan_destroy(p);
        return st;
    }
    if (p->prec == FP32 && ((st = build_fft4_table(p->tx4, p->H, 0)) || (st = build_fft4_table(p->ty4, ny, 1)) ||
                            (st = build_fft4_table(p->tz4, nz, 2)))) {
        plan_destroy(p);
        return st;
    }
    cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    Geo &G = p->geo;
    G.nx = nx; G.ny = ny; G.nz = nz; G.cz = p->cz; G.oz = p->oz; G.nxh = p->nxh; G.nzp = p->nzp;
    G.ldx = p->ldx; G.H = p->H; G.Lz = p->Lz;
    G.kx = p->dgeo + okx; G.ky = p->dgeo + oky; G.kz = p->dgeo + okz; G.z = p->dgeo + oz_;
    G.dir = p->dgeo + odir; G.fx = p->dgeo + ofx; G.fy = p->dgeo + ofy; G.fz = p->dgeo + ofz;
    G.kxf = p->dgeof + okx; G.kyf = p->dgeof + oky; G.kzf = p->dgeof + okz; G.zf = p->dgeof + oz_;
    G.fxf = p->dgeof + ofx; G.fyf = p->dgeof + ofy; G.fzf = p->dgeof + ofz;
    G.kxq = p->dgeoq + okx; G.kyq = p->dgeoq + oky; G.kzq = p->dgeoq + okz; G.zq = p->dgeoq + oz_;
    G.fxq = p->dgeoq + ofx; G.fyq = p->dgeoq + ofy; G.fzq = p->dgeoq + ofz; G.dirq = p->dgeoq + odir;
    G.xtw = p->dxtw;
    {
        // laplace_z constants of every (kx, ky) column (boundary_mod.fpp:521-549)
        std::vector<double> lc((size_t)3 * ny * p->nxh, 0.0);
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < p->nxh; i++) {
                const double kh = std::sqrt(p->kx[i] * p->kx[i] + p->ky[j] * p->ky[j]);
                double *c = &lc[((size_t)j * p->nxh + i) * 3];
                c[0] = kh;
                if (i || j) {
                    c[1] = std::exp(-(kh * p->Lz));
                    c[2] = 1.0 / (kh * (1 - std::exp(-(2 * kh * p->Lz))));
                }
            }
        if (cudaMalloc(&p->dlapc, lc.size() * sizeof(double)) != cudaSuccess) { set_error("cudaMalloc failed"); plan_destroy(p); return ERR_OOM; }
        cudaMemcpy(p->dlapc, lc.data(), lc.size() * sizeof(double), cudaMemcpyHostToDevice);
        G.lapc = p->dlapc;
    }
    p->nred = 4096;
    cudaMalloc(&p->dred, sizeof(double) * p->nred);
    {
        std::vector<double> w(2 * (size_t)nz);
        for (int k = 0; k < nz; k++) {
            cld v = std::conj(root((long)k * (p->nzp - 1), nz));
            w[2 * k] = (double)v.real();
            w[2 * k + 1] = (double)v.imag();
        }
        cudaMalloc(&p->dwtw, w.size() * sizeof(double));
        cudaMemcpy(p->dwtw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice);
        G.wtw = p->dwtw;
        std::vector<ff> wq(2 * (size_t)nz);  // (re, im) pairs of float-float: an ffc per k
        for (int k = 0; k < nz; k++) {
            cld v = std::conj(root((long)k * (p->nzp - 1), nz));
            wq[2 * k] = ff_split(v.real());
            wq[2 * k + 1] = ff_split(v.imag());
        }
        cudaMalloc(&p->dwtwq, wq.size() * sizeof(ff));
        cudaMemcpy(p->dwtwq, wq.data(), wq.size() * sizeof(ff), cudaMemcpyHostToDevice);
        G.wtwq = p->dwtwq;
    }
    cudaMallocHost(&p->hred, sizeof(double) * 64);
    if (cudaGetLastError() != cudaSuccess) { set_error("CUDA error during plan creation"); plan_destroy(p); return ERR_CUDA; }
    *out = p;
    return OK;
}

void *Plan::scratch_field(int i) {
    if ((int)scratch.size() <= i) scratch.resize(i + 1, nullptr);
    if (!scratch[i]) {
        void *m = nullptr;
        if (cudaMalloc(&m, field_bytes()) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        cudaMemsetAsync(m, 0, field_bytes(), stream);
        scratch[i] = m;
    }
    return scratch[i];
}

unsigned long long plan_bytes(const Plan &P) {
    unsigned long long b = 0;
    for (void *m : P.scratch) b += m ? P.field_bytes() : 0;
    b += (P.kx.size() + P.ky.size() + P.kz.size() + P.z.size() + P.dir.size() + P.fx.size() + P.fy.size() + P.fz.size()) * 12ull;
    auto tab = [](const FFTTable &t, size_t es) { return t.mem ? (unsigned long long)(4 * (size_t)t.d.L + 2 * (size_t)t.d.n) * es : 0ull; };
    const size_t es = P.elt();
    b += tab(P.tx, es) + tab(P.ty, es) + tab(P.tz, es);
    auto tab4 = [](const FFT4Table &t) { return t.mem ? (unsigned long long)(4 * (size_t)t.d.L + (size_t)t.d.n) * 8 : 0ull; };
    b += tab4(P.tx4) + tab4(P.ty4) + tab4(P.tz4);
    b += (unsigned long long)(P.H + 1) * es + (unsigned long long)P.nred * 8 + (unsigned long long)P.nz * 16;
    return b;
}

static cudaEvent_t take_event(Plan *p) {
    if (!p->evpool.empty()) {
        cudaEvent_t e = p->evpool.back();
        p->evpool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void Plan::prof_begin(const char *name, double bytes) {
    if (owner) { owner->prof_begin(name, bytes); return; }
    if (batch) batch->unbatchable = name;  // a launch while recording: it has no batched form
    launches++;
    if (!profile) return;
    Rec r{name, bytes, take_event(this), take_event(this)};
    cudaEventRecord(r.a, stream);
    recs.push_back(r);
}

void Plan::prof_end() {
    if (owner) { owner->prof_end(); return; }
    if (!profile || recs.empty()) return;
    cudaEventRecord(recs.back().b, stream);
    if (recs.size() >= 4096) prof_flush();
}

void Plan::prof_flush() {
    if (recs.empty()) return;
    cudaStreamSynchronize(stream);
    for (Rec &r : recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        bool found = false;
        for (Agg &g : agg)
            if (g.name == r.name) { g.n++; g.ms += ms; g.bytes += r.bytes; found = true; break; }
        if (!found) agg.push_back(Agg{r.name, 1, (double)ms, r.bytes});
        timers[4] += ms * 1e-3;
        if (strncmp(r.name, "layout", 6) == 0) timers[1] += ms * 1e-3; else timers[0] += ms * 1e-3;
        evpool.push_back(r.a);
        evpool.push_back(r.b);
    }
    recs.clear();
}

void plan_destroy(Plan *p) {
    if (!p) return;
    if (p->stream) cudaStreamSynchronize(p->stream);
    p->prof_flush();
    for (cudaEvent_t e : p->evpool) cudaEventDestroy(e);
    for (void *m : p->scratch) cudaFree(m);
    free_fft_table(p->tx); free_fft_table(p->ty); free_fft_table(p->tz);
    free_fft4_table(p->tx4); free_fft4_table(p->ty4); free_fft4_table(p->tz4);
    if (p->dgeo) cudaFree(p->dgeo);
    if (p->dgeof) cudaFree(p->dgeof);
    if (p->dgeoq) cudaFree(p->dgeoq);
    if (p->dwtwq) cudaFree(p->dwtwq);
    if (p->dlapc) cudaFree(p->dlapc);
    if (p->dxtw) cudaFree(p->dxtw);
    if (p->dred) cudaFree(p->dred);
    if (p->dwtw) cudaFree(p->dwtw);
    if (p->hred) cudaFreeHost(p->hred);
    if (p->copy_stream) { cudaStreamSynchronize(p->copy_stream); cudaStreamDestroy(p->copy_stream); }
    for (cudaEvent_t e : p->xfer_ev)
        if (e) cudaEventDestroy(e);
    if (p->stream && !p->owner) cudaStreamDestroy(p->stream);  // a companion borrows its owner's
    delete p;
}

}  // namespace sg
