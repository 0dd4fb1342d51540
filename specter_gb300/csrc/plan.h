// Host-side plan: grid geometry, wavenumbers, FC-Gram table and FFT tables for one grid.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fft.cuh"

namespace sg {

struct Batch;  // batch.h

// Plans are FP64 or FP32; FF (float-float) is the precision of internal tables and kernels of
// the precision form on FP64 plans.
enum Prec { FP64 = 0, FP32 = 1, FF = 2 };

// error status shared with the C-ABI (include/specter_gpu.h)
enum Status {
    OK = 0, ERR_SHAPE = 1, ERR_TABLE = 2, ERR_BC = 3, ERR_OOM = 4, ERR_CUDA = 5,
    ERR_NONFINITE = 6, ERR_ARG = 7, ERR_STATE = 9
};

void set_error(const std::string &msg);

struct FFTTable {
    FFTDesc d{};
    void *mem = nullptr;  // one device allocation holding tw / chirp / filters
};

// tables of the register four-step engine (fft4.cuh) for one axis; ok == 0 when the axis
// length has no compiled four-step kernel and the generic engine is used
struct FFT4Desc {
    int n, L, L1, L2, blue;
    const void *tw4, *chirp, *filtb;  // Bluestein: inverse chirp and filter (fft4.cuh)
};
struct FFT4Table {
    FFT4Desc d{};
    void *mem = nullptr;
    int ok = 0;
};

// Geometry passed to kernels by value.
struct Geo {
    int nx, ny, nz, cz, oz, nxh, nzp, ldx, H;
    const double *kx, *ky, *kz, *z, *dir;     // device, FP64
    const double *fx, *fy, *fz;               // fc_filter factors per axis (FP64)
    const float *kxf, *kyf, *kzf, *zf;         // the same tables rounded to FP32, so FP32
    const float *fxf, *fyf, *fzf;             // kernels do no FP64 conversion per element
    const ff *kxq, *kyq, *kzq, *zq;           // and split into float-float pairs, for the
    const ff *fxq, *fyq, *fzq, *dirq;         // float-float kernels of the precision form
    const double *lapc;                       // per (ky, kx) column: kh, exp(-kh Lz), Neumann 1/(kh (1 - exp(-2 kh Lz)))
    const void *xtw;                          // C2<T>[H+1]: exp(-2*pi*i*k/nx)
    const void *wtw;                          // double2[nz]: exp(+2*pi*i*k*(nzp-1)/nz)
    const void *wtwq;                         // the same as float-float complex (ffc[nz])
    double Lz;
    // table entries in the kernel's precision: (T)kx[i], read from the matching table
#define SG_GEO_TABLE(NAME, D, F, Q) \
    template <typename T> __device__ __forceinline__ T NAME(int i) const { \
        if constexpr (is_f64<T>) return __ldg(D + i); \
        else if constexpr (is_f32<T>) return __ldg(F + i); \
        else { const float2 v = __ldg((const float2 *)(Q + i)); return ff(v.x, v.y); } }
    SG_GEO_TABLE(KX, kx, kxf, kxq)
    SG_GEO_TABLE(KY, ky, kyf, kyq)
    SG_GEO_TABLE(KZ, kz, kzf, kzq)
    SG_GEO_TABLE(ZZ, z, zf, zq)
    SG_GEO_TABLE(FX, fx, fxf, fxq)
    SG_GEO_TABLE(FY, fy, fyf, fyq)
    SG_GEO_TABLE(FZ, fz, fzf, fzq)
#undef SG_GEO_TABLE
};

struct Plan {
    Prec prec = FP64;
    std::string tdir;         // FC-Gram table directory the plan was built from
    // A companion plan (the FP32 plan of the nonlinear term of a mixed-precision solver) runs on
    // its owner's stream and counts and profiles its launches in its owner's records.
    Plan *owner = nullptr;
    // while set, the batchable launchers record into it instead of launching (batch.h)
    Batch *batch = nullptr;
    int nx = 0, ny = 0, nz = 0, cz = 0, oz = 0, nxh = 0, nzp = 0, ldx = 0, H = 0;
    double Lx = 1, Ly = 1, Lz = 1, Dkx = 1, Dky = 1, Dkz = 1, dz = 1;
    std::vector<double> kx, ky, kz, z, dir, fx, fy, fz;
    double *dgeo = nullptr;   // device block holding kx, ky, kz, z, dir, fx, fy, fz
    float *dgeof = nullptr;   // the same block rounded to FP32
    ff *dgeoq = nullptr;      // and split into float-float pairs
    void *dwtwq = nullptr;    // inverse-z twiddles at the top wall as float-float complex
    double *dlapc = nullptr;  // laplace_z column constants (Geo::lapc)
    void *dxtw = nullptr;
    FFTTable tx, ty, tz;      // lengths H = nx/2, ny, nz
    FFT4Table tx4, ty4, tz4;  // four-step tables of the same lengths (FP32 plans)
    cudaStream_t stream = nullptr;
    // host transfers of several fields: copies on their own stream, double-buffered staging
    // (scratch slots kStageSlot, kStageSlot + 1) and events ordering copies with conversions
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t xfer_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    Geo geo{};
    // scratch (lazily allocated, complex fields / small buffers)
    std::vector<void *> scratch;
    double *dred = nullptr;   // reduction partials (FP64)
    double *dwtw = nullptr;   // exp(+2 pi i k (nzp-1)/nz), k < nz: inverse-z twiddles at the top wall
    double *hred = nullptr;   // pinned host mirror
    int nred = 0;
    // per-phase timers (s), mirroring the reference's ffttime/tratime/comtime/conttime/tottime
    double timers[6] = {0, 0, 0, 0, 0, 0};
    // kernel accounting: launches counted always; with profiling on, every launch is bracketed
    // by CUDA events on the plan stream and attributed to its kernel name with its
    // algorithmic bytes (compulsory reads + writes of that launch)
    // Upper bounds on the tile width of each pass family (z passes, y passes, x passes, fused
    // column kernels), set by the autotuner; a launcher uses min(cap, largest width that fits).
    enum { kTileZ = 0, kTileY = 1, kTileX = 2, kTileFused = 3 };
    int tile_cap[4] = {16, 16, 16, 16};
    // fused velocity stage as two kernels (per-component update, then the projection) or one
    int velocity_split = 1;
    // threads per block of the float-float column kernels (nl_fp32 form) on the generic
    // engine: 256 or 384
    int ff_threads = 384;
    // float-float column kernels: 1 = the three-step Bluestein engine (ffblue.cuh) where the z
    // length has one, 0 = always the generic engine
    int ff_engine = 1;
    // block shape of those kernels on the three-step engine: 0 = one 576-thread block per SM
    // (tile width 8), 1 = two 288-thread blocks (width 4); for the projection and for the other
    // column kernels separately
    int ff_pair_proj = 0;
    int ff_pair_cols = 0;
    // on that engine, wall round trips as window corrections of the spectrum (1) or as an inverse
    // and a forward transform (0)
    int ff_zoom = 1;
    // FP32 companion plans of the precision form: the nonlinear term's inputs are the owner's
    // float-float state fields (z_inverse reads the rounded sum of each pair)
    int nl_input_ff = 0;
    int capped(int t, int kind) const { return t < tile_cap[kind] ? t : tile_cap[kind]; }
    long long launches = 0;
    bool profile = false;
    struct Rec { const char *name; double bytes; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> evpool;
    struct Agg { std::string name; long long n; double ms, bytes; };
    std::vector<Agg> agg;
    void prof_begin(const char *name, double bytes);
    void prof_end();
    void prof_flush();

    size_t elt() const { return prec == FP64 ? 16 : 8; }                // bytes per complex element
    size_t rel() const { return prec == FP64 ? 8 : 4; }                 // bytes per real element
    size_t field_elems() const { return (size_t)nz * ny * ldx; }        // complex elements, kx fastest
    size_t field_bytes() const { return field_elems() * elt(); }
    size_t real_elems() const { return (size_t)nz * ny * nx; }
    void *scratch_field(int i);
};

// Brackets one kernel launch: counts it and, with profiling on, records CUDA events around it
// attributed to `name` with `bytes` algorithmic bytes.
struct Launch {
    Plan &P;
    Launch(Plan &p, const char *name, double bytes) : P(p) { P.prof_begin(name, bytes); }
    ~Launch() { P.prof_end(); }
};

int plan_create(Plan **out, const int n[3], const int c[3], const int o[3], const double len[3],
                const char *tdir, int prec);
void plan_destroy(Plan *p);
// device bytes held by the plan: tables and the scratch fields allocated so far (an estimate
// for the tables, exact for the scratch fields)
unsigned long long plan_bytes(const Plan &P);
// FC-Gram tables A{C}-{d}.dat, Q{d}.dat under tdir: out = {max |Q^T Q - I|, max |dir|,
// max_i sum_j |dir_ij|} with dir = A Q^T
int table_check(const char *tdir, int C, int d, double out[3]);
int build_fft_table(FFTTable &t, int n, Prec prec);
void free_fft_table(FFTTable &t);
int build_fft4_table(FFT4Table &t, int n, int axis);  // fast_f32.cu; axis 0 = x, 1 = y, 2 = z
void free_fft4_table(FFT4Table &t);

}  // namespace sg
