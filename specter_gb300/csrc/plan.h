// Host-side plan: grid geometry, wavenumbers, FC-Gram table and FFT tables for one grid.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fft.cuh"

namespace sg {

enum Prec { FP64 = 0, FP32 = 1 };

// error status shared with the C-ABI (include/specter_gpu.h)
enum Status {
    OK = 0, ERR_SHAPE = 1, ERR_TABLE = 2, ERR_BC = 3, ERR_OOM = 4, ERR_CUDA = 5,
    ERR_NONFINITE = 6, ERR_ARG = 7, ERR_TIMEOUT = 8, ERR_STATE = 9
};

void set_error(const std::string &msg);

struct FFTTable {
    FFTDesc d{};
    void *mem = nullptr;  // one device allocation holding tw / chirp / filters
};

// Geometry passed to kernels by value.
struct Geo {
    int nx, ny, nz, cz, oz, nxh, nzp, ldx, H;
    const double *kx, *ky, *kz, *z, *dir;     // device, FP64
    const double *fx, *fy, *fz;               // fc_filter factors per axis (FP64)
    const void *xtw;                          // C2<T>[H+1]: exp(-2*pi*i*k/nx)
    double Lz;
};

struct Plan {
    Prec prec = FP64;
    int nx = 0, ny = 0, nz = 0, cz = 0, oz = 0, nxh = 0, nzp = 0, ldx = 0, H = 0;
    double Lx = 1, Ly = 1, Lz = 1, Dkx = 1, Dky = 1, Dkz = 1, dz = 1;
    std::vector<double> kx, ky, kz, z, dir, fx, fy, fz;
    double *dgeo = nullptr;   // device block holding kx, ky, kz, z, dir, fx, fy, fz
    void *dxtw = nullptr;
    FFTTable tx, ty, tz;      // lengths H = nx/2, ny, nz
    cudaStream_t stream = nullptr;
    Geo geo{};
    // scratch (lazily allocated, complex fields / small buffers)
    std::vector<void *> scratch;
    double *dred = nullptr;   // reduction partials (FP64)
    double *dwtw = nullptr;   // exp(+2 pi i k (nzp-1)/nz), k < nz: inverse-z twiddles at the top wall
    double *hred = nullptr;   // pinned host mirror
    int nred = 0;
    // per-phase timers (ms), mirroring the reference's ffttime/tratime/comtime/conttime/tottime
    double timers[6] = {0, 0, 0, 0, 0, 0};
    bool profile = false;

    size_t elt() const { return prec == FP64 ? 16 : 8; }                // bytes per complex element
    size_t rel() const { return prec == FP64 ? 8 : 4; }                 // bytes per real element
    size_t field_elems() const { return (size_t)nz * ny * ldx; }        // complex elements, kx fastest
    size_t field_bytes() const { return field_elems() * elt(); }
    size_t real_elems() const { return (size_t)nz * ny * nx; }
    void *scratch_field(int i);
};

int plan_create(Plan **out, const int n[3], const int c[3], const int o[3], const double len[3],
                const char *tdir, int prec);
void plan_destroy(Plan *p);
int build_fft_table(FFTTable &t, int n, Prec prec);
void free_fft_table(FFTTable &t);

}  // namespace sg
