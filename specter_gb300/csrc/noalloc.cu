// specter_bouncheck_z_static: the wall check of specter_bouncheck_z with all of its working
// memory in a fixed device array instead of buffers allocated on demand.
//
// Who needs it: a caller that has handed the whole device memory budget to something else and
// must not allocate afterwards -- the serving loop that admits simulations against an HBM budget,
// or a driver that reserves all memory up front -- and a caller in the middle of the RK loop that
// cannot afford the device-wide synchronisation cudaMalloc/cudaFree imply.  Those callers get the
// same no-slip wall diagnostic without any allocation.
//
// Limits and sharing:
//   - the array holds the wall values of at most kMaxColumns (kx, ky) columns per field, two
//     fields, plus the block partial sums: 4 MiB + 4 KiB, resident on every GPU that loads the
//     library until the process exits.  Grids with more columns ((nx/2+1)*ny > 65536) are
//     rejected with SPECTER_ERR_SHAPE.
//   - every call uses the same array; calls that overlap on the GPU (from different streams or
//     threads) race on it and must be serialised by the caller.  Each call writes every slot it
//     reads afterwards, and clears the two result slots before use.
//   - the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current and keeps it for later calls; make that first call before any stream
//     capture.  The lookup is guarded by a mutex, so first calls from several host threads are
//     safe.  cudaDeviceReset unloads the module and leaves the kept address stale: a process that
//     resets a device must not call this entry point on that device afterwards.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/specter_gpu.h"
#include "handles.h"
#include "kernels_elem.cuh"
#include "ops.h"

namespace sg {

constexpr int kMaxColumns = 65536;
constexpr int kStaticBlocks = 152;
// layout (double2 units): [field A walls: 2*kMaxColumns][field B walls: 2*kMaxColumns]
//                         [partials: 2*kStaticBlocks doubles][result: 2 doubles]
constexpr size_t kWallSlots = 2 * (size_t)kMaxColumns;
constexpr size_t kStaticDoubles = 2 * 2 * kWallSlots + 2 * (size_t)kStaticBlocks + 2;

static __device__ __align__(256) double g_wall_scratch[kStaticDoubles];

// Sums the block partials in block order and scales them twice by 1/(nx ny nz), the same
// operations in the same order as the allocating variant's host-side sum: out = {bottom, top}.
static __global__ void k_wall_finish(const double *partial, int nblocks, double inv, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double bot = 0.0, top = 0.0;
    for (int b = 0; b < nblocks; b++) {
        bot += partial[2 * b];
        top += partial[2 * b + 1];
    }
    out[0] = bot * inv * inv;
    out[1] = top * inv * inv;
}

// device address of g_wall_scratch for each device, looked up once with that device current
static std::mutex g_addr_mutex;
static double *g_addr[64] = {nullptr};

static double *scratch_address() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        double *p = nullptr;
        if (cudaGetSymbolAddress((void **)&p, g_wall_scratch) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_addr[dev] = p;
    }
    return g_addr[dev];
}

template <typename T>
static int wall_check_static(Plan &P, const void *a, const void *b, double *bot, double *top) {
    double *base = scratch_address();
    if (!base) { set_error("cudaGetSymbolAddress failed for the static wall-check array"); return ERR_CUDA; }
    double2 *bcA = (double2 *)base, *bcB = bcA + kWallSlots;
    double *partial = base + 2 * 2 * kWallSlots, *result = partial + 2 * kStaticBlocks;
    const double2 *wtw = (const double2 *)P.dwtw;
    const dim3 grid(cdiv(P.nxh, 64), P.ny);
    const double col = (double)P.nz * P.ny * P.nxh * (double)P.elt();  // one field read
    if (cudaMemsetAsync(result, 0, 2 * sizeof(double), P.stream) != cudaSuccess) return check_launch("bouncheck_z_static clear");
    { Launch L_(P, "wall_eval", col); k_wall_eval<T><<<grid, 64, 0, P.stream>>>(P.geo, (const C2<T> *)a, 1.0, wtw, bcA, 0); }
    if (int st = check_launch("bouncheck_z_static wall_eval")) return st;
    if (b) {
        { Launch L_(P, "wall_eval", col); k_wall_eval<T><<<grid, 64, 0, P.stream>>>(P.geo, (const C2<T> *)b, 1.0, wtw, bcB, 0); }
        if (int st = check_launch("bouncheck_z_static wall_eval")) return st;
    }
    { Launch L_(P, "reduce_walls", 64.0 * P.nxh * P.ny); k_reduce_walls<<<kStaticBlocks, kThreads, 0, P.stream>>>(P.geo, bcA, b ? bcB : nullptr, partial); }
    if (int st = check_launch("bouncheck_z_static reduce_walls")) return st;
    const double inv = 1.0 / (double)((long long)P.nx * P.ny * P.nz);
    { Launch L_(P, "wall_finish", 16.0 * kStaticBlocks); k_wall_finish<<<1, 32, 0, P.stream>>>(partial, kStaticBlocks, inv, result); }
    if (int st = check_launch("bouncheck_z_static wall_finish")) return st;
    double host[2];
    if (cudaMemcpyAsync(host, result, sizeof host, cudaMemcpyDeviceToHost, P.stream) != cudaSuccess ||
        cudaStreamSynchronize(P.stream) != cudaSuccess) {
        set_error(std::string("bouncheck_z_static: ") + cudaGetErrorString(cudaGetLastError()));
        return ERR_CUDA;
    }
    *bot = host[0];
    *top = host[1];
    return OK;
}

}  // namespace sg

extern "C" int specter_bouncheck_z_static(specter_plan *plan, const specter_field *a, const specter_field *b,
                                          double *bot, double *top) {
    using namespace sg;
    if (!plan || !plan->p || !a || !a->d || !bot || !top) { set_error("null argument"); return SPECTER_ERR_ARG; }
    if (a->plan != plan || (b && b->plan != plan)) { set_error("field belongs to a different plan"); return SPECTER_ERR_STATE; }
    if (a->kind != SPECTER_COMPLEX || (b && b->kind != SPECTER_COMPLEX)) { set_error("expected complex fields"); return SPECTER_ERR_ARG; }
    Plan &P = *plan->p;
    const long long ncol = (long long)P.nxh * P.ny;
    if (ncol > kMaxColumns) {
        set_error("bouncheck_z_static: the grid has " + std::to_string(ncol) + " (kx, ky) columns; the static array holds at most " +
                  std::to_string(kMaxColumns) + " (use specter_bouncheck_z)");
        return SPECTER_ERR_SHAPE;
    }
    return P.prec == FP64 ? wall_check_static<double>(P, a->d, b ? b->d : nullptr, bot, top)
                          : wall_check_static<float>(P, a->d, b ? b->d : nullptr, bot, top);
}
