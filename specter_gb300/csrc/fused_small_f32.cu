// Fused column kernels on the FP32 register four-step engine, small z lengths (the ensemble and
// served grids): nz = 154, 122 and 58 via Bluestein over 320 = 20*16, 256 = 16*16 and
// 128 = 16*8, and nz = 90 = 10*9 directly.
#include "fast.h"
#include "fused_launch.cuh"

namespace sg {

int fast_fused_small(Plan &P, const FusedArgs &a, int which, double bytes) {
    if (fft4_ensure_tables() != cudaSuccess) { set_error("constant table upload failed"); return ERR_CUDA; }
    const int l1 = P.tz4.d.L1, l2 = P.tz4.d.L2;
    if (l1 == 20 && l2 == 16) return launch_fused<float, FourStep<float, 20, 16, true>>(P, P.tz4.d, a, which, bytes);
    if (l1 == 16 && l2 == 16) return launch_fused<float, FourStep<float, 16, 16, true>>(P, P.tz4.d, a, which, bytes);
    if (l1 == 16 && l2 == 8) return launch_fused<float, FourStep<float, 16, 8, true>>(P, P.tz4.d, a, which, bytes);
    if (l1 == 10 && l2 == 9) return launch_fused<float, FourStep<float, 10, 9, true>>(P, P.tz4.d, a, which, bytes);
    return kNoFast;
}

}  // namespace sg
