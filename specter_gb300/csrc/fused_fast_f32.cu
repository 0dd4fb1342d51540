// Fused column kernels on the FP32 register four-step engine, large z lengths: 538 and 282 via
// Bluestein over 1080 = 36*30 and 576 = 24*24.  The smaller z splits are compiled in
// fused_small_f32.cu.
#include "fast.h"
#include "fused_launch.cuh"

namespace sg {

int fast_fused_small(Plan &P, const FusedArgs &a, int which, double bytes);

int fast_fused(Plan &P, const FusedArgs &a, int which, double bytes) {
    if (P.prec != FP32 || !P.tz4.ok) return kNoFast;
    if (fft4_ensure_tables() != cudaSuccess) { set_error("constant table upload failed"); return ERR_CUDA; }
    const int l1 = P.tz4.d.L1, l2 = P.tz4.d.L2;
    if (l1 == 36 && l2 == 30) return launch_fused<float, FourStep<float, 36, 30, true>, 8>(P, P.tz4.d, a, which, bytes);
    if (l1 == 24 && l2 == 24) return launch_fused<float, FourStep<float, 24, 24, true>, 8>(P, P.tz4.d, a, which, bytes);
    return fast_fused_small(P, a, which, bytes);
}

}  // namespace sg
