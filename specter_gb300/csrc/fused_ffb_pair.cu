// Float-float column kernels of the precision form on the three-step Bluestein engine, as two
// 288-thread blocks per SM at a tile width of 4 (the plan options ff_pair_proj / ff_pair_cols):
// a translation unit of their own, compiled beside fused_ffb.cu.
#include "fused_launch.cuh"
#include "ops.h"

namespace sg {

int ffb_fused_pair(Plan &P, const FFBDesc &d, const FusedArgs &a, int which, double bytes) {
    // the projection's FP32 pressure transform uses this translation unit's constant twiddles
    if (fft4_ensure_tables() != cudaSuccess) { set_error("constant table upload failed"); return ERR_CUDA; }
    return launch_fused<ff, FFBlue<288, 2>, 4>(P, d, a, which, bytes);
}

}  // namespace sg
