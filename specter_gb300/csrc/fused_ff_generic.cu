// Float-float column kernels of the precision form on the generic Stockham / Bluestein engine
// (z lengths without the three-step engine, and the plan option ff_engine = 0): a translation
// unit of their own, compiled beside fused.cu.
#include "fused_launch.cuh"

namespace sg {

int ff_generic_fused(Plan &P, const FFTDesc &d, const FusedArgs &a, int which, double bytes) {
    if (P.ff_threads == 256) return launch_fused<ff, GenericFFT<ff, 256>>(P, d, a, which, bytes);
    return launch_fused<ff, GenericFFT<ff, 384>>(P, d, a, which, bytes);
}

}  // namespace sg
