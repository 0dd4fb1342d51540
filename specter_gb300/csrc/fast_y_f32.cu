// FP32 register four-step y passes.
#include "fast_launch.cuh"

namespace sg {

cudaError_t fast_y_init() { return fft4_ensure_tables(); }

int fast_y(Plan &P, const YArgs &a, int nf, int nplanes, double bytes) {
    return dispatch_y(P, P.ty4, [&](auto l1, auto l2) { return ypass<decltype(l1)::value, decltype(l2)::value>(P, a, nf, nplanes, bytes); });
}

}  // namespace sg
