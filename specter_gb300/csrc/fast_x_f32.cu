// FP32 register four-step x passes (c2r, r2c and the fused nonlinear x pass).
#include "fast_launch.cuh"

namespace sg {

cudaError_t fast_x_init() { return fft4_ensure_tables(); }

int fast_x(Plan &P, const XArgs &a, int nf, bool r2c, double bytes) {
    return dispatch_x(P, P.tx4, [&](auto l1, auto l2) { return xpass<decltype(l1)::value, decltype(l2)::value>(P, a, nf, r2c, bytes); });
}
int fast_x_nl(Plan &P, const XNLArgs &a, double bytes) {
    return dispatch_x(P, P.tx4, [&](auto l1, auto l2) { return xnl<decltype(l1)::value, decltype(l2)::value>(P, a, bytes); });
}

}  // namespace sg
