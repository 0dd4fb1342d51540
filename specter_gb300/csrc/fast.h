// Register four-step FFT passes for the lengths of the production grids (FP32).  Each
// launcher returns kNoFast when the plan has no four-step table for that axis, and the
// caller then runs the generic GPU kernel of the same pass.
#pragma once

#include "kernels.cuh"

namespace sg {

constexpr int kNoFast = -1;

// split of a working length L into L1 * L2 served by compiled four-step kernels (0 if none)
bool fast_pair(int L, int *L1, int *L2);
int fast_init_device();
cudaError_t fast_x_init();  // constant tables of the x-pass unit
cudaError_t fast_y_init();  // constant tables of the y-pass unit
int build_fft4_table(FFT4Table &t, int n);
void free_fft4_table(FFT4Table &t);

int fast_z_inverse(Plan &P, const ZInvArgs &a, int nf, double bytes);
int fast_z_forward(Plan &P, const ZFwdArgs &a, int nf, double bytes);
int fast_y(Plan &P, const YArgs &a, int nf, int nplanes, double bytes);
int fast_x(Plan &P, const XArgs &a, int nf, bool r2c, double bytes);
int fast_x_nl(Plan &P, const XNLArgs &a, double bytes);

}  // namespace sg
