// Register four-step FFT passes for the lengths of the production grids (FP32).  Each
// launcher returns kNoFast when the plan has no four-step table for that axis, and the
// caller then runs the generic GPU kernel of the same pass.
#pragma once

#include "kernels.cuh"

namespace sg {

constexpr int kNoFast = -1;

// Compiled four-step splits L = L1 * L2 per axis.  z: the Bluestein lengths of nz = 538, 282,
// 154, 122 and 58 (1080, 576, 320, 256, 128) and nz = 90 directly; y: ny = 512 ... 32; x:
// H = nx/2 = 512 ... 16.  Every L1 is even (the Bluestein body halves step A and A' on L1).
#define SG_FAST_PAIRS_Z(F) F(36, 30) F(24, 24) F(20, 16) F(16, 16) F(16, 8) F(10, 9)
#define SG_FAST_PAIRS_Y(F) F(32, 16) F(16, 16) F(16, 8) F(12, 8) F(8, 8) F(8, 6) F(8, 4)
#define SG_FAST_PAIRS_X(F) F(32, 16) F(16, 16) F(16, 8) F(8, 8) F(8, 6) F(8, 4) F(6, 4) F(4, 4)

enum FastAxis { kFastX = 0, kFastY = 1, kFastZ = 2 };  // the axis argument of build_fft4_table

// split of a working length L on an axis into L1 * L2 served by compiled four-step kernels
bool fast_pair(int axis, int L, int *L1, int *L2);
int fast_init_device();
cudaError_t fast_x_init();  // constant tables of the x-pass unit
cudaError_t fast_y_init();  // constant tables of the y-pass unit
int build_fft4_table(FFT4Table &t, int n, int axis);
void free_fft4_table(FFT4Table &t);

int fast_z_inverse(Plan &P, const ZInvArgs &a, int nf, double bytes);
int fast_z_forward(Plan &P, const ZFwdArgs &a, int nf, double bytes);
int fast_y(Plan &P, const YArgs &a, int nf, int nplanes, double bytes);
int fast_x(Plan &P, const XArgs &a, int nf, bool r2c, double bytes);
int fast_x_nl(Plan &P, const XNLArgs &a, double bytes);

}  // namespace sg
