// Fused GB300 RK-stage path: the nonlinear x/y passes, then column kernels that keep a z
// column tile resident in shared memory from the nonlinear term's forward z transform through
// the RK update, the wall conditions and the pressure projection (fused_kernels.cuh).
#pragma once

#include "ops.h"

namespace sg {

struct FusedState;

int fused_create(Plan &P, const StageParams &sp, FusedState **out);
void fused_destroy(FusedState *fs);
// one stage o on the state v (in place), with RK-step start Cold
int fused_stage(Plan &P, FusedState *fs, int o, void *const v[4], void *pr, const void *const Cold[4]);
// one full RK step on the state v: stages ord..1 with the step start held in v itself
// (stage outputs ping-pong through the state's own buffers; no copies)
int fused_step(Plan &P, FusedState *fs, void *const v[4], void *pr, int nsteps = 1);
// device bytes held by the fused-stage buffers (0 for a null state)
unsigned long long fused_bytes(const Plan &P, const FusedState *fs);

}  // namespace sg
