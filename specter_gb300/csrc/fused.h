// Fused GB300 RK-stage path: column kernels that keep a z column tile resident in shared
// memory from the nonlinear term's forward z transform through the RK update, the wall
// conditions and the pressure projection.
#pragma once

#include "ops.h"

namespace sg {

struct FusedState;

int fused_create(Plan &P, const StageParams &sp, FusedState **out);
void fused_destroy(FusedState *fs);
int fused_stage(Plan &P, FusedState *fs, int o, void *const v[4], void *pr, const void *const Cold[4]);

}  // namespace sg
