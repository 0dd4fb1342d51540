#include "fused.h"

namespace sg {

struct FusedState {
    StageParams sp;
};

int fused_create(Plan &P, const StageParams &sp, FusedState **out) {
    (void)P; (void)sp;
    *out = nullptr;
    set_error("fused stage path is not available in this build");
    return ERR_ARG;
}
void fused_destroy(FusedState *fs) { delete fs; }
int fused_stage(Plan &P, FusedState *fs, int o, void *const v[4], void *pr, const void *const Cold[4]) {
    (void)P; (void)fs; (void)o; (void)v; (void)pr; (void)Cold;
    set_error("fused stage path is not available in this build");
    return ERR_ARG;
}

}  // namespace sg
