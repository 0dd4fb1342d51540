// Definitions of the opaque C-ABI handles shared by the translation units that create or read
// them (capi.cu creates them; noalloc.cu reads them).  One definition, so a field added here
// reaches every reader.
#pragma once

#include <cstddef>

#include "plan.h"

// A plan stays alive while fields or solvers made from it exist: specter_plan_destroy only
// drops the caller's reference, so handles may be released in any order.
struct specter_plan {
    sg::Plan *p;
    int refs;
};

struct specter_field {
    specter_plan *plan;
    int kind;
    void *d;
    size_t bytes;
};
