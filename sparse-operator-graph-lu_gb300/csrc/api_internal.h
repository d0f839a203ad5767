// Definitions behind the opaque handles of include/soglu_gb300.h.
#pragma once
#include <string>

#include "../../include/soglu_gb300.h"
#include "plan.h"

struct sog_plan {
    sog::Plan p;
    bool imported = false;
    bool symmetric = false;
    int64_t nnz = 0;  // triplets as given (before mirroring)
};

struct sog_mtx {
    sog::MtxData d;
    bool from_cache = false;
};

namespace sog_internal {
extern thread_local std::string g_err;
int fail(int code, const std::string& msg);
// average tasks per dependency level of a system's task graph; *full_grid
// (if not NULL) receives its uncapped persistent factor grid
double system_parallelism(const sog_system* s, int* full_grid);
// cap the persistent factor and substitution grids (0 = none)
void system_set_grid_cap(sog_system* s, int cap);
}  // namespace sog_internal
