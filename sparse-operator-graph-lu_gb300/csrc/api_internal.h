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
}  // namespace sog_internal
