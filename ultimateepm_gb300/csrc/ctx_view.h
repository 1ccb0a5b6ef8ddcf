// ctx_view.h -- read-only view of a uepm_ctx's device tables, for entry points outside capi.cu.
#pragma once

#include "uepm_common.cuh"
#include "uepm_gb300.h"

namespace uepm {

struct CtxTables {
    DevParams         P;
    const int*        d_G;
    const cx<double>* Vloc;
    const double2*    phNL;
    const double2*    phSO;
    int               N, n;
};

// Fills `out` from `ctx`; false for a null context.
bool ctx_tables(const uepm_ctx* ctx, CtxTables* out);

}  // namespace uepm
