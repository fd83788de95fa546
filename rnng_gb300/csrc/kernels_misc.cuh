// Small shared stages: device fault word, edge sorting.
#pragma once

#include "common.cuh"

namespace rnng {

void init_device_fault(rnng_ctx* c);
// Throws RNNG_ERR_DEVICE when a kernel recorded a fault since the last check.
void check_device_fault(rnng_ctx* c);
// Sorts (u, v, w) in place by (u, v) with two stable radix passes.
void sort_edges_uv(rnng_ctx* c, int64_t* u, int64_t* v, float* w, int64_t m);

}  // namespace rnng
