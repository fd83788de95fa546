// Small shared stages: device fault word, edge sorting, uploads and result delivery.
#pragma once

#include "common.cuh"

namespace rnng {

void init_device_fault(rnng_ctx* c);
// Throws RNNG_ERR_DEVICE when a kernel recorded a fault since the last check.
void check_device_fault(rnng_ctx* c);
// Sorts (u, v, w) in place by (u, v) with two stable radix passes.
// Sorts the edge arrays by (u, v) (by_w: by (u, v, w), w >= 0), stably.
void sort_edges_uv(rnng_ctx* c, int64_t* u, int64_t* v, float* w, int64_t m, bool by_w = false);

// Device copy of a host array in `buf` (p itself when it is null or RNNG_INPUT_DEVICE is set).
const void* upload(rnng_ctx* c, DevBuf& buf, const void* p, size_t bytes, unsigned flags);
// The context's pinned host staging block, grown to at least `bytes`.
void* host_stage(rnng_ctx* c, size_t bytes);
// Hands result arrays to the caller: the device arrays themselves with RNNG_OUTPUT_DEVICE,
// else copies (queued on the context stream) in the pinned staging block.  Either way
// they are context-owned and valid until the next call; the caller synchronizes.
void deliver_edges(rnng_ctx* c, const int64_t* du, const int64_t* dv, const float* dw, int64_t m, unsigned flags,
                   rnng_edges* out);
void deliver_simplices(rnng_ctx* c, const int64_t* did, const float* dval, const uint8_t* dflag, int64_t count,
                       unsigned flags, rnng_simplices* out);

}  // namespace rnng
