// Shared definitions for the RNNG GB300 library: status codes, the context, the
// device scratch arena and small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "../../include/rnng_gpu.h"

namespace rnng {

// Raised inside the library and turned into a status code at the C boundary.
struct Error {
    int code;
    std::string msg;
};

#define RNNG_CUDA(call)                                                                                  \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            throw ::rnng::Error{RNNG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                                                   __FILE__ + ":" + std::to_string(__LINE__) + ")"};     \
        }                                                                                                \
    } while (0)

#define RNNG_REQUIRE(cond, code, text)                 \
    do {                                               \
        if (!(cond)) throw ::rnng::Error{(code), (text)}; \
    } while (0)

// Slots of the context's 64-bit device counter array (counters): 0-1 pruning, 2-3 edit counts,
// 4 edges, 5 candidates, 6 query hits, 9 edit maximum length, 10-11 rips checks,
// 12 ball widening (two floats), 13 non-finite input seen, 14 largest input magnitude
// (float bits).
constexpr int kCounterSlots = 16;
constexpr int kSlotNonfinite = 13;
constexpr int kSlotQueue = 7;  // the Gram kernel's work-queue head

// A growable device buffer owned by the context.  Buffers are reused across calls
// so that steady-state calls do not allocate.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    void reserve(size_t want)
    {
        if (want <= bytes) return;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t grow = want + want / 4 + 256;
        RNNG_CUDA(cudaMalloc(&ptr, grow));
        bytes = grow;
    }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const { return reinterpret_cast<T*>(ptr); }
};

// Device-side error word: kernels with bounded waits record a code here instead
// of spinning forever; the host checks it after the stage.
enum DeviceFault : int {
    FAULT_NONE = 0,
    FAULT_MBAR_TIMEOUT = 1,
    FAULT_QUEUE = 2,
};

// One row of the Gram kernel's tuning table (rnng_gb300/gram_tuning.json, written by the
// autotuner rnng_gb300/tune.py): for operands of padded width dp of one kind and at least
// min_pairs tile pairs, nt column tiles per item, chunk items per queue chunk and at most
// slots B slots per CTA (0: as many as fit).
struct GramTune {
    int kind = 0;               // 0: BF16 L2 tiles, 1: the FP8 edit-distance filter
    int dp = 0;
    long long min_pairs = 0;
    int nt = 0, chunk = 0, slots = 0;
};

}  // namespace rnng

// The context: one device, one stream, reusable scratch, last-call statistics.
struct rnng_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    rnng_stats stats{};
    // named scratch buffers
    rnng::DevBuf x_in, ids_in, x_sorted, xb_sorted, norms, perm, keys, keys_alt, perm_alt, cell, dist, pivots,
        tile_lo, tile_hi, super_lo, super_hi, pair_list, super_list, counters, edges_u, edges_v, edges_w,
        out_u, out_v, out_w, cub_tmp, cand, aux0, aux1, aux2, aux3, aux4, aux5, aux6, aux7, sched, clq0, clq1,
        hi_id, hi_val, hi_flag, sflag, vflag, items, items_tmp, sched_tmp, sym, shift_buf, ball_b16, ball_info, sball_b16,
        sball_info, lm_b16, xb_sortedB, part_k, part_v, part_f,
        fin_x, fin_idx;
    rnng::DevBuf host_stage;  // pinned host memory (cudaMallocHost), not device memory
    unsigned long long edge_cap_hint = 0, cand_cap_hint = 0;
    int64_t last_candidates = 0;
    // BF16 Gram operands of the current call: TMA descriptor (a CUtensorMap), padded
    // dimension, per-row candidate-test data and the widened radius
    alignas(64) unsigned char tmap[128] = {};
    alignas(64) unsigned char tmapB[128] = {};  // column-tile operand when the column terms are folded
    bool bf16_fold = false;
    int bf16_dp = 0;
    void* bf16_rowinfo = nullptr;
    void* bf16_ucol = nullptr;
    void* bf16_tileinfo = nullptr;
    float bf16_eps_p = 0.f;
    int* fault_word = nullptr;  // device error word written by kernels with bounded waits
    int64_t launches = 0;       // kernels launched by the current call
    double gram_ms = 0.0;       // device time of the Gram kernel launches of the current call
    cudaEvent_t ev[16] = {};
    bool have_events = false;
    std::vector<rnng::GramTune> gram_table;  // loaded at creation
    rnng::GramTune gram_force;                // rnng_ctx_set_gram_tuning (0 fields: not forced)
    bool fault_drill = false;                 // rnng_ctx_fault_drill
};

namespace rnng {

// Runs an entry point's body on the context's device and turns exceptions into a
// status code, keeping the message for rnng_last_error().
template <class F>
int guarded(rnng_ctx* ctx, F&& body)
{
    if (!ctx) return RNNG_ERR_INVALID;
    try {
        RNNG_CUDA(cudaSetDevice(ctx->device));
        body();
        ctx->last_error.clear();
        return RNNG_OK;
    } catch (const Error& e) {
        ctx->last_error = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        ctx->last_error = "host allocation failed";
        return RNNG_ERR_NOMEM;
    } catch (...) {
        ctx->last_error = "unknown error";
        return RNNG_ERR_INVALID;
    }
}

inline void ensure_events(rnng_ctx* c)
{
    if (c->have_events) return;
    for (auto& e : c->ev) RNNG_CUDA(cudaEventCreate(&e));
    c->have_events = true;
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Kernels one CUB radix sort launches: a single-tile kernel for small inputs,
// otherwise histogram + exclusive sum + one onesweep pass per 8 key bits.
inline int cub_sort_kernels(int64_t n, int bits)
{
    if (n <= 1) return 0;
    if (n <= 4096) return 1;
    return 2 + (bits + 7) / 8;
}

// Reference L2 (drivers/systolic.cpp:253-269): sequential difference-square-sum in
// float without contraction, then a correctly rounded square root.  The explicit
// _rn intrinsics are never fused into FMA by the compiler.
__device__ __forceinline__ float l2seq_acc(float acc, float a, float b)
{
    float d = __fsub_rn(a, b);
    return __fadd_rn(acc, __fmul_rn(d, d));
}

// NaN or +-infinity: every exponent bit set.
__device__ __forceinline__ bool nonfinite_f32(float v) { return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u; }

// Warp-level tensor-core product c += A B (mma.sync m16n8k16, BF16 operands, FP32
// accumulator) on the standard fragments: a0..a3 = A rows (g, g + 8) x k-slots
// (2t, 2t + 1) and (2t + 8, 2t + 9); b0, b1 = B column g x the same k-slots; c0..c3 =
// rows (g, g + 8) x columns (2t, 2t + 1), with g = lane / 4, t = lane % 4.
__device__ __forceinline__ void mma_bf16_16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// 16-byte asynchronous copy global -> shared (both addresses 16-byte aligned), its group
// commit and the wait for all but the newest n groups.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace rnng
