// BF16 tensor-core Gram tiles with a rigorous margin and an exact FP32 recheck.
//
// For a surviving tile pair (I, J) the squared distances of all 128 x 128 point
// pairs are estimated as ||x~||^2 + ||y~||^2 - 2 x~.y~, where x~ = bf16(x - c) is
// the point shifted by a per-dimension constant c and rounded to BF16.  The dot
// products run on the 5th-generation tensor cores (tcgen05.mma kind::f16, BF16
// inputs, FP32 accumulator in tensor memory); operands are staged in shared memory
// by TMA with 128-byte swizzling.  A pair becomes a candidate when
//
//     D~ <= (eps' + a_x + a_y)^2 + q_x + q_y
//
// where a_x >= ||(x - c) - x~|| bounds the BF16 rounding of the point, q_x bounds
// the FP32 error of the Gram form (tensor-core accumulation, norms, the final
// combination) and eps' = eps * (1 + (d+8) 2^-24) covers the rounding of the
// reference's own L2.  So every pair with L2seq(x, y) <= eps is a candidate, and
// each candidate is then re-evaluated with the reference's sequential FP32 L2 in a
// separate kernel: the edge set and every weight are exactly the reference's.
//
// Kernel roles (one CTA per SM, persistent over the tile-pair list):
//   warp 0      TMA producer: K-chunks of 64 BF16 (one 128 B swizzle span) of the
//               A tile (rows of I) and B tile (rows of J) into a 4-stage ring
//   warp 1      MMA issuer: 4 x (M=128, N=128, K=16) per chunk into one of two
//               TMEM accumulators (2 x 128 columns)
//   warps 2-5   epilogue: tcgen05.ld of the accumulator rows (one TMEM lane per
//               point of I), candidate test, warp-aggregated append
// Every mbarrier wait is bounded (about one second of wall time); on timeout the
// CTA records a fault code in the context's fault word, stops issuing work, waits
// (bounded) for its own copies and MMAs in flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>

#include "common.cuh"
#include "eps_l2.cuh"

namespace rnng {

constexpr int kNS = 4;                              // shared-memory ring stages
constexpr int kChunkK = 64;                         // BF16 elements per K-chunk
constexpr int kChunkBytes = kTile * kChunkK * 2;    // 16 KB per operand per chunk
constexpr int kStageBytes = 2 * kChunkBytes;        // A + B
constexpr int kAccCols = 128;                       // fp32 accumulator columns (N)
constexpr int kTmemCols = 2 * kAccCols;
constexpr int kEpiWarps = 4;
constexpr int kGramThreads = 64 + 32 * kEpiWarps;   // 192
constexpr uint64_t kWaitNs = 1000000000ull;         // bounded wait: 1 s

struct GramSmem {
    // offsets inside the dynamic shared block (which is 1024-aligned)
    static constexpr int stages = 0;
    static constexpr int colinfo = kNS * kStageBytes;                   // kEpiWarps x 128 float4
    static constexpr int bars = colinfo + kEpiWarps * kTile * 16;       // mbarriers
    static constexpr int nbars = 2 * kNS + 2 + 2 + 1;                   // full, empty, tfull, tempty, drain
    static constexpr int misc = bars + nbars * 8;                       // tmem slot, abort flag
    static constexpr int total = misc + 16;
};

// ------------------------------------------------------------------------------------------------
// PTX wrappers

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait.  Returns false when the CTA is aborting or the wait ran out; in
// the latter case it records the fault and raises the CTA's abort flag.
__device__ __noinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* fault,
                                       int where)
{
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u) {
            if (*abort_flag) return false;
            uint64_t now = globaltimer();
            if (t0 == 0) t0 = now;
            else if (now - t0 > kWaitNs) {
                if (atomicCAS(fault, FAULT_NONE, FAULT_MBAR_TIMEOUT) == FAULT_NONE) {
                    fault[1] = where;
                    fault[2] = (int)blockIdx.x;
                }
                *abort_flag = 1;
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 consecutive fp32 columns: thread t receives row (lane base + t).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%"
        "19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row core
// groups 1024 bytes apart (SBO), descriptor version 1 (sm_100 family).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;               // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset
    d |= (uint64_t)1 << 46;               // version
    d |= (uint64_t)2 << 61;               // SWIZZLE_128B
    return d;
}

// Instruction descriptor for kind::f16: D f32, A and B bf16, both K-major, M = N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kAccCols >> 3) << 17) |
                            ((uint32_t)(kTile >> 4) << 24);

// ------------------------------------------------------------------------------------------------
// the Gram kernel

__global__ void __launch_bounds__(kGramThreads, 1)
    k_gram_bf16(const __grid_constant__ CUtensorMap tmap, const int2* __restrict__ pairs,
                const unsigned long long* __restrict__ npairs_ptr, unsigned long long pair_cap, int kchunks,
                const float4* __restrict__ rowinfo, int64_t n, float eps_p, float kappa, uint2* __restrict__ cand,
                unsigned long long* __restrict__ cand_count, unsigned long long cand_cap, int* __restrict__ fault)
{
    extern __shared__ __align__(1024) uint8_t gsm_raw[];
    // align the dynamic block to 1024 bytes (swizzle atoms)
    uint8_t* sm = (uint8_t*)(((uintptr_t)gsm_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(sm + GramSmem::bars);
    uint64_t* full = bars;
    uint64_t* empty = bars + kNS;
    uint64_t* tfull = bars + 2 * kNS;
    uint64_t* tempty = bars + 2 * kNS + 2;
    uint64_t* drain = bars + 2 * kNS + 4;
    uint32_t* tmem_slot = (uint32_t*)(sm + GramSmem::misc);
    volatile int* abort_flag = (volatile int*)(sm + GramSmem::misc + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < kNS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const unsigned long long npairs = min(*npairs_ptr, pair_cap);

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmap) : "memory");
            uint32_t it = 0;
            uint32_t last_phase[kNS];
            bool issued[kNS];
            for (int s = 0; s < kNS; ++s) { issued[s] = false; last_phase[s] = 0; }
            bool ok = true;
            for (unsigned long long w = blockIdx.x; ok && w < npairs; w += gridDim.x) {
                const int2 tp = pairs[w];
                for (int kc = 0; kc < kchunks; ++kc, ++it) {
                    const int s = it % kNS;
                    const uint32_t ph = (it / kNS) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag, fault, 1)) { ok = false; break; }
                    uint8_t* st = sm + GramSmem::stages + s * kStageBytes;
                    mbar_expect_tx(&full[s], kStageBytes);
                    tma_load_2d(st, &tmap, &full[s], kc * kChunkK, tp.x * kTile);
                    tma_load_2d(st + kChunkBytes, &tmap, &full[s], kc * kChunkK, tp.y * kTile);
                    issued[s] = true;
                    last_phase[s] = ph;
                }
            }
            if (!ok) {
                // drain: every stage's most recent copy must land before the CTA exits
                for (int s = 0; s < kNS; ++s) {
                    if (!issued[s]) continue;
                    uint64_t t0 = globaltimer();
                    while (!mbar_try_wait(&full[s], last_phase[s]) && globaltimer() - t0 < kWaitNs) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            uint32_t it = 0, local = 0;
            bool ok = true, any = false;
            for (unsigned long long w = blockIdx.x; ok && w < npairs; w += gridDim.x, ++local) {
                const int b = local & 1;
                const uint32_t tph = (local >> 1) & 1u;
                if (!mbar_wait(&tempty[b], tph ^ 1u, abort_flag, fault, 2)) { ok = false; break; }
                tc_fence_after();
                const uint32_t tacc = tmem_base + (uint32_t)(b * kAccCols);
                for (int kc = 0; kc < kchunks; ++kc, ++it) {
                    const int s = it % kNS;
                    const uint32_t ph = (it / kNS) & 1u;
                    if (!mbar_wait(&full[s], ph, abort_flag, fault, 3)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sm + GramSmem::stages + s * kStageBytes);
                    const uint64_t adesc = sw128_desc(a0), bdesc = sw128_desc(a0 + kChunkBytes);
#pragma unroll
                    for (int k = 0; k < kChunkK / 16; ++k)
                        umma_bf16(tacc, adesc + (uint64_t)(2 * k), bdesc + (uint64_t)(2 * k), kIdesc,
                                  (kc | k) != 0 ? 1u : 0u);
                    umma_commit(&empty[s]);
                    any = true;
                }
                if (!ok) break;
                umma_commit(&tfull[b]);
            }
            if (!ok && any) {
                // wait (bounded) for the MMAs already issued before tensor memory is freed
                umma_commit(drain);
                uint64_t t0 = globaltimer();
                while (!mbar_try_wait(drain, 0) && globaltimer() - t0 < kWaitNs) {
                }
            }
        }
    } else {
        // ---------------- epilogue warps
        const int ew = warp - 2;                       // 0..3
        const int sub = warp & 3;                      // TMEM sub-partition this warp may access
        float4* colinfo = (float4*)(sm + GramSmem::colinfo) + ew * kTile;
        uint32_t local = 0;
        for (unsigned long long w = blockIdx.x; w < npairs; w += gridDim.x, ++local) {
            const int2 tp = pairs[w];
            const int b = local & 1;
            const uint32_t tph = (local >> 1) & 1u;
            // column data of tile J (norm, error radius, Gram error term)
            for (int k = lane; k < kTile; k += 32) colinfo[k] = rowinfo[(int64_t)tp.y * kTile + k];
            const int r = sub * 32 + lane;
            const int64_t gi = (int64_t)tp.x * kTile + r;
            const float4 ri = rowinfo[gi];
            const float Ai = eps_p + ri.y;
            __syncwarp();
            // lane 0 waits (bounded); the others then observe the completed phase
            bool ready = (lane == 0) ? mbar_wait(&tfull[b], tph, abort_flag, fault, 4) : false;
            ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
            if (!ready) break;
            while (!mbar_try_wait(&tfull[b], tph)) {
            }
            tc_fence_after();
            uint32_t masks[kAccCols / 32];
#pragma unroll
            for (int ch = 0; ch < kAccCols / 32; ++ch) {
                float g[32];
                tmem_ld32(tmem_base + ((uint32_t)(sub * 32) << 16) + (uint32_t)(b * kAccCols + ch * 32), g);
                uint32_t m = 0;
#pragma unroll
                for (int t = 0; t < 32; ++t) {
                    const float4 cj = colinfo[ch * 32 + t];
                    const float dd = fmaf(-2.f, g[t], ri.x + cj.x);
                    const float s = Ai + cj.y;
                    const float rhs = fmaf(s, s, ri.z + cj.z) * kappa;
                    m |= (dd <= rhs ? 1u : 0u) << t;
                }
                masks[ch] = m;
            }
            // accumulator fully read: hand it back to the MMA warp
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
            // append candidates (gi < gj inside a diagonal tile; padding rows excluded)
#pragma unroll
            for (int ch = 0; ch < kAccCols / 32; ++ch) {
                uint32_t m = masks[ch];
                const int64_t j0 = (int64_t)tp.y * kTile + ch * 32;
                if (gi >= n) m = 0;
                if (j0 + 32 > n) {
                    int64_t lim = n - j0;
                    m &= lim <= 0 ? 0u : (lim >= 32 ? 0xffffffffu : ((1u << lim) - 1u));
                }
                if (tp.x == tp.y) {
                    // keep columns j with j0 + t > gi
                    int64_t first = gi - j0 + 1;
                    m &= first <= 0 ? 0xffffffffu : (first >= 32 ? 0u : ~((1u << first) - 1u));
                }
                const int cnt = __popc(m);
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (total == 0) continue;
                unsigned long long base = 0;
                if (lane == 31) base = atomicAdd(cand_count, (unsigned long long)total);
                base = __shfl_sync(0xffffffffu, base, 31);
                unsigned long long pos = base + (unsigned long long)(incl - cnt);
                while (m) {
                    const int t = __ffs(m) - 1;
                    m &= m - 1;
                    if (pos < cand_cap) cand[pos] = make_uint2((uint32_t)gi, (uint32_t)(j0 + t));
                    ++pos;
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem_base, kTmemCols);
    }
}

// ------------------------------------------------------------------------------------------------
// exact recheck of the candidates with the reference's sequential FP32 L2

__global__ void __launch_bounds__(256) k_recheck(const float* __restrict__ Xs, int d, const uint2* __restrict__ cand,
                                                 const unsigned long long* __restrict__ ncand_ptr,
                                                 unsigned long long cand_cap, float radius, uint32_t* __restrict__ eu,
                                                 uint32_t* __restrict__ ev, float* __restrict__ ew,
                                                 unsigned long long* __restrict__ ecount, unsigned long long cap)
{
    __shared__ int s_warp[8];
    __shared__ unsigned long long s_base;
    const unsigned long long nc = min(*ncand_ptr, cand_cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // iterate in block-uniform rounds so that the block-level append stays collective
    for (unsigned long long round = (unsigned long long)blockIdx.x * blockDim.x; round < nc; round += stride) {
        const unsigned long long e = round + threadIdx.x;
        bool hit = false;
        float w = 0.f;
        uint2 c = make_uint2(0, 0);
        if (e < nc) {
            c = cand[e];
            const float* p = Xs + (int64_t)c.y * d;
            const float* q = Xs + (int64_t)c.x * d;
            float acc = 0.f;
            if ((d & 3) == 0) {
                const float4* p4 = reinterpret_cast<const float4*>(p);
                const float4* q4 = reinterpret_cast<const float4*>(q);
                for (int k = 0; k < (d >> 2); ++k) {
                    const float4 a = __ldg(p4 + k), b = __ldg(q4 + k);
                    acc = l2seq_acc(acc, a.x, b.x);
                    acc = l2seq_acc(acc, a.y, b.y);
                    acc = l2seq_acc(acc, a.z, b.z);
                    acc = l2seq_acc(acc, a.w, b.w);
                }
            } else {
                for (int k = 0; k < d; ++k) acc = l2seq_acc(acc, __ldg(p + k), __ldg(q + k));
            }
            w = __fsqrt_rn(acc);
            hit = (w <= radius);
        }
        const unsigned ball = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) s_warp[warp] = __popc(ball);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int k = 0; k < 8; ++k) { int t = s_warp[k]; s_warp[k] = acc; acc += t; }
            s_base = acc ? atomicAdd(ecount, (unsigned long long)acc) : 0ull;
        }
        __syncthreads();
        if (hit) {
            const unsigned long long pos = s_base + s_warp[warp] + __popc(ball & ((1u << lane) - 1u));
            if (pos < cap) {
                eu[pos] = c.x;
                ev[pos] = c.y;
                ew[pos] = w;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// BF16 operand preparation

// Per-dimension column sums (double) of the real rows.
__global__ void k_colsum(const float* __restrict__ Xs, int64_t n, int d, double* __restrict__ sums)
{
    for (int k0 = 0; k0 < d; k0 += blockDim.x) {
        const int k = k0 + threadIdx.x;
        if (k >= d) continue;
        double acc = 0.0;
        for (int64_t r = blockIdx.x; r < n; r += gridDim.x) acc += (double)Xs[r * d + k];
        atomicAdd(&sums[k], acc);
    }
}

__global__ void k_shift(const double* __restrict__ sums, int64_t n, int d, float* __restrict__ shift)
{
    for (int k = threadIdx.x; k < d; k += blockDim.x) shift[k] = (float)rint(sums[k] / (double)(n > 0 ? n : 1));
}

// One warp per sorted row: BF16 operand row (dp columns, zero padded) and the
// row's {norm, error radius, Gram error term} for the candidate test.
__global__ void k_to_bf16(const float* __restrict__ Xs, int64_t n, int64_t n_pad, int d, int dp,
                          const float* __restrict__ shift, float gamma, __nv_bfloat16* __restrict__ Xb,
                          float4* __restrict__ rowinfo)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float u = 5.9604644775390625e-08f;  // 2^-24
    for (int64_t r = warp; r < n_pad; r += nwarps) {
        float nrm = 0.f, res = 0.f, xc = 0.f;
        for (int k = lane; k < dp; k += 32) {
            float b = 0.f;
            if (r < n && k < d) {
                const float t = __fsub_rn(Xs[r * d + k], shift[k]);
                const __nv_bfloat16 h = __float2bfloat16_rn(t);
                b = __bfloat162float(h);
                const float e = __fsub_rn(t, b);  // exact: b is t rounded to 8 bits
                nrm = fmaf(b, b, nrm);
                res = fmaf(e, e, res);
                xc = fmaf(t, t, xc);
            }
            Xb[r * dp + k] = __float2bfloat16_rn(b);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
            res += __shfl_xor_sync(0xffffffffu, res, o);
            xc += __shfl_xor_sync(0xffffffffu, xc, o);
        }
        if (lane == 0) {
            const float grow = 1.f + (float)(d + 8) * u;
            // a >= ||(x - c) - x~||: computed residual plus the FP32 rounding of x - c
            const float a = (sqrtf(res) + u * sqrtf(xc)) * grow * grow + 1e-30f;
            // q >= Gram error share of this row: gamma * ||x~||^2 (upper bound on the norm)
            const float q = gamma * nrm * grow;
            rowinfo[r] = make_float4(nrm, a, q, 0.f);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// host side

namespace {

PFN_cuTensorMapEncodeTiled_v12000 get_encode()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        RNNG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        RNNG_REQUIRE(q == cudaDriverEntryPointSuccess && p, RNNG_ERR_CUDA, "cuTensorMapEncodeTiled not available");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

}  // namespace

bool bf16_supported(int d) { return d >= 1 && d <= 1024; }

void prepare_bf16(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    const int d = L.d;
    const int dp = (int)ceil_div(d, kChunkK) * kChunkK;
    c->xb_sorted.reserve(sizeof(__nv_bfloat16) * (size_t)L.n_pad * dp);
    c->norms.reserve(sizeof(float4) * (size_t)L.n_pad + sizeof(double) * d + sizeof(float) * d + 64);
    float4* rowinfo = c->norms.as<float4>();
    double* sums = (double*)(rowinfo + L.n_pad);
    float* shift = (float*)(sums + d);
    RNNG_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * d, s));
    k_colsum<<<std::min<int64_t>(std::max<int64_t>(L.n / 256, 1), (int64_t)c->num_sms * 4), 128, 0, s>>>(L.Xs, L.n,
                                                                                                           d, sums);
    k_shift<<<1, 256, 0, s>>>(sums, L.n, d, shift);
    const double u = std::ldexp(1.0, -24);
    // tensor-core accumulation is modelled as at most 2^-19 relative error per
    // addition (truncating adds with fewer than 24 bits), far below its real error
    const double gamma = (double)dp * std::ldexp(1.0, -19) + (double)(d + 2) * u + 8.0 * u;
    k_to_bf16<<<std::min<int64_t>(ceil_div(L.n_pad * 32, 256), (int64_t)c->num_sms * 16), 256, 0, s>>>(
        L.Xs, L.n, L.n_pad, d, dp, shift, (float)gamma, c->xb_sorted.as<__nv_bfloat16>(), rowinfo);
    RNNG_CUDA(cudaGetLastError());

    static_assert(sizeof(CUtensorMap) == sizeof(c->tmap), "tensor map storage");
    c->bf16_dp = dp;
    c->bf16_rowinfo = rowinfo;
    double ep = (double)L.radius * (1.0 + (double)(d + 8) * u) + 1e-30;
    c->bf16_eps_p = std::nextafter((float)ep, INFINITY);

    CUtensorMap& tm = *reinterpret_cast<CUtensorMap*>(c->tmap);
    cuuint64_t gdim[2] = {(cuuint64_t)dp, (cuuint64_t)L.n_pad};
    cuuint64_t gstride[1] = {(cuuint64_t)dp * 2};
    cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)kTile};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = get_encode()(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->xb_sorted.ptr, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    RNNG_REQUIRE(r == CUDA_SUCCESS, RNNG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

void run_tiles_bf16(rnng_ctx* c, Layout& L, EdgeOut& E)
{
    cudaStream_t s = c->stream;
    const int kchunks = c->bf16_dp / kChunkK;
    const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(c->tmap);
    unsigned long long* cnt = c->counters.as<unsigned long long>() + 5;
    unsigned long long ccap = std::max<unsigned long long>(1u << 20, c->cand_cap_hint);
    const size_t smem = GramSmem::total + 1024;
    static bool attr_set = false;
    if (!attr_set) {
        RNNG_CUDA(cudaFuncSetAttribute(k_gram_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    const int grid = (int)std::max<unsigned long long>(
        1, std::min<unsigned long long>(L.tile_pairs, (unsigned long long)c->num_sms));
    const float kappa = 1.f + 1.0f / (1 << 18);
    for (int attempt = 0;; ++attempt) {
        c->cand.reserve(sizeof(uint2) * ccap);
        RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        k_gram_bf16<<<grid, kGramThreads, smem, s>>>(tm, L.pairs, L.d_tile_pairs, L.tile_pairs, kchunks,
                                                      (const float4*)c->bf16_rowinfo, L.n, c->bf16_eps_p, kappa,
                                                      c->cand.as<uint2>(), cnt, ccap, c->fault_word);
        RNNG_CUDA(cudaGetLastError());
        unsigned long long got = 0;
        RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        int fw = 0;
        RNNG_CUDA(cudaMemcpy(&fw, c->fault_word, sizeof(int), cudaMemcpyDeviceToHost));
        RNNG_REQUIRE(fw == FAULT_NONE, RNNG_ERR_DEVICE, "Gram kernel: bounded wait ran out (fault word set)");
        c->last_candidates = (int64_t)got;
        if (got <= ccap) {
            c->cand_cap_hint = std::max<unsigned long long>(c->cand_cap_hint, got + got / 8);
            break;
        }
        RNNG_REQUIRE(attempt < 2, RNNG_ERR_OVERFLOW, "candidate buffer overflow after regrowth");
        ccap = got + got / 8 + 1024;
        c->stats.retries++;
    }
    const unsigned long long ncand = (unsigned long long)c->last_candidates;
    const int rgrid = (int)std::max<unsigned long long>(
        1, std::min<unsigned long long>((ncand + 255) / 256, (unsigned long long)c->num_sms * 8));
    k_recheck<<<rgrid, 256, 0, s>>>(L.Xs, L.d, c->cand.as<uint2>(), cnt, ccap, L.radius, E.si, E.sj, E.w, E.count,
                                    E.cap);
    RNNG_CUDA(cudaGetLastError());
}

}  // namespace rnng
