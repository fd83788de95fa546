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
// Kernel roles (one CTA per SM, persistent; an item is a row tile with up to two column
// tiles; the CTAs pull chunks of consecutive items from a device-side work queue, an
// atomic head in global memory, so uneven work evens out across the SMs):
//   warp 0      TMA producer: takes the next chunk from the queue and posts its first
//               item into a small ring in shared memory for the other roles; loads the
//               A tile (rows of I, all K-chunks of 64 BF16 = one 128 B swizzle span each)
//               into a resident buffer when I changes, and the B tiles (rows of J, all
//               K-chunks) into a ring of item slots
//   warp 1      MMA issuer: (M=128, N=128 per column tile, K=16) MMAs into one of the
//               accumulators of 512 TMEM columns, one commit per item
//   warps 2-17  epilogue, two groups of 8 (one column tile each): 2 warps per TMEM
//               sub-partition, each reads its 32 x 64 slice of the accumulator in the
//               16x256b fragment layout (4 rows x 16 columns per thread), tests it and
//               stages its candidates in shared memory; a full stage is written out
//               after one atomic reservation in the global candidate list
// Every mbarrier wait is bounded (about one second of wall time); on timeout the
// CTA records a fault code in the context's fault word, stops issuing work, waits
// (bounded) for its own copies and MMAs in flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <dlfcn.h>

#include <cmath>
#include <cstdlib>
#include <string>

#include "common.cuh"
#include "eps_l2.cuh"
#include "kernels_misc.cuh"

namespace rnng {

constexpr int kChunkK = 64;                         // BF16 elements per K-chunk (one 128 B swizzle span)
constexpr int kChunkBytes = kTile * kChunkK * 2;    // 16 KB per operand tile per chunk
constexpr int kMaxDp = 256;                         // padded dimension limit of the BF16 path
constexpr int kMaxSlots = 8;
constexpr int kChunkRing = 4;                       // queue chunks posted ahead to the consumers
constexpr int kAccCols = 128;                       // fp32 accumulator columns (N)
constexpr int kAccBufs = 4;                         // accumulators in tensor memory
constexpr int kTmemCols = kAccBufs * kAccCols;      // all 512 columns
constexpr int kEpiGroups = 2;                       // epilogue groups, taking alternate items
constexpr int kGroupWarps = 8;                      // per group: 2 per TMEM sub-partition
constexpr int kEpiWarps = kEpiGroups * kGroupWarps;
constexpr int kGramThreads = 64 + 32 * kEpiWarps;   // 576
// 18 warps put five on two SM sub-partitions (16K registers each): at most 96 per thread.
// __maxnreg__ rather than __launch_bounds__: at the same 96 the latter's allocation spills.
constexpr int kGramMaxRegs = 96;
constexpr int kEpiCols = kAccCols / (kGroupWarps / 4);  // accumulator columns per epilogue warp (64)
constexpr int kColuFloats = 80;                     // per epilogue warp: its 64 u_j in 4 padded rows of 20
// Candidates staged per epilogue warp before one atomic reserves their place in the global
// list: a reservation with its return on every 16 x 64 slice that had a candidate put
// the global counter's round trip on the epilogue's critical path (a third of the kernel's
// time at 1M x 128, two fifths at 5M x 32).
constexpr int kStage = 128;
constexpr uint64_t kWaitNs = 1000000000ull;         // bounded wait: 1 s
constexpr uint32_t kSmemLimit = 232448;             // opt-in dynamic shared memory per block (227 KB)

// Offsets inside the dynamic shared block (aligned to 1024 bytes in the kernel): the
// small parts first, then the resident A tile (kch chunks) and as many B item slots of
// nt tiles x kch chunks as the rest of the 227 KB holds.  Operand tiles start on
// 1024-byte boundaries (128-byte swizzle atoms).
struct GramSmem {
    uint32_t colinfo, stage, bars, misc, cq, a_tile, b_ring, slot_bytes, total;
    int nslots;
    // a_full/empty, b_full/empty, tfull/tempty, drain, chunk ring full/empty, drill
    static constexpr int nbars = 2 + 2 * kMaxSlots + 2 * kAccBufs + 1 + 2 * kChunkRing + 1;
    // max_slots > 0 caps the B ring (a tuning knob); the ring always holds at least 2 slots
    __host__ __device__ static GramSmem make(int kch, int nt, int max_slots = 0)
    {
        GramSmem g;
        g.colinfo = 0;                                     // kEpiWarps x kColuFloats floats (u_j)
        g.stage = g.colinfo + kEpiWarps * kColuFloats * 4;  // kEpiWarps x kStage staged candidates
        g.bars = g.stage + kEpiWarps * kStage * 8;          // mbarriers
        g.misc = g.bars + nbars * 8;                       // tmem slot, abort flag
        g.cq = g.misc + 16;                                // kChunkRing posted chunk starts (int64)
        g.a_tile = (g.cq + 8 * kChunkRing + 1023) & ~1023u;
        // nt = 3 (row pairs): two resident A tiles, one B tile per item
        g.slot_bytes = (uint32_t)(kch * (nt == 3 ? 1 : nt)) * kChunkBytes;
        g.b_ring = g.a_tile + (uint32_t)(kch * (nt == 3 ? 2 : 1)) * kChunkBytes;
        const uint32_t room = kSmemLimit - 1024 - g.b_ring;  // 1024: alignment slack of the block base
        g.nslots = (int)(room / g.slot_bytes);
        if (g.nslots > kMaxSlots) g.nslots = kMaxSlots;
        if (max_slots >= 2 && g.nslots > max_slots) g.nslots = max_slots;
        g.total = g.b_ring + (uint32_t)g.nslots * g.slot_bytes;
        return g;
    }
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

// Inline fast path (one try_wait), then the bounded wait.
__device__ __forceinline__ bool mbar_wait_fast(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* fault,
                                               int where)
{
    if (mbar_try_wait(bar, parity)) return true;
    return mbar_wait(bar, parity, abort_flag, fault, where);
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

// The same MMA on 8-bit operands (kind::f8f6f4; the 0/1 filter operands, E4M3 both).
__device__ __forceinline__ void umma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// tcgen05.ld.16x256b.x8 without the wait: 16 TMEM lanes x 64 columns.  Thread t gets,
// for each 8-column block m (0..7), v[4m + 0, 1] = (lane t/4, columns 8m + 2(t%4) + 0, 1)
// and v[4m + 2, 3] = (lane t/4 + 8, the same columns): the m16n8 accumulator fragment.
__device__ __forceinline__ void tmem_ld16x256b_x8(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.16x256b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%"
        "19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// tcgen05.ld.red.32x32b.x32 (sm_103a) and its wait, in one statement so that no use of the
// registers can be scheduled before the load lands: thread t gets TMEM lane (lane field
// of taddr) + t, the 32 columns from taddr's column on, and their maximum.
__device__ __forceinline__ float tmem_ld_max_32x32b_x32(uint32_t taddr, float* v)
{
    float m;
    asm volatile(
        "tcgen05.ld.red.sync.aligned.32x32b.x32.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, %32, [%33];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]),
          "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]),
          "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31]), "=f"(m)
        : "r"(taddr)
        : "memory");
    return m;
}

// 8-byte shared-memory store and load at a shared-window address.
__device__ __forceinline__ void st_shared_u2(uint32_t addr, uint32_t a, uint32_t b)
{
    asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ uint2 st_shared_ld_u2(uint32_t addr)
{
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(addr) : "memory");
    return v;
}

// Three-input maximum (exact, like fmaxf(fmaxf(a, b), c)).
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Three-input minimum (exact, like fminf(fminf(a, b), c)).
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
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

// Instruction descriptor for kind::f16: D f32, A and B bf16, both K-major, M = 128,
// N = 128 nt (nt column tiles per MMA).
__host__ __device__ constexpr uint32_t gram_idesc(int nt)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)((kAccCols * nt) >> 3) << 17) |
           ((uint32_t)(kTile >> 4) << 24);
}

// Instruction descriptor for kind::f8f6f4: D f32, A and B E4M3 (format 0), both K-major,
// M = 128, N = 128 nt.
__host__ __device__ constexpr uint32_t gram_idesc_f8(int nt)
{
    return (1u << 4) | ((uint32_t)((kAccCols * nt) >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
}

// Four-deep register prefetch of the item list, so that the dependent global load of
// the next item is issued several items ahead of its use.
// (Item indices are below 2^31: the schedule checks the tile-pair count.)
struct ItemPrefetch {
    int4 q0, q1, q2, q3;
    const int4* __restrict__ p;
    uint32_t end;
    uint32_t stride;
    __device__ __forceinline__ int4 ld(uint32_t w) const { return w < end ? p[w] : make_int4(-1, -1, -1, -1); }
    __device__ __forceinline__ void init(const int4* __restrict__ items, uint32_t w, uint32_t e, uint32_t step = 1)
    {
        p = items;
        end = e;
        stride = step;
        q0 = ld(w);
        q1 = ld(w + step);
        q2 = ld(w + 2 * step);
        q3 = ld(w + 3 * step);
    }
    // returns item w (the next item of this sequence) and prefetches item w + 4 * stride
    __device__ __forceinline__ int4 next(uint32_t w)
    {
        const int4 r = q0;
        q0 = q1;
        q1 = q2;
        q2 = q3;
        q3 = ld(w + 4u * stride);
        return r;
    }
};

// The epilogue's form of the prefetch: each item as the unit of this warp's group,
// (row tile, column tile; -1: none).  nt = 1, 2: row x, column y (group 0) or z (group 1
// of nt = 2), mapped when the item is taken.  nt = 3: row x (group 0) or z (group 1),
// column y when the group's bit of w is set, mapped when the item is loaded (eight
// registers for the four items ahead).
template <int NT>
struct UnitPrefetch {
    ItemPrefetch f;
    int half;
    __device__ __forceinline__ void init(const int4* __restrict__ items, uint32_t w, uint32_t e, uint32_t step,
                                         int h)
    {
        half = h;
        f.init(items, w, e, step);
    }
    __device__ __forceinline__ int2 next(uint32_t w)
    {
        const int4 it = f.next(w);
        return make_int2(it.x, half ? it.z : it.y);
    }
};

template <>
struct UnitPrefetch<3> {
    int2 q0, q1, q2, q3;
    const int4* __restrict__ p;
    uint32_t end;
    uint32_t stride;
    int half;
    __device__ __forceinline__ int2 ld(uint32_t w) const
    {
        if (w >= end) return make_int2(-1, -1);
        const int4 it = p[w];
        return make_int2(half ? it.z : it.x, ((it.w >> half) & 1) ? it.y : -1);
    }
    __device__ __forceinline__ void init(const int4* __restrict__ items, uint32_t w, uint32_t e, uint32_t step,
                                         int h)
    {
        p = items;
        end = e;
        stride = step;
        half = h;
        q0 = ld(w);
        q1 = ld(w + step);
        q2 = ld(w + 2 * step);
        q3 = ld(w + 3 * step);
    }
    __device__ __forceinline__ int2 next(uint32_t w)
    {
        const int2 r = q0;
        q0 = q1;
        q1 = q2;
        q2 = q3;
        q3 = ld(w + 4u * stride);
        return r;
    }
};

// Next chunk posted by the producer for a consumer at ring position (cs, cph): its first
// item, or -1 when the queue is empty.  Returns false when the wait ran out or the CTA
// aborts.  Every consumer (the MMA thread, each epilogue warp's lane 0) takes every chunk.
__device__ __forceinline__ bool take_chunk(uint64_t* cq_full, uint64_t* cq_empty, volatile long long* cqv, int& cs,
                                           uint32_t& cph, long long& start, volatile int* abort_flag, int* fault,
                                           int where)
{
    if (!mbar_wait_fast(&cq_full[cs], cph, abort_flag, fault, where)) return false;
    start = cqv[cs];
    mbar_arrive(&cq_empty[cs]);
    if (++cs == kChunkRing) {
        cs = 0;
        cph ^= 1u;
    }
    return true;
}

// ------------------------------------------------------------------------------------------------
// the Gram kernel
//
// An item is one row tile i with NT column tiles {j0, j1} of the tile-pair list (j1 = -1
// when the row had no second pair): the B slot holds the NT tiles stacked, one
// 128 x (128 NT) x 16 MMA per K step computes both tile pairs against the resident A
// tile, and the accumulator (128 NT TMEM columns; 512 / (128 NT) of them in flight)
// is read by both epilogue groups, one column tile each (NT = 2), or by the two groups
// on alternate items (NT = 1).  CTA g takes its range of the scheduled item list: the
// chunks g, g + G, ... of the items sorted by (row tile, column tile), so the A tile
// stays resident while its row lasts and all CTAs work on neighbouring rows at the
// same time (B tiles are shared through L2).

// Row pairs (NT = 3): an item is the row tiles {2 r, 2 r + 1} (x, z; z = -1 past the last
// tile) against one column tile y, w bit h set when tile pair (2 r + h, y) survived.  Both
// A tiles stay resident while the pair lasts, so one B tile feeds two 128 x 128 MMA chains
// (accumulator halves h), and the B operand bytes per tile pair halve.
//
// KCH K-chunks of 64 dimensions (dp = 64 KCH); NT column tiles per item (3: row pairs); FOLD: the column
// tiles come from tmapB with the column terms folded into their padding (k_to_bf16), so
// the accumulator already holds g - u_j / 2 and the test needs no u_j
// F8: 8-bit operands (E4M3; 128 per 128-byte chunk row, K = 32 per MMA), same byte layout.
// RAW: the diagnostic form of rnng_gram_probe_bf16, which also writes the raw accumulators.
template <int KCH, int NT, bool FOLD, bool F8, bool RAW = false>
__global__ void __maxnreg__(kGramMaxRegs)
    k_gram_bf16(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap tmapB,
                const int4* __restrict__ items, unsigned long long nitems,
                const float4* __restrict__ rowinfo, const float* __restrict__ ucol,
                const float2* __restrict__ tileinfo, int64_t n, float eps_p, float kappa, uint2* __restrict__ cand,
                unsigned long long* __restrict__ cand_count, unsigned long long cand_cap,
                unsigned long long* __restrict__ qhead, int chunk, int max_slots, int* __restrict__ fault,
                float* __restrict__ raw, int64_t raw_ld, int drill)
{
    constexpr bool PR = NT == 3;              // row pairs
    constexpr int NB = PR ? 1 : NT;           // B tiles per item
    constexpr int NH = PR ? 2 : NT;           // accumulator halves per item (epilogue groups on it)
    constexpr int kAcc = kTmemCols / (kAccCols * NH);  // accumulators in flight
    constexpr uint32_t kIdesc = F8 ? gram_idesc_f8(NB) : gram_idesc(NB);
    constexpr int kChunkElems = F8 ? 2 * kChunkK : kChunkK;  // elements per 128-byte chunk row
    extern __shared__ __align__(1024) uint8_t gsm_raw[];
    uint8_t* sm = (uint8_t*)(((uintptr_t)gsm_raw + 1023) & ~(uintptr_t)1023);
    const GramSmem SL = GramSmem::make(KCH, NT, max_slots);
    uint64_t* bars = (uint64_t*)(sm + SL.bars);
    uint64_t* a_full = bars;
    uint64_t* a_empty = bars + 1;
    uint64_t* b_full = bars + 2;
    uint64_t* b_empty = bars + 2 + kMaxSlots;
    uint64_t* tfull = bars + 2 + 2 * kMaxSlots;
    uint64_t* tempty = tfull + kAccBufs;
    uint64_t* drain = tempty + kAccBufs;
    uint64_t* cq_full = drain + 1;             // chunk ring: posted by the producer
    uint64_t* cq_empty = cq_full + kChunkRing; // read by the MMA thread and every epilogue warp
    volatile long long* cqv = (volatile long long*)(sm + SL.cq);  // chunk's first item, -1: queue empty
    uint64_t* drill_bar = cq_empty + kChunkRing;  // nothing ever arrives on it (rnng_ctx_fault_drill)
    // ring slots: one item (all K-chunks of its NT B tiles) per slot
    const int nslots = SL.nslots;
    const uint32_t slot_bytes = SL.slot_bytes;
    constexpr uint32_t kTileBytes = (uint32_t)KCH * kChunkBytes;  // one operand tile, all chunks
    uint32_t* tmem_slot = (uint32_t*)(sm + SL.misc);
    volatile int* abort_flag = (volatile int*)(sm + SL.misc + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    if (threadIdx.x == 32) {
        mbar_init(a_full, 1);
        mbar_init(a_empty, 1);
        for (int s = 0; s < kMaxSlots; ++s) {
            mbar_init(&b_full[s], 1);
            mbar_init(&b_empty[s], 1);
        }
        for (int b = 0; b < kAccBufs; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kGroupWarps * NH);
        }
        mbar_init(drain, 1);
        for (int k = 0; k < kChunkRing; ++k) {
            mbar_init(&cq_full[k], 1);
            mbar_init(&cq_empty[k], 1 + kEpiWarps);
        }
        mbar_init(drill_bar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const unsigned long long uchunk = (unsigned long long)chunk;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmap) : "memory");
            if (FOLD) asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmapB) : "memory");
            const CUtensorMap* bmap = FOLD ? &tmapB : &tmap;
            uint32_t aloads = 0;
            int cur_i = -1;
            uint32_t issued = 0, last_phase = 0;  // per ring slot: loads issued, phase of the last
            bool ok = true;
            ItemPrefetch pf, pfn;  // pfn: the first items of the next chunk, loaded ahead
            int q = 0;
            uint32_t ph = 0;
            int cs = 0;
            uint32_t cph = 0;
            // posts a chunk (its first item, or -1 when the queue is empty) to the consumers
            auto post = [&](long long v) -> bool {
                if (!mbar_wait_fast(&cq_empty[cs], cph ^ 1u, abort_flag, fault, 7)) return false;
                cqv[cs] = v;
                mbar_arrive(&cq_full[cs]);
                if (++cs == kChunkRing) {
                    cs = 0;
                    cph ^= 1u;
                }
                return true;
            };
            unsigned long long c0 = atomicAdd(qhead, 1ull) * uchunk;  // this CTA's first chunk
            bool more = c0 < nitems;
            ok = post(more ? (long long)c0 : -1ll);
            bool ahead = false;  // pfn holds the current chunk's items
            while (ok && more) {
                const unsigned long long cend = min(nitems, c0 + uchunk);
                // the next chunk's ticket, in flight while this chunk's loads are issued
                const unsigned long long tk_next = atomicAdd(qhead, 1ull);
                unsigned long long n0 = 0;
                if (ahead) pf = pfn;
                else pf.init(items, c0, cend);
                ahead = false;
                for (unsigned long long w = c0; w < cend; ++w) {
                    // four items before the end, the next chunk's first items are requested
                    if (!ahead && w + 4 >= cend) {
                        n0 = tk_next * uchunk;
                        if (n0 < nitems) {
                            pfn.init(items, n0, min(nitems, n0 + uchunk));
                            ahead = true;
                        }
                    }
                    const int4 it = pf.next(w);
                    if (it.x != cur_i) {
                        if (aloads > 0 && !mbar_wait_fast(a_empty, (aloads - 1) & 1u, abort_flag, fault, 1)) { ok = false; break; }
                        const bool a2 = PR && it.z >= 0;  // the pair's second row tile
                        mbar_expect_tx(a_full, a2 ? 2 * kTileBytes : kTileBytes);
#pragma unroll
                        for (int kc = 0; kc < KCH; ++kc)
                            tma_load_2d(sm + SL.a_tile + kc * kChunkBytes, &tmap, a_full, kc * kChunkElems, it.x * kTile);
                        if (a2)
#pragma unroll
                            for (int kc = 0; kc < KCH; ++kc)
                                tma_load_2d(sm + SL.a_tile + (KCH + kc) * kChunkBytes, &tmap, a_full, kc * kChunkElems,
                                            it.z * kTile);
                        ++aloads;
                        cur_i = it.x;
                    }
                    if (!mbar_wait_fast(&b_empty[q], ph ^ 1u, abort_flag, fault, 2)) { ok = false; break; }
                    const bool second = NT == 2 && it.z >= 0;
                    mbar_expect_tx(&b_full[q], second ? 2 * kTileBytes : kTileBytes);
                    uint8_t* slot = sm + SL.b_ring + q * slot_bytes;
                    // chunk kc of tile t at slot + (kc NB + t) 16 KB: per chunk the NB tiles are
                    // stacked rows of one 128 NB-row operand
#pragma unroll
                    for (int kc = 0; kc < KCH; ++kc) {
                        tma_load_2d(slot + (kc * NB) * kChunkBytes, bmap, &b_full[q], kc * kChunkElems, it.y * kTile);
                        if (second)
                            tma_load_2d(slot + (kc * NB + 1) * kChunkBytes, bmap, &b_full[q], kc * kChunkElems,
                                        it.z * kTile);
                    }
                    issued |= 1u << q;
                    last_phase = (last_phase & ~(1u << q)) | (ph << q);
                    if (++q == nslots) {
                        q = 0;
                        ph ^= 1u;
                    }
                }
                if (!ok) break;
                c0 = tk_next * uchunk;
                more = c0 < nitems;
                ok = post(more ? (long long)c0 : -1ll);
            }
            if (!ok) {
                // drain: the copies in flight must land before the CTA exits
                uint64_t t0 = globaltimer();
                if (aloads > 0)
                    while (!mbar_try_wait(a_full, (aloads - 1) & 1u) && globaltimer() - t0 < kWaitNs) {
                    }
                for (int qq = 0; qq < kMaxSlots; ++qq) {
                    if (!((issued >> qq) & 1u)) continue;
                    t0 = globaltimer();
                    while (!mbar_try_wait(&b_full[qq], (last_phase >> qq) & 1u) && globaltimer() - t0 < kWaitNs) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            // One thread issues every MMA, so the loop keeps its scalar work minimal: slot,
            // accumulator and phases advance incrementally, descriptors step by constants,
            // and the K loop is unrolled at compile time.
            uint32_t aidx = 0, ph = 0, tph = 0;
            int q = 0, b = 0;
            int cur_i = -1;
            bool ok = true, any = false;
            const uint64_t adesc0 = sw128_desc(smem_u32(sm + SL.a_tile));
            const uint64_t bdesc_ring = sw128_desc(smem_u32(sm + SL.b_ring));
            const uint64_t slot_step = (uint64_t)(slot_bytes >> 4);  // descriptor address units
            uint64_t bdesc_q = bdesc_ring;
            ItemPrefetch pf;
            int cs = 0;
            uint32_t cph = 0;
            long long st = -1;
            ok = take_chunk(cq_full, cq_empty, cqv, cs, cph, st, abort_flag, fault, 8);
            while (ok && st >= 0) {
            const unsigned long long c0 = (unsigned long long)st, cend = min(nitems, c0 + uchunk);
            long long nst = -1;  // the next chunk, taken at this chunk's last item
            pf.init(items, c0, cend);
            for (unsigned long long w = c0; w < cend; ++w) {
                const int4 it = pf.next(w);
                if (it.x != cur_i) {
                    if (!mbar_wait_fast(a_full, aidx & 1u, abort_flag, fault, 3)) { ok = false; break; }
                    ++aidx;
                    cur_i = it.x;
                    tc_fence_after();
                }
                if (!mbar_wait_fast(&tempty[b], tph ^ 1u, abort_flag, fault, 4)) { ok = false; break; }
                if (!mbar_wait_fast(&b_full[q], ph, abort_flag, fault, 5)) { ok = false; break; }
                tc_fence_after();
                const uint32_t tacc = tmem_base + (uint32_t)(b * kAccCols * NH);
                if constexpr (PR) {
                    // one chain per surviving tile pair of the row pair, A tile h into half h
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (!((it.w >> h) & 1)) continue;
#pragma unroll
                        for (int kc = 0; kc < KCH; ++kc)
#pragma unroll
                            for (int k = 0; k < kChunkK / 16; ++k)
                                umma_bf16(tacc + (uint32_t)(h * kAccCols),
                                          adesc0 + (uint64_t)((h * KCH + kc) * (kChunkBytes >> 4) + 2 * k),
                                          bdesc_q + (uint64_t)(kc * (kChunkBytes >> 4) + 2 * k), kIdesc,
                                          (kc | k) != 0 ? 1u : 0u);
                    }
                } else {
#pragma unroll
                for (int kc = 0; kc < KCH; ++kc)
#pragma unroll
                    for (int k = 0; k < kChunkK / 16; ++k)
                        if constexpr (F8)
                            umma_f8(tacc, adesc0 + (uint64_t)(kc * (kChunkBytes >> 4) + 2 * k),
                                      bdesc_q + (uint64_t)(kc * NT * (kChunkBytes >> 4) + 2 * k), kIdesc,
                                      (kc | k) != 0 ? 1u : 0u);
                        else
                            umma_bf16(tacc, adesc0 + (uint64_t)(kc * (kChunkBytes >> 4) + 2 * k),
                                      bdesc_q + (uint64_t)(kc * NT * (kChunkBytes >> 4) + 2 * k), kIdesc,
                                      (kc | k) != 0 ? 1u : 0u);
                }
                any = true;
                umma_commit(&b_empty[q]);
                umma_commit(&tfull[b]);
                // release the A tile after its last item's MMAs; the next item is pf.q0 inside the
                // chunk, else the first item of the next chunk (-1 at the end of the queue)
                int next_row;
                if (w + 1 < cend) {
                    next_row = pf.q0.x;
                } else {
                    if (!take_chunk(cq_full, cq_empty, cqv, cs, cph, nst, abort_flag, fault, 9)) {
                        ok = false;
                        nst = -1;
                    }
                    next_row = nst >= 0 ? items[nst].x : -1;
                }
                if (next_row != cur_i) umma_commit(a_empty);
                if (++q == nslots) {
                    q = 0;
                    ph ^= 1u;
                    bdesc_q = bdesc_ring;
                } else {
                    bdesc_q += slot_step;
                }
                if (++b == kAcc) {
                    b = 0;
                    tph ^= 1u;
                }
            }
            st = nst;
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
        // Candidate test per element: -2 g + u_j <= W_i, where u_j = n_j - a_j^2 - q_j
        // and W_i = A_i^2 + q_i - n_i + 2 A_i amax_J (+ rounding slack), A_i = eps' + a_i.
        // Replacing a_j by the column tile's max a only widens the test, so it still
        // admits every pair with (eps' + a_i + a_j)^2 + q_i + q_j >= D~.
        //
        // Units: NT = 2: every item, this group's column tile (half = group);
        //        NT = 3: every item, this group's row tile of the pair (half = group);
        //        NT = 1: the items of this group (grp, grp + 2, ...), their only tile.
        const int ew = warp - 2;
        const int grp = ew / kGroupWarps;
        const int sub = warp & 3;                      // TMEM sub-partition this warp may access
        const int cg = (ew % kGroupWarps) >> 2;        // column group: columns [kEpiCols cg, +kEpiCols)
        const int half = NH == 2 ? grp : 0;
        const unsigned ustride = NH == 2 ? 1u : (unsigned)kEpiGroups;
        const uint32_t goff = NH == 2 ? 0u : (uint32_t)grp;  // first unit in a chunk
        float* colu = (float*)(sm + SL.colinfo) + ew * kColuFloats;
        // this warp's stage: shared-memory address recomputed where used (a register less)
        const uint32_t stage_base = smem_u32(sm + SL.stage) + (uint32_t)(ew * kStage * 8);
        uint32_t fill = 0;  // candidates in this warp's stage (warp-uniform)
        // writes the stage to the global list after one reservation (the count grows past
        // the capacity, so that the caller learns the total and regrows the list)
        auto flush = [&]() {
            __syncwarp();
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(cand_count, (unsigned long long)fill);
            base = __shfl_sync(0xffffffffu, base, 0);
            for (uint32_t k = (uint32_t)lane; k < fill; k += 32)
                if (base + k < cand_cap) cand[base + k] = st_shared_ld_u2(stage_base + 8 * k);
            __syncwarp();
            fill = 0;
        };
        const int r = sub * 32 + lane;
        // Fragment layout (tcgen05.ld.16x256b): thread (rq, q4) = (lane / 4, lane % 4) holds
        // rows rq + 8 k (k = 0..3) of this sub-partition and columns 8 m + 2 q4 + e
        // (m = 0..7, e = 0..1) of the warp's 64: 16 column terms u_j per thread and item
        // (with a 32x32b load every thread would need all 64).
        const int rq = lane >> 2, q4 = lane & 3;
        const int n32 = (int)n;
        int cs = 0;
        uint32_t cph = 0;
        bool alive = true;
        // The queue's chunks as this warp sees them: (c0, cend) the current chunk, base the
        // CTA-sequence index of its item c0.  take_next() moves to the next chunk in which
        // this warp has a unit and returns false at the end of the queue (or when the wait
        // ran out); it runs one unit ahead, while the current unit waits for its accumulator.
        const uint32_t nit = (uint32_t)nitems, uch = (uint32_t)chunk;
        uint32_t c0 = 0, cend = 0;
        uint32_t base = 0;
        auto take_next = [&]() -> bool {
            for (;;) {
                long long st = -1;
                bool got = true;
                if (lane == 0) got = take_chunk(cq_full, cq_empty, cqv, cs, cph, st, abort_flag, fault, 10);
                got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
                st = __shfl_sync(0xffffffffu, st, 0);
                if (!got) alive = false;
                if (!got || st < 0) return false;
                base += cend - c0;
                c0 = (uint32_t)st;
                cend = min(nit, c0 + uch);
                if (c0 + (uint32_t)goff < cend) return true;  // chunks other than the last have even sizes
            }
        };
        // row / column data of the current unit, loaded one unit ahead; of an item only its
        // row tile and this group's column tile are kept (it_i, it_j)
        int it_i = -1, it_j = -1;
        float2 uc = make_float2(0.f, 0.f);
        float4 ri = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 tj = make_float2(0.f, 0.f);
        uint32_t w = 0;
        uint32_t local = 0;  // item index in the CTA's sequence
        UnitPrefetch<NT> pf;
        if (drill) {
            // failure drill: wait on a barrier that nothing arrives on; the bounded wait runs
            // out, records the fault and raises the abort flag, and the whole CTA winds down
            const bool ok_ = lane == 0 ? mbar_wait(drill_bar, 0, abort_flag, fault, 11) : false;
            alive = __shfl_sync(0xffffffffu, ok_ ? 1 : 0, 0) != 0;
        }
        bool have = alive && take_next();
        if (have) {
            w = c0 + goff;
            local = base + (uint32_t)goff;
            pf.init(items, w, cend, ustride, half);
            const int2 it = pf.next(w);
            it_i = it.x;
            it_j = it.y;
            if (it_j >= 0) {
                if (!FOLD) uc = reinterpret_cast<const float2*>(ucol)[((int64_t)it_j * kTile + cg * kEpiCols) / 2 + lane];
                ri = rowinfo[(int64_t)it_i * kTile + r];
                tj = tileinfo[it_j];
            }
        }
        while (have) {
            const int b = (int)(local % (uint32_t)kAcc);
            const uint32_t tph = (local / (uint32_t)kAcc) & 1u;
            const int jt = it_j;  // this unit's column tile (-1: none)
            // (indices fit int: n < 2^31 - 128 is checked at the boundary)
            const int rb = it_i * kTile + sub * 32 + rq;          // row of k = 0
            const int cb = jt * kTile + cg * kEpiCols + 2 * q4;   // column of m = e = 0, chunk 0
            const bool diag = it_i == jt;
            // staged for the fragment threads: column 8 m + 2 q + e at float 20 q + 2 m + e, so that
            // thread (., q) reads its 16 terms as four 16-byte loads, the four q rows in distinct banks
            if (!FOLD) reinterpret_cast<float2*>(colu)[(lane & 3) * 10 + (lane >> 2)] = uc;
            float Wk[4];
            float Wi;  // the threshold of row r (this lane's row of the sub-partition)
            {
                const float A = eps_p + ri.y;
                const float AA = A * A, cross = 2.f * A * tj.x;
                Wi = (AA + ri.z - ri.x + cross) + kappa * (ri.x + tj.y + AA + ri.z + cross);
                if (!FOLD)
#pragma unroll
                    for (int k = 0; k < 4; ++k) Wk[k] = __shfl_sync(0xffffffffu, Wi, rq + 8 * k);
            }
            // the next unit (in this chunk, or the first of the next one) and its loads, issued
            // now: they complete while this unit is tested
            uint32_t wn = w + ustride;
            uint32_t ln = local + ustride;
            bool nhave = true;
            {
                int2 itn;
                if (wn < cend) {
                    itn = pf.next(wn);
                } else {
                    nhave = take_next();
                    if (nhave) {
                        wn = c0 + goff;
                        ln = base + (uint32_t)goff;
                        pf.init(items, wn, cend, ustride, half);
                        itn = pf.next(wn);
                    }
                }
                it_i = nhave ? itn.x : -1;
                it_j = nhave ? itn.y : -1;
                if (nhave && it_j >= 0) {
                    if (!FOLD) uc = reinterpret_cast<const float2*>(ucol)[((int64_t)it_j * kTile + cg * kEpiCols) / 2 + lane];
                    ri = rowinfo[(int64_t)it_i * kTile + r];
                    tj = tileinfo[it_j];
                }
            }
            __syncwarp();
            // fast path: the accumulator is usually ready; otherwise lane 0 waits (bounded)
            if (!__all_sync(0xffffffffu, mbar_try_wait(&tfull[b], tph))) {
                bool ready = (lane == 0) ? mbar_wait(&tfull[b], tph, abort_flag, fault, 6) : false;
                ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
                if (!ready) {
                    alive = false;
                    break;
                }
                while (!mbar_try_wait(&tfull[b], tph)) {
                }
            }
            tc_fence_after();
            if (jt < 0) {
                // no second tile in this item: nothing to test, hand the accumulator back
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[b]);
            } else {
            const uint32_t taddr = tmem_base + ((uint32_t)(sub * 32) << 16) +
                                   (uint32_t)(b * kAccCols * NH + half * kAccCols + cg * kEpiCols);
            // this thread's column terms: u2[m] = u_j of columns 8 m + 2 q4 + {0, 1}
            float2 u2[8];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float4 v = FOLD ? make_float4(0.f, 0.f, 0.f, 0.f) : reinterpret_cast<const float4*>(colu + 20 * q4)[t];
                u2[2 * t] = make_float2(v.x, v.y);
                u2[2 * t + 1] = make_float2(v.z, v.w);
            }
            for (int hh = 0; hh < 2; ++hh) {
                uint32_t msk = 0;
                // candidate x of this thread is (r0, c0 + x) in the FOLD layout, else
                // (r0 + 8 ((x >> 1) & 1), c0 + 8 (x >> 2) + (x & 1))
                int r0, c0;
                if constexpr (FOLD) {
                    // 32x32b layout: this thread's row is lane r of the sub-partition, the load
                    // brings columns 32 hh .. 32 hh + 31 of the warp's 64 and their maximum
                    // (tcgen05.ld.red).  The accumulator holds g - u_j / 2, so the term
                    // -2 g + u_j is -2 g (exact) and the row's smallest term is -2 max g.
                    float g[32];
                    const float gmax = tmem_ld_max_32x32b_x32(taddr + 32u * (uint32_t)hh, g);
                    if (hh == 1) {
                        // accumulator slice read: hand it back to the MMA warp
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&tempty[b]);
                    }
                    const bool mine = -2.f * gmax <= Wi;
                    if (!__any_sync(0xffffffffu, mine)) continue;
                    r0 = rb - rq + lane;
                    c0 = cb - 2 * q4 + 32 * hh;
                    if (mine) {
                        if (!diag && r0 < n32 && c0 + 31 < n32) {
#pragma unroll
                            for (int x = 0; x < 32; ++x) msk |= (-2.f * g[x] <= Wi ? 1u : 0u) << x;
                        } else {
#pragma unroll
                            for (int x = 0; x < 32; ++x) {
                                const int gj = c0 + x;
                                // padding rows / columns and, inside a diagonal tile, j <= i excluded
                                const bool ok = -2.f * g[x] <= Wi && r0 < n32 && gj < n32 && (!diag || gj > r0);
                                msk |= (ok ? 1u : 0u) << x;
                            }
                        }
                    }
                } else {
                // lanes 16 hh .. 16 hh + 15 of the sub-partition, all 64 columns:
                // g[4 m + 2 hi + e] = row rq + 8 hi + 16 hh, column 8 m + 2 q4 + e
                float g[32];
                tmem_ld16x256b_x8(taddr + ((uint32_t)(16 * hh) << 16), g);
                tmem_ld_wait();
                if constexpr (RAW) {
                    // diagnostic output (rnng_gram_probe_bf16): the accumulator as the tensor cores left it
#pragma unroll
                    for (int x = 0; x < 32; ++x)
                        raw[(int64_t)(rb + 16 * hh + 8 * ((x >> 1) & 1)) * raw_ld + cb + 8 * (x >> 2) + (x & 1)] = g[x];
                }
                if (hh == 1) {
                    // accumulator slice read: hand it back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[b]);
                }
                // most rows have no candidate: test each row's minimum term first.  Packed
                // pairs: __ffma2_rn forms two terms -2 g + u_j, each rounded once as fmaf; a
                // three-input minimum takes both into one of the row's running minima
                float mk[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) mk[q] = INFINITY;
                const float2 k2 = make_float2(-2.f, -2.f);
#pragma unroll
                for (int m = 0; m < 8; ++m)
#pragma unroll
                    for (int hi = 0; hi < 2; ++hi) {
                        const int x = 4 * m + 2 * hi;
                        const float2 p = __ffma2_rn(make_float2(g[x], g[x + 1]), k2, u2[m]);
                        g[x] = p.x;  // g now holds the terms
                        g[x + 1] = p.y;
                        mk[2 * hi + (m & 1)] = min3f(mk[2 * hi + (m & 1)], p.x, p.y);
                    }
                const float W0 = Wk[2 * hh], W1 = Wk[2 * hh + 1];
                const bool mine = fminf(mk[0], mk[1]) <= W0 || fminf(mk[2], mk[3]) <= W1;
                if (!__any_sync(0xffffffffu, mine)) continue;
                r0 = rb + 16 * hh;
                c0 = cb;
                if (mine) {
                    // all 2 rows x 16 columns real and off the diagonal tile: the test alone
                    if (!diag && r0 + 8 < n32 && cb + 57 < n32) {
#pragma unroll
                        for (int x = 0; x < 32; ++x) msk |= (g[x] <= ((x & 2) ? W1 : W0) ? 1u : 0u) << x;
                    } else {
#pragma unroll
                        for (int x = 0; x < 32; ++x) {
                            const int gi = r0 + 8 * ((x >> 1) & 1);
                            const int gj = cb + 8 * (x >> 2) + (x & 1);
                            // padding rows / columns and, inside a diagonal tile, j <= i excluded
                            const bool ok = g[x] <= ((x & 2) ? W1 : W0) && gi < n32 && gj < n32 && (!diag || gj > gi);
                            msk |= (ok ? 1u : 0u) << x;
                        }
                    }
                }
                }
                const auto cand_i = [&](int x) -> uint32_t {
                    return FOLD ? (uint32_t)r0 : (uint32_t)(r0 + 8 * ((x >> 1) & 1));
                };
                const auto cand_j = [&](int x) -> uint32_t {
                    return FOLD ? (uint32_t)(c0 + x) : (uint32_t)(c0 + 8 * (x >> 2) + (x & 1));
                };
                const int cnt = __popc(msk);
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (total > 0) {
                    if (fill + (uint32_t)total > (uint32_t)kStage && fill > 0) flush();
                    if (total > kStage) {
                        // more than a stage in one slice: reserved and written directly
                        unsigned long long base = 0;
                        if (lane == 31) base = atomicAdd(cand_count, (unsigned long long)total);
                        base = __shfl_sync(0xffffffffu, base, 31);
                        unsigned long long pos = base + (unsigned long long)(incl - cnt);
                        while (msk) {
                            const int x = __ffs(msk) - 1;
                            msk &= msk - 1;
                            if (pos < cand_cap) cand[pos] = make_uint2(cand_i(x), cand_j(x));
                            ++pos;
                        }
                    } else {
                        uint32_t sa = stage_base + 8 * (fill + (uint32_t)(incl - cnt));
                        while (msk) {
                            const int x = __ffs(msk) - 1;
                            msk &= msk - 1;
                            st_shared_u2(sa, cand_i(x), cand_j(x));
                            sa += 8;
                        }
                        fill += (uint32_t)total;
                    }
                }
            }
            }
            __syncwarp();
            w = wn;
            local = ln;
            have = nhave;
        }
        if (fill > 0) flush();  // also after an abort: the staged candidates are complete
        (void)alive;
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

// Exact recheck, any d: one candidate per thread reading its two rows directly (short
// rows are a few cache lines each).
__global__ void __launch_bounds__(256) k_recheck_direct(const float* __restrict__ Xs, int d, const uint2* __restrict__ cand,
                                                 const unsigned long long* __restrict__ ncand_ptr,
                                                 unsigned long long cand_cap, float radius, const EdgeSink sink,
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
            if (pos < cap) sink.put(pos, c.x, c.y, w);
        }
        __syncthreads();
    }
}

// Exact recheck for d a multiple of 32 (k_recheck_direct otherwise).
// One candidate per thread, summed in RNNG's order (dimension 0, 1, ...).  A warp's 32
// candidates read their two rows through shared memory, 32 dimensions at a time: the
// warp loads the 32 rows' slices together (coalesced, many loads in flight) and stores
// them transposed, slice[k][j] with rows padded to 33 floats, so that the per-thread
// reads (fixed k, j = lane) hit 32 distinct banks.
constexpr int kRecheckWarps = 4;

__global__ void __launch_bounds__(32 * kRecheckWarps) k_recheck(const float* __restrict__ Xs, int d,
                                                                const uint2* __restrict__ cand,
                                                                const unsigned long long* __restrict__ ncand_ptr,
                                                                unsigned long long cand_cap, float radius,
                                                                const EdgeSink sink,
                                                                unsigned long long* __restrict__ ecount,
                                                                unsigned long long cap)
{
    __shared__ float slice[kRecheckWarps][2][32][33];
    __shared__ int64_t rowp[kRecheckWarps][2][32];
    __shared__ int s_warp[kRecheckWarps];
    __shared__ unsigned long long s_base;
    const unsigned long long nc = min(*ncand_ptr, cand_cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float(*sp)[33] = slice[warp][0];
    float(*sq)[33] = slice[warp][1];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // iterate in block-uniform rounds so that the block-level append stays collective
    for (unsigned long long round = (unsigned long long)blockIdx.x * blockDim.x; round < nc; round += stride) {
        const unsigned long long e = round + threadIdx.x;
        const bool valid = e < nc;
        const uint2 c = valid ? cand[e] : make_uint2(0, 0);
        rowp[warp][0][lane] = valid ? (int64_t)c.y * d : -1;
        rowp[warp][1][lane] = valid ? (int64_t)c.x * d : -1;
        float acc = 0.f;
        for (int k0 = 0; k0 < d; k0 += 32) {
            __syncwarp();
            {
                // 16-byte loads: lane l takes dimensions k0 + 4 (l % 8) .. + 3 of rows j0 + l / 8;
                // all 16 loads are independent, and (4 (l % 8) + i) * 33 + j0 + l / 8 keeps the
                // transposed stores in distinct banks
                const int kq = 4 * (lane & 7), jr = lane >> 3;
                float4 vp[8], vq[8];
#pragma unroll
                for (int j0 = 0; j0 < 8; ++j0) {
                    const int64_t pr = rowp[warp][0][4 * j0 + jr], qr = rowp[warp][1][4 * j0 + jr];
                    vp[j0] = pr >= 0 ? __ldg(reinterpret_cast<const float4*>(Xs + pr + k0 + kq)) : make_float4(0.f, 0.f, 0.f, 0.f);
                    vq[j0] = pr >= 0 ? __ldg(reinterpret_cast<const float4*>(Xs + qr + k0 + kq)) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int j0 = 0; j0 < 8; ++j0) {
                    const int j = 4 * j0 + jr;
                    sp[kq + 0][j] = vp[j0].x; sp[kq + 1][j] = vp[j0].y; sp[kq + 2][j] = vp[j0].z; sp[kq + 3][j] = vp[j0].w;
                    sq[kq + 0][j] = vq[j0].x; sq[kq + 1][j] = vq[j0].y; sq[kq + 2][j] = vq[j0].z; sq[kq + 3][j] = vq[j0].w;
                }
            }
            __syncwarp();
            if (valid)
#pragma unroll 8
                for (int k = 0; k < 32; ++k) acc = l2seq_acc(acc, sp[k][lane], sq[k][lane]);
        }
        float w = 0.f;
        bool hit = false;
        if (valid) {
            w = __fsqrt_rn(acc);
            hit = (w <= radius);
        }
        const unsigned ball = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) s_warp[warp] = __popc(ball);
        __syncthreads();
        if (threadIdx.x == 0) {
            int a = 0;
            for (int k = 0; k < kRecheckWarps; ++k) { const int t = s_warp[k]; s_warp[k] = a; a += t; }
            s_base = a ? atomicAdd(ecount, (unsigned long long)a) : 0ull;
        }
        __syncthreads();
        if (hit) {
            const unsigned long long pos = s_base + s_warp[warp] + __popc(ball & ((1u << lane) - 1u));
            if (pos < cap) sink.put(pos, c.x, c.y, w);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// BF16 operand preparation

// Per-dimension column sums (double) of the real rows, d <= 256: a block step covers
// 256 / d whole rows as one contiguous run of floats, so thread t always adds dimension
// t % d; per-thread float partials, then one double atomic per dimension and block.
// screen (optional, zeroed by the caller): screen[0] = 1 if a value is NaN or infinite,
// screen[1] = the float bits of the largest |value| (NaNs aside).
__global__ void __launch_bounds__(256) k_colsum(const float* __restrict__ Xs, int64_t n, int d, double* __restrict__ sums,
                                                unsigned long long* __restrict__ screen)
{
    __shared__ float part[256];
    const int rpb = 256 / d;  // rows per step
    const int t = threadIdx.x;
    const bool active = t < rpb * d;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    float acc = 0.f, mx = 0.f;
    bool bad = false;
    if (active)
        for (int64_t r = r0 + t / d; r < r1; r += rpb) {
            const float v = Xs[r * d + t % d];
            bad |= nonfinite_f32(v);
            mx = fmaxf(mx, fabsf(v));
            acc += v;
        }
    part[t] = acc;
    if (screen) {
        // non-negative floats order as their bit patterns
        const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
        if ((t & 31) == 0 && m) atomicMax(&screen[1], (unsigned long long)m);
    }
    if (__syncthreads_or(bad) && screen && t == 0) screen[0] = 1ull;
    if (t < d) {
        double s2 = 0.0;
        for (int q = 0; q < rpb; ++q) s2 += (double)part[q * d + t];
        if (r0 < r1) atomicAdd(&sums[t], s2);
    }
}

// The same sums for d a multiple of 4: each thread adds four consecutive dimensions from
// 16-byte loads, four rows per round in flight (the scalar form left HBM latency exposed:
// 3 TB/s at 1M x 128).
__global__ void __launch_bounds__(256) k_colsum4(const float* __restrict__ Xs, int64_t n, int d,
                                                 double* __restrict__ sums, unsigned long long* __restrict__ screen)
{
    __shared__ float4 part[256];
    const int nq = d >> 2;      // float4 per row (d <= 256: at most 64)
    const int rps = 256 / nq;   // rows per step
    const int t = threadIdx.x;
    const bool active = t < rps * nq;
    const int q = t % nq;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float mx = 0.f;
    bool bad = false;
    auto add = [&](const float4 v) {
        bad |= nonfinite_f32(v.x) | nonfinite_f32(v.y) | nonfinite_f32(v.z) | nonfinite_f32(v.w);
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
        acc.w += v.w;
    };
    if (active) {
        const float4* X4 = reinterpret_cast<const float4*>(Xs);
        int64_t r = r0 + t / nq;
        for (; r + 3 * rps < r1; r += 4 * rps) {
            const float4 a = __ldg(X4 + r * nq + q), b = __ldg(X4 + (r + rps) * nq + q);
            const float4 c = __ldg(X4 + (r + 2 * rps) * nq + q), e = __ldg(X4 + (r + 3 * rps) * nq + q);
            add(a);
            add(b);
            add(c);
            add(e);
        }
        for (; r < r1; r += rps) add(__ldg(X4 + r * nq + q));
    }
    part[t] = acc;
    if (screen) {
        // non-negative floats order as their bit patterns
        const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
        if ((t & 31) == 0 && m) atomicMax(&screen[1], (unsigned long long)m);
    }
    if (__syncthreads_or(bad) && screen && t == 0) screen[0] = 1ull;
    if (t < nq && r0 < r1) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int k = 0; k < rps; ++k) {
            const float4 p = part[k * nq + t];
            s0 += (double)p.x;
            s1 += (double)p.y;
            s2 += (double)p.z;
            s3 += (double)p.w;
        }
        atomicAdd(&sums[4 * t], s0);
        atomicAdd(&sums[4 * t + 1], s1);
        atomicAdd(&sums[4 * t + 2], s2);
        atomicAdd(&sums[4 * t + 3], s3);
    }
}

// Rounded column means.  A non-finite column sum (a NaN or infinite coordinate, or a
// float partial that overflowed) gets shift 0: any finite shift keeps the BF16 error
// bounds valid.
__global__ void k_shift(const double* __restrict__ sums, int64_t n, int d, float* __restrict__ shift)
{
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        const double s = sums[k];
        const bool fin = (__double_as_longlong(s) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll;
        shift[k] = fin ? (float)rint(s / (double)(n > 0 ? n : 1)) : 0.f;
    }
}

// One warp: the BF16 row of x (d floats; zeros when !real) shifted by `shift` and zero
// padded to dp, written to out, and the row's {norm of the BF16 row, error radius a,
// Gram error term q} in every lane.  a >= ||(x - shift) - bf16 row|| (the BF16 residual
// plus the FP32 rounding of x - shift); q = gamma ||x~||^2, an upper bound on this
// row's share of the FP32 error of a tensor-core Gram entry.
__device__ __forceinline__ float3 bf16_row(const float* __restrict__ x, bool real, int d, int dp,
                                           const float* __restrict__ shift, float gamma,
                                           __nv_bfloat16* __restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const float u = 5.9604644775390625e-08f;  // 2^-24
    float nrm = 0.f, res = 0.f, xc = 0.f;
    for (int k = lane; k < dp; k += 32) {
        float b = 0.f;
        if (real && k < d) {
            const float t = __fsub_rn(x[k], shift[k]);
            const __nv_bfloat16 h = __float2bfloat16_rn(t);
            b = __bfloat162float(h);
            const float e = __fsub_rn(t, b);  // exact: b is t rounded to 8 bits
            nrm = fmaf(b, b, nrm);
            res = fmaf(e, e, res);
            xc = fmaf(t, t, xc);
        }
        out[k] = __float2bfloat16_rn(b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        res += __shfl_xor_sync(0xffffffffu, res, o);
        xc += __shfl_xor_sync(0xffffffffu, xc, o);
    }
    const float grow = 1.f + (float)(d + 8) * u;
    const float a = (sqrtf(res) + u * sqrtf(xc)) * grow * grow + 1e-30f;
    const float q = gamma * nrm * grow;
    return make_float3(nrm, a, q);
}

// bf16_row for d a multiple of 4 and x on a 16-byte boundary: lane l takes columns 4 l ..
// 4 l + 3 (then 4 l + 128 ..), one 16-byte load and one 8-byte store each; outB, when
// given, receives the same row (zeros past d).  Same terms as bf16_row, summed in another
// order (the bounds hold for any order of the FP32 sums).
__device__ __forceinline__ float3 bf16_row4(const float* __restrict__ x, bool real, int d, int dp,
                                            const float* __restrict__ shift, float gamma,
                                            __nv_bfloat16* __restrict__ out, __nv_bfloat16* __restrict__ outB)
{
    const int lane = threadIdx.x & 31;
    const float u = 5.9604644775390625e-08f;  // 2^-24
    float nrm = 0.f, res = 0.f, xc = 0.f;
    for (int k = 4 * lane; k < dp; k += 128) {
        float b[4] = {0.f, 0.f, 0.f, 0.f};
        if (real && k < d) {
            const float4 xv = *reinterpret_cast<const float4*>(x + k);
            const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float t = __fsub_rn(xs[j], shift[k + j]);
                b[j] = __bfloat162float(__float2bfloat16_rn(t));
                const float e = __fsub_rn(t, b[j]);  // exact: b is t rounded to 8 bits
                nrm = fmaf(b[j], b[j], nrm);
                res = fmaf(e, e, res);
                xc = fmaf(t, t, xc);
            }
        }
        const __nv_bfloat162 lo = __floats2bfloat162_rn(b[0], b[1]), hi = __floats2bfloat162_rn(b[2], b[3]);
        uint2 pk;
        pk.x = *reinterpret_cast<const uint32_t*>(&lo);
        pk.y = *reinterpret_cast<const uint32_t*>(&hi);
        *reinterpret_cast<uint2*>(out + k) = pk;
        if (outB) *reinterpret_cast<uint2*>(outB + k) = pk;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        res += __shfl_xor_sync(0xffffffffu, res, o);
        xc += __shfl_xor_sync(0xffffffffu, xc, o);
    }
    const float grow = 1.f + (float)(d + 8) * u;
    const float a = (sqrtf(res) + u * sqrtf(xc)) * grow * grow + 1e-30f;
    const float q = gamma * nrm * grow;
    return make_float3(nrm, a, q);
}

// One warp per sorted row: BF16 operand row (dp columns, zero padded) and the
// row's {norm, error radius, Gram error term, norm - a^2 - q} for the candidate test.
// With fold (dp >= d + 4) the row is written twice: as a row-tile operand (Xb) with
// 1 in columns d .. d + 3, and as a column-tile operand (XbB) with -v there, v = u/2
// split exactly into four BF16 terms, u = n - a^2 - q - 2 gamma (n + a^2 + q).  A
// tensor-core Gram entry of the two is then g - u_j / 2 directly: the folded column
// term rides in the accumulation, whose error bound grows by gamma |u|, which the
// extra 2 gamma (n + a^2 + q) in u absorbs, so the candidate test -2 g' <= W_i keeps
// exactly the guarantee of -2 g + u_j <= W_i.
__global__ void k_to_bf16(const float* __restrict__ Xs, int64_t n, int64_t n_pad, int d, int dp,
                          const float* __restrict__ shift, float gamma, __nv_bfloat16* __restrict__ Xb,
                          float4* __restrict__ rowinfo, bool fold, __nv_bfloat16* __restrict__ XbB)
{
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const bool vec = (d & 3) == 0;  // rows on 16-byte boundaries
    for (int64_t r = warp; r < n_pad; r += nwarps) {
        float3 v;
        if (vec) {
            // the row-tile and (fold) column-tile operands together; columns d .. d + 3 below
            v = bf16_row4(Xs + r * d, r < n, d, dp, shift, gamma, Xb + r * dp, fold ? XbB + r * dp : nullptr);
        } else {
            v = bf16_row(Xs + r * d, r < n, d, dp, shift, gamma, Xb + r * dp);
            if (fold) {
                // the same row as a column-tile operand (padding written below)
                for (int k = lane; k < d; k += 32) XbB[r * dp + k] = Xb[r * dp + k];
                for (int k = d + 4 + lane; k < dp; k += 32) XbB[r * dp + k] = __float2bfloat16_rn(0.f);
            }
        }
        __syncwarp();  // the zeros other lanes wrote to columns d .. d + 3 come first
        if (lane == 0) {
            rowinfo[r] = make_float4(v.x, v.y, v.z, v.x - v.y * v.y - v.z);
            if (fold) {
                const float big = v.x + v.y * v.y + v.z;
                float rest = 0.5f * (v.x - v.y * v.y - v.z - 2.f * gamma * big);
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const __nv_bfloat16 h = __float2bfloat16_rn(rest);
                    rest = __fsub_rn(rest, __bfloat162float(h));  // exact
                    Xb[r * dp + d + t] = __float2bfloat16_rn(1.f);
                    XbB[r * dp + d + t] = __hneg(h);
                }
            }
        }
    }
}

// One warp per ball: BF16 centre row and {norm, a, q, radius} (radius -1: no ball; its
// row is zero).  Rows nb .. nb_pad - 1 are padding (no ball).  widen[0] accumulates, over
// the balls, how much a and q widen a ball pair's squared threshold relative to
// E = eps' + 2 r (the ball paired with itself), widen[1] the number of balls.
__global__ void k_balls_bf16(const float* __restrict__ cen, const float* __restrict__ rad, int64_t nb, int64_t nb_pad,
                             int d, int dp, const float* __restrict__ shift, float gamma, float eps_p,
                             __nv_bfloat16* __restrict__ out, float4* __restrict__ info, float* __restrict__ widen)
{
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float wsum = 0.f, wcnt = 0.f;
    for (int64_t b = warp; b < nb_pad; b += nwarps) {
        const float r = b < nb ? rad[b] : -1.f;
        const float3 v = bf16_row(cen + b * d, r >= 0.f, d, dp, shift, gamma, out + b * dp);
        if ((threadIdx.x & 31) == 0) {
            info[b] = make_float4(v.x, v.y, v.z, r >= 0.f ? r : -1.f);
            if (r >= 0.f) {
                const float E = eps_p + 2.f * r, Ew = E + 2.f * v.y;
                wsum += (Ew * Ew + 2.f * v.z) / fmaxf(E * E, 1e-30f) - 1.f;
                wcnt += 1.f;
            }
        }
    }
    if ((threadIdx.x & 31) == 0 && wcnt > 0.f) {
        atomicAdd(&widen[0], wsum);
        atomicAdd(&widen[1], wcnt);
    }
}

// Per tile: max error radius a and max of (n + a^2 + q) over its rows, plus the
// column array u = n - a^2 - q used by the candidate test.
__global__ void k_tile_info(const float4* __restrict__ rowinfo, int64_t T, float* __restrict__ ucol,
                            float2* __restrict__ tileinfo)
{
    const int64_t t = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ float s_a[4], s_n[4];
    const float4 ri = rowinfo[t * kTile + threadIdx.x];
    ucol[t * kTile + threadIdx.x] = ri.w;
    float amax = ri.y, nmax = ri.x + ri.y * ri.y + ri.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        nmax = fmaxf(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
    }
    if (lane == 0) { s_a[warp] = amax; s_n[warp] = nmax; }
    __syncthreads();
    if (threadIdx.x == 0) {
        const float grow = 1.0f + 1.0f / (1 << 20);
        tileinfo[t] = make_float2(fmaxf(fmaxf(s_a[0], s_a[1]), fmaxf(s_a[2], s_a[3])) * grow,
                                  fmaxf(fmaxf(s_n[0], s_n[1]), fmaxf(s_n[2], s_n[3])) * grow);
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

bool bf16_supported(int d) { return d >= 1 && d <= kMaxDp; }

double bf16_gamma(int d)
{
    // tensor-core accumulation is modelled as at most 2^-19 relative error per
    // addition (truncating adds with fewer than 24 bits), far below its real error
    const int dp = (int)ceil_div(d, kChunkK) * kChunkK;
    return (double)dp * std::ldexp(1.0, -19) + (double)(d + 8) * std::ldexp(1.0, -24) + 2.0 * std::ldexp(1.0, -24);
}

bool bf16_in_range(const Layout& L)
{
    // the centred rows lie within 2 max|x| + 1 (the shift is a rounded column mean): their
    // squared norms, the Gram entries and the test's thresholds stay finite when
    // d (2 max|x| + 1)^2 <= 2^124; a widened radius of at least 2^-40 keeps the underflow of
    // products, norms and error radii (absolute errors of order d 2^-126) far below the
    // test's relative slack kappa (eps_p)^2
    const double m = 2.0 * (double)L.maxabs + 1.0;
    return (double)L.d * m * m <= std::ldexp(1.0, 124) && widened_radius(L.radius, L.d) >= std::ldexp(1.f, -40);
}

const float* bf16_shift(rnng_ctx* c, Layout& L, const float* X, unsigned long long* screen)
{
    if (L.shift) return L.shift;
    if (!X) X = L.Xs;
    cudaStream_t s = c->stream;
    const int d = L.d;
    c->shift_buf.reserve(sizeof(double) * d + sizeof(float) * d + 16);
    double* sums = c->shift_buf.as<double>();
    float* shift = (float*)(sums + d);
    RNNG_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * d, s));
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(L.n, 512), (int64_t)c->num_sms * 4));
    if (screen) RNNG_CUDA(cudaMemsetAsync(screen, 0, 2 * sizeof(unsigned long long), s));
    if ((d & 3) == 0)
        k_colsum4<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(L.n, 512), (int64_t)c->num_sms * 8)), 256,
                    0, s>>>(X, L.n, d, sums, screen);
    else
        k_colsum<<<(unsigned)blocks, 256, 0, s>>>(X, L.n, d, sums, screen);
    ++c->launches;
    k_shift<<<1, 256, 0, s>>>(sums, L.n, d, shift); ++c->launches;
    L.shift = shift;
    return shift;
}

float prepare_ball_bf16(rnng_ctx* c, Layout& L, const float* cen, const float* rad, int64_t nb, int64_t nb_pad,
                        float eps_p, __nv_bfloat16* out, float4* info)
{
    cudaStream_t s = c->stream;
    const int dp = (int)ceil_div(L.d, kChunkK) * kChunkK;
    const float* shift = bf16_shift(c, L);
    float* widen = reinterpret_cast<float*>(c->counters.as<unsigned long long>() + 12);
    RNNG_CUDA(cudaMemsetAsync(widen, 0, 2 * sizeof(float), s));
    k_balls_bf16<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nb_pad * 32, 256), (int64_t)c->num_sms * 16)),
                   256, 0, s>>>(cen, rad, nb, nb_pad, L.d, dp, shift, (float)bf16_gamma(L.d), eps_p, out, info, widen);
    ++c->launches;
    float h[2] = {0.f, 0.f};
    RNNG_CUDA(cudaMemcpyAsync(h, widen, sizeof(h), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    return h[1] > 0.f ? h[0] / h[1] : 0.f;
}

void prepare_bf16(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    const int d = L.d;
    const int dp = (int)ceil_div(d, kChunkK) * kChunkK;
    c->xb_sorted.reserve(sizeof(__nv_bfloat16) * (size_t)L.n_pad * dp);
    c->norms.reserve(sizeof(float4) * (size_t)L.n_pad + sizeof(float) * (size_t)L.n_pad +
                     sizeof(float2) * (size_t)L.T + 64);
    float4* rowinfo = c->norms.as<float4>();
    float* ucol = (float*)(rowinfo + L.n_pad);
    float2* tileinfo = (float2*)(ucol + L.n_pad);
    const float* shift = bf16_shift(c, L);
    // four free padding columns carry the column terms through the tensor cores
    c->bf16_fold = dp - d >= 4;
    if (c->bf16_fold) c->xb_sortedB.reserve(sizeof(__nv_bfloat16) * (size_t)L.n_pad * dp);
    k_to_bf16<<<std::min<int64_t>(ceil_div(L.n_pad * 32, 256), (int64_t)c->num_sms * 16), 256, 0, s>>>(
        L.Xs, L.n, L.n_pad, d, dp, shift, (float)bf16_gamma(d), c->xb_sorted.as<__nv_bfloat16>(), rowinfo,
        c->bf16_fold, c->bf16_fold ? c->xb_sortedB.as<__nv_bfloat16>() : nullptr); ++c->launches;
    k_tile_info<<<(unsigned)L.T, kTile, 0, s>>>(rowinfo, L.T, ucol, tileinfo); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
    c->bf16_ucol = ucol;
    c->bf16_tileinfo = tileinfo;

    static_assert(sizeof(CUtensorMap) == sizeof(c->tmap), "tensor map storage");
    c->bf16_dp = dp;
    c->bf16_rowinfo = rowinfo;
    c->bf16_eps_p = widened_radius(L.radius, d);

    CUtensorMap& tm = *reinterpret_cast<CUtensorMap*>(c->tmap);
    cuuint64_t gdim[2] = {(cuuint64_t)dp, (cuuint64_t)L.n_pad};
    cuuint64_t gstride[1] = {(cuuint64_t)dp * 2};
    cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)kTile};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = get_encode()(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->xb_sorted.ptr, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    RNNG_REQUIRE(r == CUDA_SUCCESS, RNNG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    CUtensorMap& tmb = *reinterpret_cast<CUtensorMap*>(c->tmapB);
    r = get_encode()(&tmb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->bf16_fold ? c->xb_sortedB.ptr : c->xb_sorted.ptr,
                     gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    RNNG_REQUIRE(r == CUDA_SUCCESS, RNNG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

template <int KCH, int NT, bool FOLD, bool F8, bool RAW = false>
static void gram_instance(bool launch, int grid, size_t smem, cudaStream_t s, const CUtensorMap& tm,
                          const CUtensorMap& tmb, const int4* items,
                          unsigned long long nitems, const float4* rowinfo, const float* ucol, const float2* tileinfo,
                          int64_t n, float eps_p, float kappa, uint2* cand, unsigned long long* cnt,
                          unsigned long long ccap, unsigned long long* qhead, int chunk, int max_slots, int* fault,
                          float* raw, int64_t raw_ld, int drill)
{
    if (!launch) {
        RNNG_CUDA(cudaFuncSetAttribute(k_gram_bf16<KCH, NT, FOLD, F8, RAW>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return;
    }
    k_gram_bf16<KCH, NT, FOLD, F8, RAW><<<grid, kGramThreads, smem, s>>>(tm, tmb, items, nitems, rowinfo, ucol, tileinfo, n,
                                                                eps_p, kappa, cand, cnt, ccap, qhead, chunk,
                                                                max_slots, fault, raw, raw_ld, drill);
}

// Sets the shared-memory size (launch = false) or launches the instance for (kch, nt, fold).
template <bool FOLD, class... Args>
static void gram_dispatch_fold(int kch, int nt, Args... args)
{
    if (nt == 2) {
        if (kch == 1) gram_instance<1, 2, FOLD, false>(args...);
        else gram_instance<2, 2, FOLD, false>(args...);
    } else if (nt == 3) {
        if (kch == 1) gram_instance<1, 3, FOLD, false>(args...);
        else gram_instance<2, 3, FOLD, false>(args...);
    } else {
        switch (kch) {
            case 1: gram_instance<1, 1, FOLD, false>(args...); break;
            case 2: gram_instance<2, 1, FOLD, false>(args...); break;
            case 3: gram_instance<3, 1, FOLD, false>(args...); break;
            default: gram_instance<4, 1, FOLD, false>(args...); break;
        }
    }
}

// The diagnostic instances (raw accumulators out; no folded column terms, BF16 operands).
template <class... Args>
static void gram_dispatch_raw(int kch, int nt, Args... args)
{
    if (nt == 2) {
        if (kch == 1) gram_instance<1, 2, false, false, true>(args...);
        else gram_instance<2, 2, false, false, true>(args...);
    } else {
        switch (kch) {
            case 1: gram_instance<1, 1, false, false, true>(args...); break;
            case 2: gram_instance<2, 1, false, false, true>(args...); break;
            case 3: gram_instance<3, 1, false, false, true>(args...); break;
            default: gram_instance<4, 1, false, false, true>(args...); break;
        }
    }
}

template <class... Args>
static void gram_dispatch(bool fold, bool f8, int kch, int nt, Args... args)
{
    if (f8) gram_instance<4, 1, false, true>(args...);  // the 0/1 filter operand: 512 bytes per row
    else if (fold) gram_dispatch_fold<true>(kch, nt, args...);
    else gram_dispatch_fold<false>(kch, nt, args...);
}

GramTune gram_tune(rnng_ctx* c, int kind, int dp, int64_t tile_pairs)
{
    GramTune t;
    t.kind = kind;
    t.dp = dp;
    // two column tiles per item (N = 256 MMAs) while two B slots of them fit next to A
    t.nt = (kind == 0 && dp <= 2 * kChunkK) ? 2 : 1;
    const int nt_table = t.nt;
    t.chunk = 64;
    t.slots = 0;
    const GramTune* best = nullptr;
    for (const GramTune& r : c->gram_table)
        if (r.kind == kind && r.dp == dp && r.min_pairs <= tile_pairs && (!best || r.min_pairs >= best->min_pairs))
            best = &r;
    const GramTune* src[2] = {best, &c->gram_force};
    for (const GramTune* r : src) {
        if (!r) continue;
        if (r->nt > 0) t.nt = r->nt;
        if (r->chunk > 0) t.chunk = r->chunk;
        if (r->slots > 0) t.slots = r->slots;
    }
    // compiled forms: two column tiles (nt = 2) and row pairs (nt = 3) only for BF16
    // operands of at most two K-chunks
    if (t.nt < 1 || t.nt > 3) t.nt = nt_table;
    if (kind != 0 || dp > 2 * kChunkK) t.nt = 1;
    t.chunk = std::max(1, std::min(t.chunk, 1 << 20));
    // with one column tile the two epilogue groups take alternate items of a chunk: even sizes
    if (t.nt == 1) t.chunk = (t.chunk + 1) & ~1;
    if (t.slots == 1) t.slots = 2;
    return t;
}

namespace {

// The integer after "key": in a JSON object's text (nullopt-like: returns false if absent).
bool json_int(const std::string& obj, const char* key, long long* out)
{
    const std::string k = std::string("\"") + key + "\"";
    size_t p = obj.find(k);
    if (p == std::string::npos) return false;
    p = obj.find(':', p + k.size());
    if (p == std::string::npos) return false;
    ++p;
    while (p < obj.size() && (obj[p] == ' ' || obj[p] == '\t' || obj[p] == '\n' || obj[p] == '\r')) ++p;
    char* end = nullptr;
    const long long v = std::strtoll(obj.c_str() + p, &end, 10);
    if (end == obj.c_str() + p) return false;
    *out = v;
    return true;
}

std::string library_dir()
{
    Dl_info info;
    if (dladdr((const void*)&library_dir, &info) && info.dli_fname) {
        std::string f = info.dli_fname;
        const size_t s = f.rfind('/');
        return s == std::string::npos ? std::string(".") : f.substr(0, s);
    }
    return ".";
}

}  // namespace

void load_gram_table(rnng_ctx* c)
{
    c->gram_table.clear();
    const char* env = std::getenv("RNNG_GRAM_TUNING");
    // the library sits in rnng_gb300/_build/, the table in rnng_gb300/
    const std::string path = env && *env ? std::string(env) : library_dir() + "/../gram_tuning.json";
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return;
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    // {"rows": [{"kind": "bf16" | "f8", "dp": .., "min_pairs": .., "nt": .., "chunk": .., "slots": ..}, ...]}
    size_t p = text.find("\"rows\"");
    if (p == std::string::npos) return;
    while ((p = text.find('{', p)) != std::string::npos) {
        const size_t e = text.find('}', p);
        if (e == std::string::npos) break;
        const std::string obj = text.substr(p, e - p + 1);
        p = e + 1;
        long long dp = 0, mp = 0, nt = 0, ch = 0, sl = 0;
        if (!json_int(obj, "dp", &dp)) continue;
        GramTune r;
        r.kind = obj.find("\"f8\"") != std::string::npos ? 1 : 0;
        r.dp = (int)dp;
        if (json_int(obj, "min_pairs", &mp)) r.min_pairs = mp;
        if (json_int(obj, "nt", &nt)) r.nt = (int)nt;
        if (json_int(obj, "chunk", &ch)) r.chunk = (int)ch;
        if (json_int(obj, "slots", &sl)) r.slots = (int)sl;
        c->gram_table.push_back(r);
    }
}

// Candidates of the scheduled items of L by the tensor-core kernel, with the candidate
// buffer regrown (at most twice) until it holds them all; the count is left in *cnt and
// returned.
static unsigned long long gram_candidates(rnng_ctx* c, const Layout& L, const CUtensorMap& tm,
                                          const CUtensorMap& tmb, int kchunks, int nt, bool fold, bool f8,
                                          const float4* rowinfo, const float* ucol, const float2* tileinfo,
                                          float eps_p, unsigned long long* cnt)
{
    cudaStream_t s = c->stream;
    unsigned long long ccap = std::max<unsigned long long>(1u << 20, c->cand_cap_hint);
    const GramSmem layout = GramSmem::make(kchunks, nt, L.gram_slots);
    RNNG_REQUIRE(layout.nslots >= 2, RNNG_ERR_UNSUPPORTED, "BF16 operand tiles too large for shared memory");
    const size_t smem = layout.total + 1024;
    const int chunk = std::max(1, L.gram_chunk);
    unsigned long long* qhead = c->counters.as<unsigned long long>() + kSlotQueue;
    if (L.gram_raw)
        gram_dispatch_raw(kchunks, nt, false, 0, smem, s, tm, tmb, L.items, L.num_items, rowinfo, ucol, tileinfo, L.n,
                          eps_p, 0.f, (uint2*)nullptr, cnt, 0ull, qhead, chunk, L.gram_slots, c->fault_word,
                          (float*)nullptr, (int64_t)0, 0);
    else
        gram_dispatch(fold, f8, kchunks, nt, false, 0, smem, s, tm, tmb, L.items, L.num_items, rowinfo, ucol, tileinfo,
                      L.n, eps_p, 0.f, (uint2*)nullptr, cnt, 0ull, qhead, chunk, L.gram_slots, c->fault_word,
                      (float*)nullptr, (int64_t)0, 0);
    // one CTA per SM, fewer when there are fewer chunks
    const int grid = (int)std::max<unsigned long long>(
        1, std::min<unsigned long long>((L.num_items + chunk - 1) / chunk, (unsigned long long)c->num_sms));
    c->stats.gram_nt = nt;
    c->stats.gram_chunk = chunk;
    c->stats.gram_slots = layout.nslots;
    const float kappa = 1.0f / (1 << 20);  // relative slack for the fp32 evaluation of the test
    unsigned long long got = 0;
    for (int attempt = 0;; ++attempt) {
        c->cand.reserve(sizeof(uint2) * ccap);
        RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        RNNG_CUDA(cudaMemsetAsync(qhead, 0, sizeof(unsigned long long), s));
        RNNG_CUDA(cudaEventRecord(c->ev[9], s));
        if (L.gram_raw)
            gram_dispatch_raw(kchunks, nt, true, grid, smem, s, tm, tmb, L.items, L.num_items, rowinfo, ucol, tileinfo,
                              L.n, eps_p, kappa, c->cand.as<uint2>(), cnt, ccap, qhead, chunk, L.gram_slots,
                              c->fault_word, L.gram_raw, L.n_pad, 0);
        else
            gram_dispatch(fold, f8, kchunks, nt, true, grid, smem, s, tm, tmb, L.items, L.num_items, rowinfo, ucol,
                          tileinfo, L.n, eps_p, kappa, c->cand.as<uint2>(), cnt, ccap, qhead, chunk, L.gram_slots,
                          c->fault_word, (float*)nullptr, (int64_t)0, c->fault_drill ? 1 : 0);
        ++c->launches;
        RNNG_CUDA(cudaGetLastError());
        RNNG_CUDA(cudaEventRecord(c->ev[10], s));
        RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        {
            float gms = 0.f;
            if (cudaEventElapsedTime(&gms, c->ev[9], c->ev[10]) == cudaSuccess) c->gram_ms += gms;
        }
        check_device_fault(c);  // a bounded wait that ran out: RNNG_ERR_DEVICE, the word cleared for the next call
        if (got <= ccap) {
            c->cand_cap_hint = std::max<unsigned long long>(c->cand_cap_hint, got + got / 8);
            break;
        }
        RNNG_REQUIRE(attempt < 2, RNNG_ERR_OVERFLOW, "candidate buffer overflow after regrowth");
        ccap = got + got / 8 + 1024;
        c->stats.retries++;
    }
    return got;
}

unsigned long long run_filter_f8(rnng_ctx* c, const Layout& L, const uint8_t* x8, const float4* rowinfo,
                                 const float* ucol, const float2* tileinfo, float thr_sqrt, unsigned long long* cnt)
{
    CUtensorMap& tm = *reinterpret_cast<CUtensorMap*>(c->tmap);
    cuuint64_t gdim[2] = {(cuuint64_t)kFilterBytes, (cuuint64_t)L.n_pad};
    cuuint64_t gstride[1] = {(cuuint64_t)kFilterBytes};
    cuuint32_t box[2] = {(cuuint32_t)(2 * kChunkK), (cuuint32_t)kTile};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = get_encode()(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)x8, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    RNNG_REQUIRE(r == CUDA_SUCCESS, RNNG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return gram_candidates(c, L, tm, tm, kFilterBytes / (2 * kChunkK), 1, false, true, rowinfo, ucol, tileinfo,
                           thr_sqrt, cnt);
}

void run_tiles_bf16(rnng_ctx* c, Layout& L, EdgeOut& E)
{
    cudaStream_t s = c->stream;
    const int kchunks = c->bf16_dp / kChunkK;
    const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(c->tmap);
    const CUtensorMap& tmb = *reinterpret_cast<const CUtensorMap*>(c->tmapB);
    unsigned long long* cnt = c->counters.as<unsigned long long>() + 5;
    c->last_candidates = (int64_t)gram_candidates(
        c, L, tm, tmb, kchunks, L.item_tiles, c->bf16_fold, false, (const float4*)c->bf16_rowinfo,
        (const float*)c->bf16_ucol, (const float2*)c->bf16_tileinfo, c->bf16_eps_p, cnt);
    const unsigned long long ccap = std::max<unsigned long long>(1u << 20, c->cand_cap_hint);
    RNNG_CUDA(cudaEventRecord(c->ev[8], s));
    const unsigned long long ncand = (unsigned long long)c->last_candidates;
    EdgeSink sink;
    sink.eu = E.si;
    sink.ev = E.sj;
    sink.ew = E.w;
    if (E.direct) {
        // every candidate can be an edge: room for all of them in the pinned staging block,
        // written through its device address
        const unsigned long long cap = std::max<unsigned long long>(ncand, 1);
        char* h = nullptr;
        try {
            h = (char*)host_stage(c, (size_t)cap * (2 * sizeof(int64_t) + sizeof(float)));
        } catch (const Error&) {
            h = nullptr;  // no pinned block that large: the results go the usual way
        }
        void* dptr = nullptr;
        if (h && cudaHostGetDevicePointer(&dptr, h, 0) == cudaSuccess && dptr) {
            E.hu = reinterpret_cast<int64_t*>(h);
            E.hv = E.hu + cap;
            E.hw = reinterpret_cast<float*>(E.hv + cap);
            sink.du = reinterpret_cast<int64_t*>(dptr);
            sink.dv = sink.du + cap;
            sink.dw = reinterpret_cast<float*>(sink.dv + cap);
            sink.perm = E.perm;
            sink.ids = E.ids;
            E.cap = cap;
        } else {
            (void)cudaGetLastError();  // no device address for the staging block: the usual path
            E.direct = false;
        }
    }
    const int rthreads = 32 * kRecheckWarps;
    const int rgrid = (int)std::max<unsigned long long>(
        1, std::min<unsigned long long>((ncand + rthreads - 1) / rthreads, (unsigned long long)c->num_sms * 16));
    if ((L.d & 31) == 0)
        k_recheck<<<rgrid, rthreads, 0, s>>>(L.Xs, L.d, c->cand.as<uint2>(), cnt, ccap, L.radius, sink, E.count, E.cap);
    else
        k_recheck_direct<<<(int)std::max<unsigned long long>(
                               1, std::min<unsigned long long>((ncand + 255) / 256, (unsigned long long)c->num_sms * 8)),
                           256, 0, s>>>(L.Xs, L.d, c->cand.as<uint2>(), cnt, ccap, L.radius, sink, E.count, E.cap);
    ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

}  // namespace rnng

// Diagnostic entry point (include/rnng_gpu.h): one tile pair through the Gram kernel with
// its raw accumulator written out.
extern "C" int rnng_gram_probe_bf16(rnng_ctx* c, const float* X, int64_t d, float* G, float* Xb, float* rowinfo)
{
    using namespace rnng;
    return guarded(c, [&] {
        RNNG_REQUIRE(X && G && Xb && rowinfo, RNNG_ERR_INVALID, "null pointer");
        RNNG_REQUIRE(d >= 64 && d <= kMaxDp && d % kChunkK == 0, RNNG_ERR_INVALID,
                     "the probe takes d = 64, 128, 192 or 256");
        cudaStream_t s = c->stream;
        const int64_t n = 2 * kTile;
        c->x_in.reserve(sizeof(float) * (size_t)n * d);
        RNNG_CUDA(cudaMemcpyAsync(c->x_in.ptr, X, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, s));
        Layout L;
        L.n = n;
        L.n_pad = n;
        L.T = 2;
        L.S = 1;
        L.d = (int)d;
        L.radius = 1.f;
        L.Xs = c->x_in.as<float>();
        prepare_bf16(c, L);  // the operands exactly as the epsilon graph builds them (shift, rounding, row terms)
        const int4 item = make_int4(0, 1, -1, 0);
        c->items.reserve(sizeof(int4));
        RNNG_CUDA(cudaMemcpyAsync(c->items.ptr, &item, sizeof(int4), cudaMemcpyHostToDevice, s));
        L.items = c->items.as<int4>();
        L.num_items = 1;
        // the probe's one item is a row tile with one column tile (the row-pair form only
        // changes which resident A tile the MMAs read)
        L.item_tiles = std::min(2, gram_tune(c, 0, (int)d, 1).nt);
        L.gram_chunk = 2;
        c->aux7.reserve(sizeof(float) * (size_t)n * n);
        L.gram_raw = c->aux7.as<float>();
        RNNG_CUDA(cudaMemsetAsync(L.gram_raw, 0, sizeof(float) * (size_t)n * n, s));
        c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
        unsigned long long* cnt = c->counters.as<unsigned long long>() + 5;
        const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(c->tmap);
        const CUtensorMap& tmb = *reinterpret_cast<const CUtensorMap*>(c->tmapB);
        gram_candidates(c, L, tm, tmb, (int)d / kChunkK, L.item_tiles, c->bf16_fold, false,
                        (const float4*)c->bf16_rowinfo, (const float*)c->bf16_ucol, (const float2*)c->bf16_tileinfo,
                        c->bf16_eps_p, cnt);
        // G[i][j] = accumulator of A row i (input row i) and B row j (input row 128 + j)
        for (int i = 0; i < kTile; ++i)
            RNNG_CUDA(cudaMemcpyAsync(G + (int64_t)i * kTile, L.gram_raw + (int64_t)i * n + kTile, sizeof(float) * kTile,
                                      cudaMemcpyDeviceToHost, s));
        std::vector<__nv_bfloat16> xb((size_t)n * d);
        RNNG_CUDA(cudaMemcpyAsync(xb.data(), c->xb_sorted.ptr, sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyDeviceToHost,
                                  s));
        RNNG_CUDA(cudaMemcpyAsync(rowinfo, c->bf16_rowinfo, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        for (size_t k = 0; k < xb.size(); ++k) Xb[k] = __bfloat162float(xb[k]);
        c->aux7.release();
    });
}
