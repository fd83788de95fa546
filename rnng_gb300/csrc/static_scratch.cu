// Allocation-free epsilon graph: rnng_eps_graph_l2_static (include/rnng_gpu.h).
//
// Some callers cannot allocate device memory at the point where they need the graph:
// a process whose device memory is owned by a framework's pool (the framework hands
// out buffers but a plugin may not call cudaMalloc beside it), a real-time loop that
// must not allocate after start-up, or a plugin host that forbids allocation inside
// the plugin.  For them this entry point takes only caller-owned device buffers
// (points in, edges out) and keeps its own scratch in a fixed, file-scope device
// array, so it never calls cudaMalloc, cudaFree or any allocating library routine.
//
// Scratch: an edge counter, a flag word and up to kStaticEdges staged edges (two 32-bit
// point indices and the distance, 12 bytes each) - about 12 MiB that every GPU which
// loads the library keeps until the process exits.  Points are evaluated all pairs by
// all pairs in 128 x 128 tiles with RNNG's sequential FP32 L2 (no partition, so no
// further scratch), which bounds the problem size: n <= kStaticMaxPoints,
// d <= kStaticMaxDim.
//
// The device address of the array is looked up with cudaGetSymbolAddress once per
// device, on the first call made with that device current; make that first call
// before any stream capture.  All calls share the one array and it keeps the last
// call's contents; the counter and the flag are cleared at the start of every call.
// Calls whose GPU work overlaps (different streams, or different host threads on one
// device) race on the array and must be serialised by the caller.  Every call reads
// the edge count back to the host, so it synchronises the caller's stream before it
// returns.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "../../include/rnng_gpu.h"

namespace rnng_static {

constexpr int64_t kStaticEdges = 1 << 20;       // staged edges
constexpr int64_t kStaticMaxPoints = 1 << 16;   // points per call
constexpr int64_t kStaticMaxDim = 4096;         // dimensions per point
constexpr int kTileS = 128, kKCS = 32;
constexpr int kMaxDevices = 64;

struct __align__(256) Scratch {
    unsigned long long count;
    unsigned long long flag;  // 1: a row holds an infinity and no NaN (set only at radius +inf)
    unsigned long long pad[30];
    uint32_t si[kStaticEdges];
    uint32_t sj[kStaticEdges];
    float w[kStaticEdges];
};

static __device__ __align__(256) unsigned char g_scratch[sizeof(Scratch)];

// Tile pair (ti <= tj) of the implicit upper-triangular tile grid from a linear index.
__device__ __forceinline__ void tile_pair(int64_t t, int64_t T, int64_t& ti, int64_t& tj)
{
    // row ti holds T - ti pairs; walk rows (T is at most kStaticMaxPoints / 128 = 512)
    ti = 0;
    while (t >= T - ti) {
        t -= T - ti;
        ++ti;
    }
    tj = ti + t;
}

// All pairs of the two tiles with the reference L2 (sequential, no contraction,
// correctly rounded sqrt) <= radius, appended to the scratch with one atomic per
// block.  Same arithmetic as the library's FP32-direct tiles.
__global__ void __launch_bounds__(256) k_static_tiles(const float* __restrict__ X, int64_t n, int d, float radius,
                                                      Scratch* __restrict__ sc)
{
    __shared__ __align__(16) float As[kKCS][kTileS + 4];
    __shared__ __align__(16) float Bs[kKCS][kTileS + 4];
    __shared__ int s_warp[8];
    __shared__ unsigned long long s_base;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15, lane = tid & 31, warp = tid >> 5;
    const int64_t T = (n + kTileS - 1) / kTileS;
    const int64_t npairs = T * (T + 1) / 2;
    for (int64_t p = blockIdx.x; p < npairs; p += gridDim.x) {
        int64_t ti, tj;
        tile_pair(p, T, ti, tj);
        const int64_t i0 = ti * kTileS, j0 = tj * kTileS;
        float acc[8][8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[r][c] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kKCS) {
            __syncthreads();
            for (int idx = tid; idx < kTileS * kKCS; idx += 256) {
                const int r = idx / kKCS, c = idx % kKCS, k = k0 + c;
                As[c][r] = (k < d && i0 + r < n) ? X[(i0 + r) * d + k] : 0.f;
                Bs[c][r] = (k < d && j0 + r < n) ? X[(j0 + r) * d + k] : 0.f;
            }
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kKCS; ++k) {
                const float4 a0 = *reinterpret_cast<const float4*>(&As[k][ty * 8]);
                const float4 a1 = *reinterpret_cast<const float4*>(&As[k][ty * 8 + 4]);
                const float4 b0 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8]);
                const float4 b1 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8 + 4]);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const float t = __fsub_rn(a[r], b[c]);
                        acc[r][c] = __fadd_rn(acc[r][c], __fmul_rn(t, t));
                    }
            }
        }
        int nhit = 0;
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                acc[r][c] = __fsqrt_rn(acc[r][c]);
                nhit += (gi < n && gj < n && (ti != tj || gi < gj) && acc[r][c] <= radius);
            }
        // block prefix over the hit counts, one atomic per block
        int incl = nhit;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (tid == 0) {
            int a = 0;
            for (int k = 0; k < 8; ++k) { const int t = s_warp[k]; s_warp[k] = a; a += t; }
            s_base = a ? atomicAdd(&sc->count, (unsigned long long)a) : 0ull;
        }
        __syncthreads();
        unsigned long long pos = s_base + (unsigned long long)(s_warp[warp] + incl - nhit);
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                if (gi < n && gj < n && (ti != tj || gi < gj) && acc[r][c] <= radius) {
                    if (pos < (unsigned long long)kStaticEdges) {
                        sc->si[pos] = (uint32_t)gi;
                        sc->sj[pos] = (uint32_t)gj;
                        sc->w[pos] = acc[r][c];
                    }
                    ++pos;
                }
            }
    }
}

// Radius +inf only: raises sc->flag when some row holds an infinite coordinate and no
// NaN.  Such a row is at L2 +inf (not NaN) from the finite rows, so `+inf <= +inf`
// would make those pairs edges; the regular entry point refuses that case, and so does
// this one.  One warp per row.
__global__ void k_static_screen(const float* __restrict__ X, int64_t n, int d, Scratch* __restrict__ sc)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
        bool has_inf = false, has_nan = false;
        for (int k = lane; k < d; k += 32) {
            const float x = X[r * d + k];
            has_inf |= isinf(x);
            has_nan |= isnan(x);
        }
        has_inf = __any_sync(0xffffffffu, has_inf);
        has_nan = __any_sync(0xffffffffu, has_nan);
        if (lane == 0 && has_inf && !has_nan) atomicExch(&sc->flag, 1ull);
    }
}

// Staged edges -> the caller's arrays in id space with u < v.
__global__ void k_static_out(const Scratch* __restrict__ sc, int64_t m, const int64_t* __restrict__ ids,
                             int64_t* __restrict__ u, int64_t* __restrict__ v, float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = ids ? ids[sc->si[e]] : (int64_t)sc->si[e];
        const int64_t b = ids ? ids[sc->sj[e]] : (int64_t)sc->sj[e];
        u[e] = a < b ? a : b;
        v[e] = a < b ? b : a;
        w[e] = sc->w[e];
    }
}

// Device address of the scratch array, looked up once per device.
std::mutex g_mu;
Scratch* g_addr[kMaxDevices] = {};

cudaError_t scratch_for_current_device(Scratch** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<Scratch*>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace rnng_static

extern "C" int rnng_eps_graph_l2_static(const float* X, const int64_t* ids, int64_t n, int64_t d, float radius,
                                        int64_t* u, int64_t* v, float* w, int64_t capacity, int64_t* count,
                                        void* stream)
{
    using namespace rnng_static;
    if (count) *count = 0;
    if (!count || n < 0 || d < 1 || capacity < 0 || (n > 0 && !X)) return RNNG_ERR_INVALID;
    if (n > kStaticMaxPoints || d > kStaticMaxDim) return RNNG_ERR_INVALID;  // beyond the fixed scratch's limits
    if (capacity > 0 && (!u || !v || !w)) return RNNG_ERR_INVALID;
    if (radius != radius) return RNNG_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Scratch* sc = nullptr;
    if (scratch_for_current_device(&sc) != cudaSuccess) return RNNG_ERR_CUDA;
    // the counter and the flag start at zero on every call (the array keeps the previous
    // call's contents)
    if (cudaMemsetAsync(&sc->count, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess) return RNNG_ERR_CUDA;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return RNNG_ERR_CUDA;
    if (n >= 2 && radius == INFINITY) {
        const int64_t blocks = (n + 7) / 8;
        k_static_screen<<<(int)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8), 256, 0, s>>>(X, n, (int)d,
                                                                                                  sc);
        if (cudaGetLastError() != cudaSuccess) return RNNG_ERR_CUDA;
    }
    if (n >= 2 && radius >= 0.f) {
        const int64_t T = (n + kTileS - 1) / kTileS;
        const int64_t pairs = T * (T + 1) / 2;
        const int grid = (int)(pairs < (int64_t)sms * 4 ? pairs : (int64_t)sms * 4);
        k_static_tiles<<<grid, 256, 0, s>>>(X, n, (int)d, radius, sc);
        if (cudaGetLastError() != cudaSuccess) return RNNG_ERR_CUDA;
    }
    // the count and the flag, read back together
    unsigned long long head[2] = {0ull, 0ull};
    if (cudaMemcpyAsync(head, &sc->count, sizeof(head), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return RNNG_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RNNG_ERR_CUDA;
    if (head[1]) return RNNG_ERR_UNSUPPORTED;  // radius +inf with an infinite, NaN-free row
    const unsigned long long found = head[0];
    *count = (int64_t)found;
    const int64_t staged = (int64_t)found < kStaticEdges ? (int64_t)found : kStaticEdges;
    const int64_t m = staged < capacity ? staged : capacity;
    if (m > 0) {
        const int grid = (int)((m + 255) / 256 < 1024 ? (m + 255) / 256 : 1024);
        k_static_out<<<grid, 256, 0, s>>>(sc, m, ids, u, v, w);
        if (cudaGetLastError() != cudaSuccess) return RNNG_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return RNNG_ERR_CUDA;
    }
    if ((int64_t)found > kStaticEdges || (int64_t)found > capacity) return RNNG_ERR_OVERFLOW;
    return RNNG_OK;
}
