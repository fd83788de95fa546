// Radius queries of a batch against an indexed set, exact Voronoi assignment, and the
// Graph edge-list finalisation.
//
//   rnng_radius_query_l2  - CoverTree::radius_query_batched / BruteForce::radius_query
//                           (include/search.hpp:267-340, 390-407): every (query, point)
//                           with the reference L2 <= radius.  Every tile of 128 queries
//                           meets every tile of 128 points (RNNG issues these queries per
//                           cell, on cell-sized batches), evaluated with the sequential
//                           FP32 L2.
//   rnng_voronoi_l2       - VoronoiDiagram::VoronoiDiagram (include/point.hpp:537-559):
//                           nearest centre with `dist <= best` over centres in increasing
//                           order (ties go to the last centre), distances bit-identical.
//   rnng_graph_finalize   - Graph(edges) + redistribute_edges at one rank
//                           (include/graph.h:14, include/graph.hpp:59-116): both
//                           orientations of every edge plus the self-loop (i, i, 0) of
//                           every vertex, sorted by (u, v), duplicates removed.
#include <cub/cub.cuh>

#include <algorithm>
#include <cfloat>
#include <cstring>

#include "common.cuh"
#include "eps_l2.cuh"
#include "kernels_misc.cuh"

namespace rnng {

constexpr int kQT = 128, kQK = 32;

// (query tile, point tile) pairs of the cross join, FP32-direct, one block per pair.
__global__ void __launch_bounds__(256) k_cross_tiles(const float* __restrict__ Q, int64_t nq,
                                                     const float* __restrict__ X, int64_t n, int d, float radius,
                                                     int64_t tiles_x, uint32_t* __restrict__ eu,
                                                     uint32_t* __restrict__ ev, float* __restrict__ ew,
                                                     unsigned long long* __restrict__ ecount, unsigned long long cap)
{
    __shared__ __align__(16) float As[kQK][kQT + 4];
    __shared__ __align__(16) float Bs[kQK][kQT + 4];
    __shared__ int s_warp[8];
    __shared__ unsigned long long s_base;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15, lane = tid & 31, warp = tid >> 5;
    const int64_t tiles_q = (nq + kQT - 1) / kQT;
    for (int64_t p = blockIdx.x; p < tiles_q * tiles_x; p += gridDim.x) {
        const int64_t i0 = (p / tiles_x) * kQT, j0 = (p % tiles_x) * kQT;
        float acc[8][8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[r][c] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kQK) {
            __syncthreads();
            for (int idx = tid; idx < kQT * kQK; idx += 256) {
                const int r = idx / kQK, c = idx % kQK, k = k0 + c;
                As[c][r] = (k < d && i0 + r < nq) ? Q[(i0 + r) * d + k] : 0.f;
                Bs[c][r] = (k < d && j0 + r < n) ? X[(j0 + r) * d + k] : 0.f;
            }
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kQK; ++k) {
                const float4 a0 = *reinterpret_cast<const float4*>(&As[k][ty * 8]);
                const float4 a1 = *reinterpret_cast<const float4*>(&As[k][ty * 8 + 4]);
                const float4 b0 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8]);
                const float4 b1 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8 + 4]);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[r][c] = l2seq_acc(acc[r][c], b[c], a[r]);
            }
        }
        int nhit = 0;
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                acc[r][c] = __fsqrt_rn(acc[r][c]);
                nhit += (gi < nq && gj < n && acc[r][c] <= radius);
            }
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
            s_base = a ? atomicAdd(ecount, (unsigned long long)a) : 0ull;
        }
        __syncthreads();
        unsigned long long pos = s_base + (unsigned long long)(s_warp[warp] + incl - nhit);
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                if (gi < nq && gj < n && acc[r][c] <= radius) {
                    if (pos < cap) {
                        eu[pos] = (uint32_t)gi;
                        ev[pos] = (uint32_t)gj;
                        ew[pos] = acc[r][c];
                    }
                    ++pos;
                }
            }
    }
}

__global__ void k_cross_out(const uint32_t* __restrict__ si, const uint32_t* __restrict__ sj,
                            const float* __restrict__ sw, int64_t m, const int64_t* __restrict__ qids,
                            const int64_t* __restrict__ ids, int64_t* __restrict__ u, int64_t* __restrict__ v,
                            float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        u[e] = qids ? qids[si[e]] : (int64_t)si[e];
        v[e] = ids ? ids[sj[e]] : (int64_t)sj[e];
        w[e] = sw[e];
    }
}

// Exact Voronoi assignment: one thread per point, centres staged through shared
// memory 32 dimensions at a time; every distance is the reference's sequential sum.
constexpr int kVP = 128, kVC = 32, kVK = 32;

__global__ void __launch_bounds__(kVP) k_voronoi(const float* __restrict__ X, int64_t n, const float* __restrict__ C,
                                                 int64_t m, int d, int64_t* __restrict__ cell, float* __restrict__ dist)
{
    __shared__ float cs[kVC][kVK + 1];
    __shared__ float xs[kVP][kVK + 1];
    const int64_t i = (int64_t)blockIdx.x * kVP + threadIdx.x;
    float best = FLT_MAX;  // the reference starts from std::numeric_limits<Real>::max()
    int64_t bi = 0;
    for (int64_t c0 = 0; c0 < m; c0 += kVC) {
        float acc[kVC];
#pragma unroll
        for (int c = 0; c < kVC; ++c) acc[c] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kVK) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < kVC * kVK; idx += kVP) {
                const int c = idx / kVK, k = k0 + idx % kVK;
                cs[c][idx % kVK] = (c0 + c < m && k < d) ? C[(c0 + c) * d + k] : 0.f;
            }
            for (int idx = threadIdx.x; idx < kVP * kVK; idx += kVP) {
                const int r = idx / kVK, k = k0 + idx % kVK;
                const int64_t row = (int64_t)blockIdx.x * kVP + r;
                xs[r][idx % kVK] = (row < n && k < d) ? X[row * d + k] : 0.f;
            }
            __syncthreads();
            const int kk = min(kVK, d - k0);
            for (int k = 0; k < kk; ++k) {
                const float xv = xs[threadIdx.x][k];
#pragma unroll
                for (int c = 0; c < kVC; ++c) acc[c] = l2seq_acc(acc[c], cs[c][k], xv);
            }
        }
#pragma unroll
        for (int c = 0; c < kVC; ++c) {
            if (c0 + c >= m) break;
            const float dv = __fsqrt_rn(acc[c]);
            if (dv <= best) {
                best = dv;
                bi = c0 + c;
            }
        }
    }
    if (i < n) {
        cell[i] = bi;
        dist[i] = best;
    }
}

// Finalisation: both orientations of every edge plus self-loops.
__global__ void k_orient(const int64_t* __restrict__ u, const int64_t* __restrict__ v, const float* __restrict__ w,
                         int64_t m, int64_t nv, int64_t* __restrict__ ou, int64_t* __restrict__ ov,
                         float* __restrict__ ow)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nv + 2 * m;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (e < nv) {
            ou[e] = e;
            ov[e] = e;
            ow[e] = 0.f;
        } else {
            const int64_t k = (e - nv) >> 1;
            const bool fwd = ((e - nv) & 1) == 0;
            ou[e] = fwd ? u[k] : v[k];
            ov[e] = fwd ? v[k] : u[k];
            ow[e] = w[k];
        }
    }
}

// Marks entries equal (u, v, w bits) to their predecessor in sorted order.
__global__ void k_mark_unique(const int64_t* __restrict__ u, const int64_t* __restrict__ v,
                              const float* __restrict__ w, int64_t m, int32_t* __restrict__ keep)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        keep[e] = (e == 0 || u[e] != u[e - 1] || v[e] != v[e - 1] ||
                   __float_as_uint(w[e]) != __float_as_uint(w[e - 1]))
                      ? 1
                      : 0;
}

}  // namespace rnng

using namespace rnng;

extern "C" {

int rnng_radius_query_l2(rnng_ctx* c, const float* X, const int64_t* ids, int64_t n, const float* Q,
                         const int64_t* qids, int64_t nq, int64_t d, float radius, unsigned flags, rnng_edges* out)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && nq >= 0 && d >= 1, RNNG_ERR_INVALID, "bad sizes");
        RNNG_REQUIRE((n == 0 || X) && (nq == 0 || Q), RNNG_ERR_INVALID, "null points");
        RNNG_REQUIRE(n < (int64_t(1) << 31) && nq < (int64_t(1) << 31), RNNG_ERR_INVALID, "too many points");
        RNNG_REQUIRE(radius == radius, RNNG_ERR_INVALID, "radius is NaN");
        c->stats = rnng_stats{};
        c->launches = 0;
        cudaStream_t s = c->stream;
        const float* dX = (const float*)upload(c, c->x_in, X, sizeof(float) * n * d, flags);
        const int64_t* dI = (const int64_t*)upload(c, c->ids_in, ids, sizeof(int64_t) * n, flags);
        const float* dQ = (const float*)upload(c, c->x_sorted, Q, sizeof(float) * nq * d, flags);
        const int64_t* dQI = (const int64_t*)upload(c, c->aux7, qids, sizeof(int64_t) * nq, flags);
        unsigned long long cap = std::max<unsigned long long>(1u << 16, c->edge_cap_hint);
        c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
        unsigned long long* cnt = c->counters.as<unsigned long long>() + 6;
        unsigned long long got = 0;
        if (n > 0 && nq > 0 && radius >= 0.f) {
            const int64_t tx = ceil_div(n, kQT), tq = ceil_div(nq, kQT);
            const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tx * tq, (int64_t)c->num_sms * 4));
            for (int attempt = 0;; ++attempt) {
                c->edges_u.reserve(sizeof(uint32_t) * cap);
                c->edges_v.reserve(sizeof(uint32_t) * cap);
                c->edges_w.reserve(sizeof(float) * cap);
                RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
                k_cross_tiles<<<grid, 256, 0, s>>>(dQ, nq, dX, n, (int)d, radius, tx, c->edges_u.as<uint32_t>(),
                                                   c->edges_v.as<uint32_t>(), c->edges_w.as<float>(), cnt, cap);
                ++c->launches;
                RNNG_CUDA(cudaGetLastError());
                RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
                RNNG_CUDA(cudaStreamSynchronize(s));
                if (got <= cap) break;
                RNNG_REQUIRE(attempt < 2, RNNG_ERR_OVERFLOW, "edge buffer overflow after regrowth");
                cap = got + got / 8 + 1024;
            }
        }
        const int64_t m = (int64_t)got;
        c->out_u.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
        c->out_v.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
        c->out_w.reserve(sizeof(float) * std::max<int64_t>(m, 1));
        if (m) {
            k_cross_out<<<(unsigned)std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8), 256, 0, s>>>(
                c->edges_u.as<uint32_t>(), c->edges_v.as<uint32_t>(), c->edges_w.as<float>(), m, dQI, dI,
                c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>());
            ++c->launches;
            if (flags & RNNG_SORT_OUTPUT)
                sort_edges_uv(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m);
        }
        deliver_edges(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m, flags, out);
        RNNG_CUDA(cudaStreamSynchronize(s));
        c->stats.edges = m;
        c->stats.kernel_launches = c->launches;
    });
}

int rnng_voronoi_l2(rnng_ctx* c, const float* X, int64_t n, const float* C, int64_t m, int64_t d, unsigned flags,
                    int64_t* cell, float* dist)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(n >= 0 && m >= 1 && d >= 1, RNNG_ERR_INVALID, "bad sizes (need at least one centre)");
        RNNG_REQUIRE((n == 0 || (X && cell && dist)) && C, RNNG_ERR_INVALID, "null pointer");
        c->stats = rnng_stats{};
        c->launches = 0;
        if (n == 0) return;
        cudaStream_t s = c->stream;
        const float* dX = (const float*)upload(c, c->x_in, X, sizeof(float) * n * d, flags);
        const float* dC = (const float*)upload(c, c->pivots, C, sizeof(float) * m * d, flags);
        int64_t* dcell = cell;
        float* ddist = dist;
        if (!(flags & RNNG_OUTPUT_DEVICE)) {
            c->out_u.reserve(sizeof(int64_t) * n);
            c->out_w.reserve(sizeof(float) * n);
            dcell = c->out_u.as<int64_t>();
            ddist = c->out_w.as<float>();
        }
        k_voronoi<<<(unsigned)ceil_div(n, kVP), kVP, 0, s>>>(dX, n, dC, m, (int)d, dcell, ddist);
        ++c->launches;
        RNNG_CUDA(cudaGetLastError());
        if (!(flags & RNNG_OUTPUT_DEVICE)) {
            RNNG_CUDA(cudaMemcpyAsync(cell, dcell, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaMemcpyAsync(dist, ddist, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
        }
        RNNG_CUDA(cudaStreamSynchronize(s));
        c->stats.kernel_launches = c->launches;
    });
}

int rnng_graph_finalize(rnng_ctx* c, const rnng_edges* edges, int64_t nv, unsigned flags, rnng_edges* out)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(edges && out && nv >= 0 && edges->count >= 0, RNNG_ERR_INVALID, "bad arguments");
        std::memset(out, 0, sizeof(*out));
        c->stats = rnng_stats{};
        c->launches = 0;
        cudaStream_t s = c->stream;
        const int64_t m = edges->count;
        const bool as_given = (flags & RNNG_FINALIZE_AS_GIVEN) != 0;
        const int64_t nself = as_given ? 0 : nv;  // self-loops added
        const int64_t total = nself + 2 * m;
        RNNG_REQUIRE(total < (int64_t(1) << 31), RNNG_ERR_INVALID, "too many edges");
        const unsigned in_flags = edges->on_device ? RNNG_INPUT_DEVICE : 0u;
        const int64_t* du = (const int64_t*)upload(c, c->x_in, edges->u, sizeof(int64_t) * m, in_flags);
        const int64_t* dv = (const int64_t*)upload(c, c->ids_in, edges->v, sizeof(int64_t) * m, in_flags);
        const float* dw = (const float*)upload(c, c->x_sorted, edges->w, sizeof(float) * m, in_flags);
        c->out_u.reserve(sizeof(int64_t) * std::max<int64_t>(total, 1));
        c->out_v.reserve(sizeof(int64_t) * std::max<int64_t>(total, 1));
        c->out_w.reserve(sizeof(float) * std::max<int64_t>(total, 1));
        int64_t* ou = c->out_u.as<int64_t>();
        int64_t* ov = c->out_v.as<int64_t>();
        float* ow = c->out_w.as<float>();
        int64_t kept = 0;
        if (total > 0) {
            const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(total, 256), (int64_t)c->num_sms * 8);
            k_orient<<<grid, 256, 0, s>>>(du, dv, dw, m, nself, ou, ov, ow);
            ++c->launches;
            // sort by (u, v) (as given: by (u, v, w)); equal (u, v) keep their weights adjacent
            // for the duplicate scan
            sort_edges_uv(c, ou, ov, ow, total, as_given);
            c->aux5.reserve(sizeof(int32_t) * total);
            c->aux4.reserve(sizeof(int64_t) * 2 * total + sizeof(float) * total + 16);
            int32_t* keep = c->aux5.as<int32_t>();
            k_mark_unique<<<grid, 256, 0, s>>>(ou, ov, ow, total, keep);
            ++c->launches;
            int64_t* cu = c->aux4.as<int64_t>();
            int64_t* cv = cu + total;
            float* cw = (float*)(cv + total);
            c->aux3.reserve(sizeof(int64_t) * 4);
            size_t tmp = 0;
            int64_t* dsel = c->aux3.as<int64_t>();
            RNNG_CUDA(cub::DeviceSelect::Flagged(nullptr, tmp, ou, keep, cu, dsel, (int)total, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceSelect::Flagged(c->cub_tmp.ptr, tmp, ou, keep, cu, dsel, (int)total, s));
            RNNG_CUDA(cub::DeviceSelect::Flagged(c->cub_tmp.ptr, tmp, ov, keep, cv, dsel, (int)total, s));
            RNNG_CUDA(cub::DeviceSelect::Flagged(c->cub_tmp.ptr, tmp, ow, keep, cw, dsel, (int)total, s));
            c->launches += 6;
            RNNG_CUDA(cudaMemcpyAsync(&kept, dsel, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            RNNG_CUDA(cudaMemcpyAsync(ou, cu, sizeof(int64_t) * kept, cudaMemcpyDeviceToDevice, s));
            RNNG_CUDA(cudaMemcpyAsync(ov, cv, sizeof(int64_t) * kept, cudaMemcpyDeviceToDevice, s));
            RNNG_CUDA(cudaMemcpyAsync(ow, cw, sizeof(float) * kept, cudaMemcpyDeviceToDevice, s));
        }
        deliver_edges(c, ou, ov, ow, kept, flags, out);
        RNNG_CUDA(cudaStreamSynchronize(s));
        c->stats.edges = kept;
        c->stats.kernel_launches = c->launches;
    });
}

}  // extern "C"
