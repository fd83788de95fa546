// Vietoris-Rips filtration up to triangles: rnng_rips_l2 (include/rnng_gpu.h).
//
// Replaces, on one GPU, RNNG's per-cell VoronoiComplex::build_filtration and the final
// merge (include/point.hpp:1136-1267, include/simplex.hpp:130-196).  RNNG builds each
// cell's complex over cell points plus ghosts and unions the cells; the union is the
// Rips complex of the whole point set, which is built here directly:
//   1. the epsilon graph of all points (the L2 pipeline, exact reference distances);
//   2. vertices are ranked by id, every edge is stored once as (a < b) in rank space and
//      sorted, giving a CSR of higher-ranked neighbours;
//   3. triangles a < b < c are found once each by intersecting, for every edge (a, b),
//      the neighbours of a after b with the neighbours of b (both lists sorted);
//   4. values: vertex 0, edge = its reference distance, triangle = the largest of its
//      three edges (RNNG's max over facet values, include/point.hpp:1194-1208);
//   5. ids: sum over the sorted vertex ids v_i of C(v_i, i + 1), OR-ed with dim << 60
//      (include/simplex.hpp:5-19), binomials as RNNG's Binom forms them
//      (include/utils.hpp:116-144): a falling product in 64-bit integers divided by k!;
//   6. all simplices sorted by (value, id).  Each simplex is built exactly once, so the
//      merge's unique-by-id step (include/simplex.hpp:173-174) has nothing to remove.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "eps_l2.cuh"
#include "kernels_misc.cuh"

namespace rnng {

__device__ __forceinline__ int64_t ref_binom(int64_t n, int64_t k)
{
    if (k > n) return 0;
    uint64_t a = 1, b = 1;
    for (int64_t i = n; i >= n - k + 1; --i) a *= (uint64_t)i;
    for (int64_t i = k; i >= 1; --i) b *= (uint64_t)i;
    return (int64_t)a / (int64_t)b;
}

__device__ __forceinline__ int64_t simplex_id1(int64_t a) { return (int64_t)((uint64_t)ref_binom(a, 1)); }
__device__ __forceinline__ int64_t simplex_id2(int64_t a, int64_t b)
{
    const uint64_t uid = (uint64_t)ref_binom(b, 2) + (uint64_t)ref_binom(a, 1);
    return (int64_t)(uid | (1ull << 60));
}
__device__ __forceinline__ int64_t simplex_id3(int64_t a, int64_t b, int64_t c)
{
    const uint64_t uid = (uint64_t)ref_binom(c, 3) + (uint64_t)ref_binom(b, 2) + (uint64_t)ref_binom(a, 1);
    return (int64_t)(uid | (2ull << 60));
}

__global__ void k_rank_iota(int64_t* __restrict__ keys, int32_t* __restrict__ rows, const int64_t* __restrict__ ids,
                            int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = ids ? ids[i] : i;
        rows[i] = (int32_t)i;
    }
}

__global__ void k_rank_of_row(const int32_t* __restrict__ row_of_rank, int64_t n, int32_t* __restrict__ rank)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        rank[row_of_rank[r]] = (int32_t)r;
}

// Sorted-index edges -> rank-space keys (a << 32 | b), a < b, with their weights.
__global__ void k_edge_keys(const uint32_t* __restrict__ si, const uint32_t* __restrict__ sj,
                            const float* __restrict__ sw, int64_t m, const int32_t* __restrict__ perm,
                            const int32_t* __restrict__ rank, uint64_t* __restrict__ key, float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)rank[perm[si[e]]], b = (uint32_t)rank[perm[sj[e]]];
        key[e] = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        w[e] = sw[e];
    }
}

__global__ void k_degree(const uint64_t* __restrict__ key, int64_t m, int32_t* __restrict__ deg)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&deg[key[e] >> 32], 1);
}

// For edge e = (a, b): the neighbours of a after b (CSR positions e+1 .. end of row a)
// intersected with the neighbours of b.  Counts (emit == false) or writes triangles.
template <bool emit>
__global__ void k_triangles(const uint64_t* __restrict__ key, const float* __restrict__ w,
                            const int32_t* __restrict__ row, int64_t m, const int64_t* __restrict__ id_of_rank,
                            int32_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t* __restrict__ out_id,
                            float* __restrict__ out_val)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)(key[e] >> 32), b = (uint32_t)(key[e] & 0xffffffffu);
        int64_t x = e + 1;
        const int64_t xe = row[a + 1];
        int64_t y = row[b];
        const int64_t ye = row[b + 1];
        const float wab = w[e];
        int64_t pos = emit ? off[e] : 0;
        int32_t found = 0;
        while (x < xe && y < ye) {
            const uint32_t cx = (uint32_t)(key[x] & 0xffffffffu), cy = (uint32_t)(key[y] & 0xffffffffu);
            if (cx < cy) {
                ++x;
            } else if (cx > cy) {
                ++y;
            } else {
                if (emit) {
                    const float v = fmaxf(fmaxf(wab, w[x]), w[y]);
                    const int64_t ia = id_of_rank[a], ib = id_of_rank[b], ic = id_of_rank[cx];
                    out_id[pos] = simplex_id3(ia, ib, ic);
                    out_val[pos] = v;
                    ++pos;
                }
                ++found;
                ++x;
                ++y;
            }
        }
        if (!emit) cnt[e] = found;
    }
}

__global__ void k_vertices_edges(const int64_t* __restrict__ id_of_rank, int64_t n, const uint64_t* __restrict__ key,
                                 const float* __restrict__ w, int64_t m, bool with_edges, int64_t* __restrict__ out_id,
                                 float* __restrict__ out_val)
{
    const int64_t total = n + (with_edges ? m : 0);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < n) {
            out_id[t] = simplex_id1(id_of_rank[t]);
            out_val[t] = 0.f;
        } else {
            const int64_t e = t - n;
            const uint32_t a = (uint32_t)(key[e] >> 32), b = (uint32_t)(key[e] & 0xffffffffu);
            out_id[t] = simplex_id2(id_of_rank[a], id_of_rank[b]);
            out_val[t] = w[e];
        }
    }
}

__global__ void k_id_of_rank(const int64_t* __restrict__ sorted_ids, int64_t n, int64_t* __restrict__ id_of_rank)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        id_of_rank[r] = sorted_ids[r];
}

__global__ void k_value_bits(const float* __restrict__ v, int64_t m, uint32_t* __restrict__ bits,
                             int32_t* __restrict__ idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        bits[i] = __float_as_uint(v[i]);  // values are >= +0, so bit order is numeric order
        idx[i] = (int32_t)i;
    }
}

template <class T>
__global__ void k_permute(const T* __restrict__ src, const int32_t* __restrict__ idx, int64_t m, T* __restrict__ dst)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

}  // namespace rnng

using namespace rnng;

extern "C" int rnng_rips_l2(rnng_ctx* c, const float* X, const int64_t* ids, int64_t n, int64_t d, float radius,
                            int maxdim, int mode, unsigned flags, rnng_simplices* out)
{
    if (!c) return RNNG_ERR_INVALID;
    try {
        RNNG_CUDA(cudaSetDevice(c->device));
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && d >= 1 && (n == 0 || X), RNNG_ERR_INVALID, "bad points");
        RNNG_REQUIRE(n < (int64_t(1) << 31) - kTile, RNNG_ERR_INVALID, "n too large");
        RNNG_REQUIRE(maxdim >= 0 && maxdim <= 2, RNNG_ERR_UNSUPPORTED, "maxdim above 2 is not supported");
        RNNG_REQUIRE(mode == RNNG_MODE_FP32_DIRECT || mode == RNNG_MODE_BF16_RECHECK, RNNG_ERR_INVALID, "bad mode");
        if (mode == RNNG_MODE_BF16_RECHECK)
            RNNG_REQUIRE(bf16_supported((int)d), RNNG_ERR_UNSUPPORTED, "BF16 mode supports d <= 256");
        RNNG_REQUIRE(radius == radius, RNNG_ERR_INVALID, "radius is NaN");
        c->stats = rnng_stats{};
        c->launches = 0;
        c->gram_ms = 0.0;
        cudaStream_t s = c->stream;
        RNNG_CUDA(cudaEventRecord(c->ev[0], s));
        const float* dX = X;
        const int64_t* dids = ids;
        if (!(flags & RNNG_INPUT_DEVICE)) {
            c->x_in.reserve(sizeof(float) * (size_t)std::max<int64_t>(n * d, 1));
            if (n) RNNG_CUDA(cudaMemcpyAsync(c->x_in.ptr, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
            dX = c->x_in.as<float>();
            if (ids) {
                c->ids_in.reserve(sizeof(int64_t) * (size_t)std::max<int64_t>(n, 1));
                RNNG_CUDA(cudaMemcpyAsync(c->ids_in.ptr, ids, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
                dids = c->ids_in.as<int64_t>();
            }
        }
        RNNG_CUDA(cudaEventRecord(c->ev[1], s));
        const int64_t ng = std::max<int64_t>(n, 1);
        const unsigned gn = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ng, 256), (int64_t)c->num_sms * 8));
        // ---- ranks: order of vertices by id (identity without ids)
        c->aux0.reserve(sizeof(int64_t) * 2 * (size_t)ng);
        c->aux1.reserve(sizeof(int32_t) * 3 * (size_t)ng + 16);
        int64_t* idk = c->aux0.as<int64_t>();
        int64_t* id_of_rank = idk + ng;
        int32_t* rows = c->aux1.as<int32_t>();
        int32_t* row_of_rank = rows + ng;
        int32_t* rank = row_of_rank + ng;
        k_rank_iota<<<gn, 256, 0, s>>>(idk, rows, dids, n);
        ++c->launches;
        if (dids && n > 1) {
            size_t tmp = 0;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, idk, id_of_rank, rows, row_of_rank, (int)n, 0, 64, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, idk, id_of_rank, rows, row_of_rank, (int)n, 0,
                                                      64, s));
            c->launches += cub_sort_kernels(n, 64);
        } else {
            RNNG_CUDA(cudaMemcpyAsync(id_of_rank, idk, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
            RNNG_CUDA(cudaMemcpyAsync(row_of_rank, rows, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
        }
        k_rank_of_row<<<gn, 256, 0, s>>>(row_of_rank, n, rank);
        ++c->launches;
        // ---- epsilon graph
        int64_t m = 0;
        Layout L;
        EdgeOut E;
        if (maxdim >= 1 && n >= 2 && radius >= 0.f) m = eps_core(c, dX, n, (int)d, radius, mode, L, E);
        RNNG_REQUIRE(n < (int64_t(1) << 32), RNNG_ERR_INVALID, "too many vertices");
        // ---- rank-space edge list sorted by (a, b) and its CSR
        const int64_t mg = std::max<int64_t>(m, 1);
        c->aux2.reserve(sizeof(uint64_t) * 2 * (size_t)mg + sizeof(float) * 2 * (size_t)mg + 32);
        uint64_t* k0 = c->aux2.as<uint64_t>();
        uint64_t* k1 = k0 + mg;
        float* w0 = (float*)(k1 + mg);
        float* w1 = w0 + mg;
        c->aux3.reserve(sizeof(int32_t) * 2 * ((size_t)ng + 1) + sizeof(int64_t) * ((size_t)mg + 1) +
                        sizeof(int32_t) * ((size_t)mg + 1) + 64);
        int32_t* deg = c->aux3.as<int32_t>();
        int32_t* rowp = deg + ng + 1;
        int32_t* tcnt = rowp + ng + 1;
        int64_t* toff = (int64_t*)(((uintptr_t)(tcnt + mg + 1) + 15) & ~(uintptr_t)15);
        int64_t ntri = 0;
        if (m > 0) {
            const unsigned gm = (unsigned)std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8);
            k_edge_keys<<<gm, 256, 0, s>>>(E.si, E.sj, E.w, m, L.perm, rank, k0, w0);
            ++c->launches;
            size_t tmp = 0;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, k0, k1, w0, w1, (int)m, 0, 64, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, k0, k1, w0, w1, (int)m, 0, 64, s));
            c->launches += cub_sort_kernels(m, 64);
            RNNG_CUDA(cudaMemsetAsync(deg, 0, sizeof(int32_t) * (ng + 1), s));
            k_degree<<<gm, 256, 0, s>>>(k1, m, deg);
            ++c->launches;
            exclusive_scan_i32(c, deg, rowp, n + 1);
            if (maxdim >= 2) {
                k_triangles<false><<<gm, 256, 0, s>>>(k1, w1, rowp, m, id_of_rank, tcnt, nullptr, nullptr, nullptr);
                ++c->launches;
                RNNG_CUDA(cudaMemsetAsync(tcnt + m, 0, sizeof(int32_t), s));
                tmp = 0;
                RNNG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, tcnt, toff, (int)(m + 1), s));
                c->cub_tmp.reserve(tmp);
                RNNG_CUDA(cub::DeviceScan::ExclusiveSum(c->cub_tmp.ptr, tmp, tcnt, toff, (int)(m + 1), s));
                c->launches += 2;
                RNNG_CUDA(cudaMemcpyAsync(&ntri, toff + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
                RNNG_CUDA(cudaStreamSynchronize(s));
            }
        }
        // ---- all simplices, then sort by (value, id)
        const int64_t nedge = maxdim >= 1 ? m : 0;
        const int64_t total = n + nedge + ntri;
        RNNG_REQUIRE(total < (int64_t(1) << 31), RNNG_ERR_INVALID, "too many simplices for one call");
        const int64_t tg = std::max<int64_t>(total, 1);
        c->out_u.reserve(sizeof(int64_t) * 2 * (size_t)tg);   // ids (two buffers)
        c->out_w.reserve(sizeof(float) * 2 * (size_t)tg);     // values
        c->out_v.reserve(sizeof(int32_t) * 2 * (size_t)tg + sizeof(uint32_t) * 2 * (size_t)tg);
        int64_t* id0 = c->out_u.as<int64_t>();
        int64_t* id1 = id0 + tg;
        float* v0 = c->out_w.as<float>();
        float* v1 = v0 + tg;
        int32_t* p0 = c->out_v.as<int32_t>();
        int32_t* p1 = p0 + tg;
        uint32_t* b0 = (uint32_t*)(p1 + tg);
        uint32_t* b1 = b0 + tg;
        const unsigned gt = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(tg, 256), (int64_t)c->num_sms * 8));
        if (n + nedge > 0) {
            k_vertices_edges<<<gt, 256, 0, s>>>(id_of_rank, n, k1, w1, m, maxdim >= 1, id0, v0);
            ++c->launches;
        }
        if (ntri > 0) {
            const unsigned gm = (unsigned)std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8);
            k_triangles<true><<<gm, 256, 0, s>>>(k1, w1, rowp, m, id_of_rank, nullptr, toff, id0 + n + nedge,
                                                 v0 + n + nedge);
            ++c->launches;
        }
        int64_t* ids_out = id0;
        float* vals_out = v0;
        if (total > 1) {
            // stable passes: by id, then by value bits
            size_t tmp = 0;
            k_value_bits<<<gt, 256, 0, s>>>(v0, total, b0, p0);
            ++c->launches;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, id0, id1, p0, p1, (int)total, 0, 64, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, id0, id1, p0, p1, (int)total, 0, 64, s));
            c->launches += cub_sort_kernels(total, 64);
            k_permute<uint32_t><<<gt, 256, 0, s>>>(b0, p1, total, b1);
            ++c->launches;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, b1, b0, p1, p0, (int)total, 0, 32, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, b1, b0, p1, p0, (int)total, 0, 32, s));
            c->launches += cub_sort_kernels(total, 32);
            k_permute<int64_t><<<gt, 256, 0, s>>>(id0, p0, total, id1);
            k_permute<float><<<gt, 256, 0, s>>>(v0, p0, total, v1);
            c->launches += 2;
            ids_out = id1;
            vals_out = v1;
        }
        // ---- deliver
        out->count = total;
        out->staged = 1;
        if (flags & RNNG_OUTPUT_DEVICE) {
            out->on_device = 1;
            out->id = ids_out;
            out->value = vals_out;
        } else {
            DevBuf& slot = c->host_stage;
            const size_t bi = sizeof(int64_t) * (size_t)tg, bf = sizeof(float) * (size_t)tg;
            if (bi + bf > slot.bytes) {
                if (slot.ptr) cudaFreeHost(slot.ptr);
                slot.ptr = nullptr;
                slot.bytes = 0;
                RNNG_CUDA(cudaMallocHost(&slot.ptr, bi + bf + 256));
                slot.bytes = bi + bf + 256;
            }
            out->id = (int64_t*)slot.ptr;
            out->value = (float*)((char*)slot.ptr + bi);
            if (total) {
                RNNG_CUDA(cudaMemcpyAsync(out->id, ids_out, sizeof(int64_t) * total, cudaMemcpyDeviceToHost, s));
                RNNG_CUDA(cudaMemcpyAsync(out->value, vals_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
            }
        }
        RNNG_CUDA(cudaEventRecord(c->ev[7], s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[7]);
        c->stats.ms_total = ms;
        c->stats.edges = m;
        c->stats.simplices = total;
        c->stats.tile_pairs = (int64_t)L.tile_pairs;
        c->stats.kernel_launches = c->launches;
        c->stats.ms_gram = c->gram_ms;
        c->last_error.clear();
        return RNNG_OK;
    } catch (const Error& e) {
        c->last_error = e.msg;
        return e.code;
    } catch (...) {
        c->last_error = "unknown error";
        return RNNG_ERR_INVALID;
    }
}
