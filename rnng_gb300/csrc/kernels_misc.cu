// Device fault word, edge sorting, uploads and result delivery shared by the pipelines.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>

#include "kernels_misc.cuh"

namespace rnng {

void init_device_fault(rnng_ctx* c)
{
    if (!c->fault_word) RNNG_CUDA(cudaMalloc(&c->fault_word, sizeof(int) * 4));
    RNNG_CUDA(cudaMemset(c->fault_word, 0, sizeof(int) * 4));
}

void check_device_fault(rnng_ctx* c)
{
    int h[4] = {0, 0, 0, 0};
    RNNG_CUDA(cudaMemcpyAsync(h, c->fault_word, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    RNNG_CUDA(cudaStreamSynchronize(c->stream));
    if (h[0] != FAULT_NONE) {
        RNNG_CUDA(cudaMemsetAsync(c->fault_word, 0, sizeof(int) * 4, c->stream));
        throw Error{RNNG_ERR_DEVICE, "kernel fault word " + std::to_string(h[0]) + " (detail " + std::to_string(h[1]) +
                                         ", " + std::to_string(h[2]) + ")"};
    }
}

__global__ void k_iota(int32_t* out, int64_t m)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)i;
}

template <class T>
__global__ void k_gather(const T* __restrict__ src, const int32_t* __restrict__ idx, T* __restrict__ dst, int64_t m)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

// Weight bits of the edges in order idx (non-negative floats order as their bits).
__global__ void k_weight_keys(const float* __restrict__ w, const int32_t* __restrict__ idx, int64_t m,
                              uint32_t* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __float_as_uint(w[idx ? idx[i] : i]);
}

void sort_edges_uv(rnng_ctx* c, int64_t* u, int64_t* v, float* w, int64_t m, bool by_w)
{
    if (m <= 1) return;
    RNNG_REQUIRE(m < (int64_t(1) << 31), RNNG_ERR_INVALID, "too many edges to sort");
    cudaStream_t s = c->stream;
    c->aux6.reserve(sizeof(int64_t) * 2 * m);
    c->aux7.reserve(sizeof(int32_t) * 2 * m + sizeof(float) * m);
    int64_t* kbuf = c->aux6.as<int64_t>();
    int32_t* i0 = c->aux7.as<int32_t>();
    int32_t* i1 = i0 + m;
    float* wtmp = (float*)(i1 + m);
    int grid = (int)std::min<int64_t>((m + 255) / 256, (int64_t)c->num_sms * 8);
    k_iota<<<grid, 256, 0, s>>>(i0, m); ++c->launches;
    size_t tmp = 0;
    if (by_w) {
        // pass 0: by the weight (stable), so that (u, v) ties end up ordered by w
        uint32_t* wk = reinterpret_cast<uint32_t*>(kbuf);
        k_weight_keys<<<grid, 256, 0, s>>>(w, nullptr, m, wk); ++c->launches;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, wk, wk + m, i0, i1, (int)m, 0, 32, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, wk, wk + m, i0, i1, (int)m, 0, 32, s));
        c->launches += cub_sort_kernels(m, 32);
        // v in that order, then continue from it
        k_gather<int64_t><<<grid, 256, 0, s>>>(v, i1, kbuf + m, m); ++c->launches;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kbuf + m, kbuf, i1, i0, (int)m, 0, 64, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, kbuf + m, kbuf, i1, i0, (int)m, 0, 64, s));
        c->launches += cub_sort_kernels(m, 64);
        std::swap(i0, i1);  // i1 = order after the v pass
    } else {
    // pass 1: by v (stable), pass 2: by u (stable) -> ordered by (u, v)
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, v, kbuf, i0, i1, (int)m, 0, 64, s));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, v, kbuf, i0, i1, (int)m, 0, 64, s)); c->launches += cub_sort_kernels(m, 64);
    }
    k_gather<int64_t><<<grid, 256, 0, s>>>(u, i1, kbuf + m, m); ++c->launches;
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kbuf + m, kbuf, i1, i0, (int)m, 0, 64, s));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, kbuf + m, kbuf, i1, i0, (int)m, 0, 64, s)); c->launches += cub_sort_kernels(m, 64);
    // i0 = final order; u sorted = kbuf; v and w gathered
    RNNG_CUDA(cudaMemcpyAsync(u, kbuf, sizeof(int64_t) * m, cudaMemcpyDeviceToDevice, s));
    k_gather<int64_t><<<grid, 256, 0, s>>>(v, i0, kbuf, m); ++c->launches;
    RNNG_CUDA(cudaMemcpyAsync(v, kbuf, sizeof(int64_t) * m, cudaMemcpyDeviceToDevice, s));
    k_gather<float><<<grid, 256, 0, s>>>(w, i0, wtmp, m); ++c->launches;
    RNNG_CUDA(cudaMemcpyAsync(w, wtmp, sizeof(float) * m, cudaMemcpyDeviceToDevice, s));
}

const void* upload(rnng_ctx* c, DevBuf& buf, const void* p, size_t bytes, unsigned flags)
{
    // device data off a 16-byte boundary is copied, so that the kernels' 16-byte loads and
    // copies stay aligned
    const bool dev = flags & RNNG_INPUT_DEVICE;
    if (!p || (dev && (bytes == 0 || ((uintptr_t)p & 15u) == 0))) return p;
    buf.reserve(std::max<size_t>(bytes, 1));
    if (bytes)
        RNNG_CUDA(cudaMemcpyAsync(buf.ptr, p, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream));
    return buf.ptr;
}

void* host_stage(rnng_ctx* c, size_t bytes)
{
    DevBuf& slot = c->host_stage;  // a DevBuf holding a cudaMallocHost block
    if (bytes <= slot.bytes) return slot.ptr;
    if (slot.ptr) {
        RNNG_CUDA(cudaStreamSynchronize(c->stream));  // earlier copies may still target it
        cudaFreeHost(slot.ptr);
    }
    slot.ptr = nullptr;
    slot.bytes = 0;
    const size_t grow = bytes + bytes / 4 + 256;
    RNNG_CUDA(cudaMallocHost(&slot.ptr, grow));
    slot.bytes = grow;
    return slot.ptr;
}

void deliver_edges(rnng_ctx* c, const int64_t* du, const int64_t* dv, const float* dw, int64_t m, unsigned flags,
                   rnng_edges* out)
{
    std::memset(out, 0, sizeof(*out));
    out->count = m;
    out->staged = 1;
    if (flags & RNNG_OUTPUT_DEVICE) {
        out->on_device = 1;
        out->u = const_cast<int64_t*>(du);
        out->v = const_cast<int64_t*>(dv);
        out->w = const_cast<float*>(dw);
        return;
    }
    const size_t bi = sizeof(int64_t) * (size_t)std::max<int64_t>(m, 1);
    const size_t bf = sizeof(float) * (size_t)std::max<int64_t>(m, 1);
    char* h = (char*)host_stage(c, 2 * bi + bf);
    out->u = (int64_t*)h;
    out->v = (int64_t*)(h + bi);
    out->w = (float*)(h + 2 * bi);
    if (m) {
        RNNG_CUDA(cudaMemcpyAsync(out->u, du, sizeof(int64_t) * m, cudaMemcpyDeviceToHost, c->stream));
        RNNG_CUDA(cudaMemcpyAsync(out->v, dv, sizeof(int64_t) * m, cudaMemcpyDeviceToHost, c->stream));
        RNNG_CUDA(cudaMemcpyAsync(out->w, dw, sizeof(float) * m, cudaMemcpyDeviceToHost, c->stream));
    }
}

void deliver_simplices(rnng_ctx* c, const int64_t* did, const float* dval, const uint8_t* dflag, int64_t count,
                       unsigned flags, rnng_simplices* out)
{
    std::memset(out, 0, sizeof(*out));
    out->count = count;
    out->staged = 1;
    if (flags & RNNG_OUTPUT_DEVICE) {
        out->on_device = 1;
        out->id = const_cast<int64_t*>(did);
        out->value = const_cast<float*>(dval);
        out->flag = const_cast<uint8_t*>(dflag);
        return;
    }
    const size_t bi = sizeof(int64_t) * (size_t)std::max<int64_t>(count, 1);
    const size_t bf = sizeof(float) * (size_t)std::max<int64_t>(count, 1);
    const size_t bg = dflag ? (size_t)std::max<int64_t>(count, 1) : 0;
    char* h = (char*)host_stage(c, bi + bf + bg);
    out->id = (int64_t*)h;
    out->value = (float*)(h + bi);
    out->flag = dflag ? (uint8_t*)(h + bi + bf) : nullptr;
    if (count) {
        RNNG_CUDA(cudaMemcpyAsync(out->id, did, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, c->stream));
        RNNG_CUDA(cudaMemcpyAsync(out->value, dval, sizeof(float) * count, cudaMemcpyDeviceToHost, c->stream));
        if (dflag) RNNG_CUDA(cudaMemcpyAsync(out->flag, dflag, (size_t)count, cudaMemcpyDeviceToHost, c->stream));
    }
}

}  // namespace rnng
