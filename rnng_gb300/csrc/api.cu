// C ABI of librnng_gpu.so (declared in include/rnng_gpu.h).  Every entry point
// validates its arguments, runs on the context's stream, converts exceptions into
// status codes and records the message for rnng_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <new>

#include "common.cuh"
#include "eps_l2.cuh"
#include "balls.cuh"
#include "kernels_misc.cuh"

using namespace rnng;

namespace {

float elapsed(rnng_ctx* c, int a, int b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]) != cudaSuccess) return 0.f;
    return ms;
}

// Host points are copied to the context's buffer.  Device points are used in place when
// they start on a 16-byte boundary (the kernels read rows with 16-byte loads and copies);
// otherwise they are copied into the (aligned) buffer first.
const float* upload_f32(rnng_ctx* c, DevBuf& buf, const float* X, int64_t count, unsigned flags)
{
    const bool dev = flags & RNNG_INPUT_DEVICE;
    if (dev && (count == 0 || ((uintptr_t)X & 15u) == 0)) return X;
    buf.reserve(sizeof(float) * (size_t)std::max<int64_t>(count, 1));
    if (count)
        RNNG_CUDA(cudaMemcpyAsync(buf.ptr, X, sizeof(float) * count,
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
    return buf.as<float>();
}

const int64_t* upload_i64(rnng_ctx* c, DevBuf& buf, const int64_t* v, int64_t count, unsigned flags)
{
    if (!v) return nullptr;
    if (flags & RNNG_INPUT_DEVICE) return v;
    buf.reserve(sizeof(int64_t) * (size_t)std::max<int64_t>(count, 1));
    if (count) RNNG_CUDA(cudaMemcpyAsync(buf.ptr, v, sizeof(int64_t) * count, cudaMemcpyHostToDevice, c->stream));
    return buf.as<int64_t>();
}

// Runs the tile stage, growing the edge buffer and re-running when it overflowed.
int64_t tiles_with_retry(rnng_ctx* c, Layout& L, int mode, EdgeOut& E)
{
    unsigned long long cap = std::max<unsigned long long>(1u << 20, c->edge_cap_hint);
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    E.count = c->counters.as<unsigned long long>() + 4;
    for (int attempt = 0;; ++attempt) {
        c->edges_u.reserve(sizeof(uint32_t) * cap);
        c->edges_v.reserve(sizeof(uint32_t) * cap);
        c->edges_w.reserve(sizeof(float) * cap);
        E.si = c->edges_u.as<uint32_t>();
        E.sj = c->edges_v.as<uint32_t>();
        E.w = c->edges_w.as<float>();
        E.cap = cap;
        RNNG_CUDA(cudaMemsetAsync(E.count, 0, sizeof(unsigned long long), c->stream));
        if (mode == RNNG_MODE_BF16_RECHECK) run_tiles_bf16(c, L, E);
        else run_tiles_fp32(c, L, E);
        unsigned long long got = 0;
        RNNG_CUDA(cudaMemcpyAsync(&got, E.count, sizeof(got), cudaMemcpyDeviceToHost, c->stream));
        RNNG_CUDA(cudaStreamSynchronize(c->stream));
        check_device_fault(c);
        if (got <= E.cap) {  // (the direct output sizes E.cap to the candidates)
            c->edge_cap_hint = std::max<unsigned long long>(c->edge_cap_hint, got + got / 8);
            return (int64_t)got;
        }
        RNNG_REQUIRE(attempt < 2, RNNG_ERR_OVERFLOW, "edge buffer overflow after regrowth");
        cap = got + got / 8 + 1024;
        c->stats.retries++;
    }
}


// Stage times (CUDA events 0..10 of the call) and counts of an epsilon-graph call.
void record_eps_stats(rnng_ctx* c, const Layout& L, int mode, int64_t m)
{
    rnng_stats& st = c->stats;
    st.ms_h2d = elapsed(c, 0, 1);
    st.ms_partition = elapsed(c, 1, 2);
    st.ms_bounds = elapsed(c, 2, 3);
    st.ms_prune = elapsed(c, 3, 4);
    if (mode == RNNG_MODE_BF16_RECHECK) {
        st.ms_tiles = elapsed(c, 4, 8);
        st.ms_recheck = elapsed(c, 8, 5);
    } else {
        st.ms_tiles = elapsed(c, 4, 5);
    }
    st.ms_finalize = elapsed(c, 5, 6);
    st.ms_d2h = elapsed(c, 6, 7);
    st.ms_total = elapsed(c, 0, 7);
    st.num_cells = L.num_cells;
    st.super_pairs = (int64_t)L.super_pairs;
    st.tile_pairs = (int64_t)L.tile_pairs;
    st.tile_pairs_all = L.T * (L.T + 1) / 2;
    st.pairs_evaluated = (int64_t)L.tile_pairs * kTile * kTile;
    st.edges = m;
    st.candidates = c->last_candidates;
    st.kernel_launches = c->launches;
    st.ms_gram = c->gram_ms;
}

}  // namespace

namespace rnng {

// The L2 epsilon-graph pipeline on device-resident points (n >= 2, radius >= 0):
// partition, covers, pruning, tiles.  Edges stay in sorted-index space in E; the
// context events 2..5 (and 8..10 in BF16 mode) mark the stages.  Rows with a NaN or
// infinite coordinate get no edges (RNNG_ERR_UNSUPPORTED if the radius is +inf and a
// row has an infinity without a NaN).
int64_t eps_core(rnng_ctx* c, const float* dX, int64_t n, int d, float radius, int mode, Layout& L, EdgeOut& E)
{
    cudaStream_t s = c->stream;
    L = build_layout(c, dX, n, d, radius, true);
    int64_t n_in = n;
    bool remap = false;
    if (L.nonfinite) {
        // rows with a NaN or infinite coordinate have no edge under a finite radius: the
        // graph of the finite rows, mapped back to input rows at the end
        // (a row with a NaN is at L2 NaN from every row, so it has no edge at any radius;
        // rows with infinities only are at +inf from some rows, which an infinite radius
        // would admit)
        const float* Xf = dX;
        bool inf_rows = false;
        n = compact_finite_rows(c, dX, n_in, d, &Xf, &inf_rows);
        remap = n < n_in;
        RNNG_REQUIRE(!inf_rows || radius < std::numeric_limits<float>::infinity(), RNNG_ERR_UNSUPPORTED,
                     "infinite coordinates with an infinite radius");
        if (n < 2) {
            L = Layout{};
            L.d = d;
            for (int e : {2, 3, 4, 8, 5}) RNNG_CUDA(cudaEventRecord(c->ev[e], s));
            return 0;
        }
        L = build_layout(c, Xf, n, d, radius, false);
    }
    // sorted position -> input row from here on (the direct output maps through it)
    if (remap) remap_rows(c, L.perm, n, n_in);
    RNNG_CUDA(cudaEventRecord(c->ev[2], s));
    build_covers(c, L);
    RNNG_CUDA(cudaEventRecord(c->ev[3], s));
    prune_covers(c, L);
    RNNG_CUDA(cudaEventRecord(c->ev[4], s));
    // the BF16 candidate test needs its squared terms in FP32's normal range (coordinates
    // up to about 2^61 / sqrt(d), a radius of at least 2^-40); beyond it the FP32-direct
    // tiles evaluate the surviving tile pairs
    // tiles of few dimensions (d < kBf16MinDim, padded to 64 for the tensor cores) are
    // faster on the CUDA cores: at d = 8 (20k points) the FP32-direct tiles took 1.05 ms per
    // call against 1.25 ms for the BF16 Gram form, at d = 16 the Gram form was 1.2x faster
    const bool bf16_tiles = bf16_in_range(L) && L.d >= kBf16MinDim;
    const int tmode = (mode == RNNG_MODE_BF16_RECHECK && !bf16_tiles) ? RNNG_MODE_FP32_DIRECT : mode;
    if (tmode == RNNG_MODE_BF16_RECHECK) {
        const GramTune t = gram_tune(c, 0, (int)ceil_div(L.d, 64) * 64, (int64_t)L.tile_pairs);
        L.gram_chunk = t.chunk;
        L.gram_slots = t.slots;
        schedule_items(c, L, t.nt);
        prepare_bf16(c, L);
    }
    E.perm = L.perm;
    if (tmode != RNNG_MODE_BF16_RECHECK) E.direct = false;  // the FP32-direct tiles write sorted positions
    const int64_t m = tiles_with_retry(c, L, tmode, E);
    if (tmode != mode) RNNG_CUDA(cudaEventRecord(c->ev[8], s));
    RNNG_CUDA(cudaEventRecord(c->ev[5], s));
    return m;
}

}  // namespace rnng

extern "C" {

int rnng_ctx_create(int device, rnng_ctx** out)
{
    if (!out) return RNNG_ERR_INVALID;
    *out = nullptr;
    rnng_ctx* c = new (std::nothrow) rnng_ctx;
    if (!c) return RNNG_ERR_NOMEM;
    c->device = device;
    int rc = guarded(c, [&] {
        int ndev = 0;
        RNNG_CUDA(cudaGetDeviceCount(&ndev));
        RNNG_REQUIRE(device >= 0 && device < ndev, RNNG_ERR_INVALID, "no such device");
        RNNG_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        RNNG_CUDA(cudaGetDeviceProperties(&prop, device));
        RNNG_REQUIRE(prop.major >= 10, RNNG_ERR_UNSUPPORTED, "librnng_gpu needs a Blackwell (sm_100 family) GPU");
        c->num_sms = prop.multiProcessorCount;
        RNNG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
        ensure_events(c);
        init_device_fault(c);
        load_gram_table(c);
    });
    if (rc != RNNG_OK) {
        delete c;
        return rc;
    }
    *out = c;
    return RNNG_OK;
}

int rnng_ctx_destroy(rnng_ctx* c)
{
    if (!c) return RNNG_ERR_INVALID;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    rnng_ctx_trim(c);
    if (c->have_events)
        for (auto& e : c->ev) cudaEventDestroy(e);
    if (c->fault_word) cudaFree(c->fault_word);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RNNG_OK;
}

const char* rnng_last_error(const rnng_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int rnng_get_stats(const rnng_ctx* c, rnng_stats* out)
{
    if (!c || !out) return RNNG_ERR_INVALID;
    *out = c->stats;
    return RNNG_OK;
}

int rnng_ctx_stream(rnng_ctx* c, void** stream)
{
    if (!c || !stream) return RNNG_ERR_INVALID;
    *stream = (void*)c->stream;
    return RNNG_OK;
}

int rnng_ctx_set_gram_tuning(rnng_ctx* c, int nt, int chunk, int slots)
{
    if (!c || nt < 0 || nt > 3 || chunk < 0 || slots < 0 || slots == 1) return RNNG_ERR_INVALID;
    c->gram_force.nt = nt;
    c->gram_force.chunk = chunk;
    c->gram_force.slots = slots;
    return RNNG_OK;
}

int rnng_ctx_fault_drill(rnng_ctx* c, int on)
{
    if (!c) return RNNG_ERR_INVALID;
    c->fault_drill = on != 0;
    return RNNG_OK;
}

int rnng_ctx_trim(rnng_ctx* c)
{
    if (!c) return RNNG_ERR_INVALID;
    return guarded(c, [&] {
        RNNG_CUDA(cudaStreamSynchronize(c->stream));
        DevBuf* bufs[] = {&c->x_in, &c->ids_in, &c->x_sorted, &c->xb_sorted, &c->norms, &c->perm, &c->keys,
                          &c->keys_alt, &c->perm_alt, &c->cell, &c->dist, &c->pivots, &c->tile_lo, &c->tile_hi,
                          &c->super_lo, &c->super_hi, &c->pair_list, &c->super_list, &c->counters, &c->edges_u,
                          &c->edges_v, &c->edges_w, &c->out_u, &c->out_v, &c->out_w, &c->cub_tmp, &c->cand,
                          &c->aux0, &c->aux1, &c->aux2, &c->aux3, &c->aux4, &c->aux5, &c->aux6, &c->aux7, &c->sched,
                          &c->clq0, &c->clq1, &c->hi_id, &c->hi_val, &c->hi_flag, &c->sflag, &c->vflag,
                          &c->items, &c->items_tmp, &c->sched_tmp, &c->sym, &c->shift_buf, &c->ball_b16,
                          &c->ball_info, &c->sball_b16, &c->sball_info, &c->lm_b16, &c->xb_sortedB, &c->fin_x,
                          &c->fin_idx, &c->part_k, &c->part_v, &c->part_f};
        for (DevBuf* b : bufs) b->release();
        if (c->host_stage.ptr) cudaFreeHost(c->host_stage.ptr);
        c->host_stage.ptr = nullptr;
        c->host_stage.bytes = 0;
        c->edge_cap_hint = 0;
    });
}

int rnng_eps_graph_l2(rnng_ctx* c, const float* X, const int64_t* ids, int64_t n, int64_t d, float radius, int mode,
                      unsigned flags, rnng_edges* out)
{
    if (!c) return RNNG_ERR_INVALID;
    return guarded(c, [&] {
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && d >= 1 && (n == 0 || X != nullptr), RNNG_ERR_INVALID, "bad points");
        RNNG_REQUIRE(n < (int64_t(1) << 31) - kTile, RNNG_ERR_INVALID, "n too large (int32 point indices)");
        RNNG_REQUIRE(d <= 65536, RNNG_ERR_INVALID, "d too large");
        RNNG_REQUIRE(mode == RNNG_MODE_FP32_DIRECT || mode == RNNG_MODE_BF16_RECHECK, RNNG_ERR_INVALID, "bad mode");
        RNNG_REQUIRE(!(radius != radius), RNNG_ERR_INVALID, "radius is NaN");
        if (mode == RNNG_MODE_BF16_RECHECK)
            RNNG_REQUIRE(bf16_supported((int)d), RNNG_ERR_UNSUPPORTED, "BF16 mode supports d <= 256");
        c->stats = rnng_stats{};
        c->launches = 0;
        c->gram_ms = 0.0;
        cudaStream_t s = c->stream;
        RNNG_CUDA(cudaEventRecord(c->ev[0], s));
        const float* dX = upload_f32(c, c->x_in, X, n * d, flags);
        const int64_t* dids = upload_i64(c, c->ids_in, ids, n, flags);
        RNNG_CUDA(cudaEventRecord(c->ev[1], s));
        if (n < 2 || radius < 0.f) {
            // no pair can be an edge (a negative radius admits no distance)
            RNNG_CUDA(cudaEventRecord(c->ev[2], s));
            c->out_u.reserve(8);
            c->out_v.reserve(8);
            c->out_w.reserve(8);
            deliver_edges(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), 0, flags, out);
            RNNG_CUDA(cudaStreamSynchronize(s));
            return;
        }
        Layout L;
        EdgeOut E;
        // host results in any order: the recheck writes them to the pinned staging block itself
        E.direct = !(flags & (RNNG_OUTPUT_DEVICE | RNNG_SORT_OUTPUT)) && mode == RNNG_MODE_BF16_RECHECK;
        E.ids = dids;
        const int64_t m = eps_core(c, dX, n, (int)d, radius, mode, L, E);
        if (E.direct && E.hu) {
            RNNG_CUDA(cudaEventRecord(c->ev[6], s));
            std::memset(out, 0, sizeof(*out));
            out->count = m;
            out->staged = 1;
            out->u = E.hu;
            out->v = E.hv;
            out->w = E.hw;
            RNNG_CUDA(cudaEventRecord(c->ev[7], s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            RNNG_CUDA(cudaGetLastError());
            record_eps_stats(c, L, mode, m);
            return;
        }
        c->out_u.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
        c->out_v.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
        c->out_w.reserve(sizeof(float) * std::max<int64_t>(m, 1));
        finalize_edges(c, L, dids, E, m, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>());
        if (flags & RNNG_SORT_OUTPUT)
            sort_edges_uv(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m);
        RNNG_CUDA(cudaEventRecord(c->ev[6], s));
        deliver_edges(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m, flags, out);
        RNNG_CUDA(cudaEventRecord(c->ev[7], s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        RNNG_CUDA(cudaGetLastError());
        record_eps_stats(c, L, mode, m);
    });
}

int rnng_edges_free(rnng_edges* e)
{
    if (!e) return RNNG_ERR_INVALID;
    if (e->on_device && !e->staged) {
        cudaFree(e->u);
        cudaFree(e->v);
        cudaFree(e->w);
    }
    std::memset(e, 0, sizeof(*e));
    return RNNG_OK;
}

int rnng_simplices_free(rnng_simplices* s)
{
    if (!s) return RNNG_ERR_INVALID;
    if (s->on_device && !s->staged) {
        cudaFree(s->id);
        cudaFree(s->value);
    }
    std::memset(s, 0, sizeof(*s));
    return RNNG_OK;
}

}  // extern "C"
