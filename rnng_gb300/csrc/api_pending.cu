// Entry points whose GPU pipelines are still being built report RNNG_ERR_UNSUPPORTED.
#include <cstring>

#include "common.cuh"

extern "C" {

int rnng_radius_query_l2(rnng_ctx* c, const float*, const int64_t*, int64_t, const float*, const int64_t*, int64_t,
                         int64_t, float, unsigned, rnng_edges* out)
{
    if (out) std::memset(out, 0, sizeof(*out));
    if (c) c->last_error = "rnng_radius_query_l2: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

int rnng_voronoi_l2(rnng_ctx* c, const float*, int64_t, const float*, int64_t, int64_t, unsigned, int64_t*, float*)
{
    if (c) c->last_error = "rnng_voronoi_l2: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

int rnng_eps_graph_edit(rnng_ctx* c, const uint8_t*, const int64_t*, const int64_t*, int64_t, float, unsigned,
                        rnng_edges* out)
{
    if (out) std::memset(out, 0, sizeof(*out));
    if (c) c->last_error = "rnng_eps_graph_edit: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

int rnng_rips_l2(rnng_ctx* c, const float*, const int64_t*, int64_t, int64_t, float, int, int, unsigned,
                 rnng_simplices* out)
{
    if (out) std::memset(out, 0, sizeof(*out));
    if (c) c->last_error = "rnng_rips_l2: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

int rnng_graph_finalize(rnng_ctx* c, const rnng_edges*, int64_t, unsigned, rnng_edges* out)
{
    if (out) std::memset(out, 0, sizeof(*out));
    if (c) c->last_error = "rnng_graph_finalize: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

}  // extern "C"
