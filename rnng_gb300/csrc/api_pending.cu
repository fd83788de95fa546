// Entry points whose GPU pipelines are still being built report RNNG_ERR_UNSUPPORTED.
#include <cstring>

#include "common.cuh"

extern "C" {

int rnng_rips_l2(rnng_ctx* c, const float*, const int64_t*, int64_t, int64_t, float, int, int, unsigned,
                 rnng_simplices* out)
{
    if (out) std::memset(out, 0, sizeof(*out));
    if (c) c->last_error = "rnng_rips_l2: not available in this build";
    return RNNG_ERR_UNSUPPORTED;
}

}  // extern "C"
