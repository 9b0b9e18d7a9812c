// Serving engine (filled in later in this file's history).
#include "stride_gb300.h"
#include "stride_internal.h"

using namespace stride;

struct stride_server {
    int unused;
};

extern "C" {
int stride_server_create(const stride_server_opts*, stride_server** out) {
    if (out) *out = nullptr;
    return fail(STRIDE_ERR_UNSUPPORTED, "serving engine not built yet");
}
int stride_server_submit(stride_server*, const uint8_t*, size_t, uint64_t*) { return STRIDE_ERR_UNSUPPORTED; }
int stride_server_wait(stride_server*, uint64_t, int, stride_result*) { return STRIDE_ERR_UNSUPPORTED; }
int stride_server_release(stride_server*, uint64_t) { return STRIDE_ERR_UNSUPPORTED; }
int stride_server_stats(stride_server*, uint64_t*, uint64_t*, uint64_t*) { return STRIDE_ERR_UNSUPPORTED; }
void stride_server_destroy(stride_server*) {}
}
