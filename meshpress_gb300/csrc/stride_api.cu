// C ABI of the single-mesh decoder (include/stride_gb300.h): host header
// parse, device buffers, enqueue and status.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "stride_common.cuh"
#include "stride_gb300.h"
#include "stride_internal.h"

namespace stride {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(STRIDE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

static uint32_t be32(const uint8_t* p) {
    return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) |
           (static_cast<uint32_t>(p[2]) << 8) | p[3];
}

static float bef32(const uint8_t* p) {
    const uint32_t u = be32(p);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Global header of a DPR4 v3 stream (encoder/paradelta_v5_dup.py:412-447,
// read back at :472-501).
int parse_header(const uint8_t* data, size_t len, MeshParams* p, char* why, size_t why_len) {
    auto say = [&](int code, const char* msg) {
        if (why && why_len) snprintf(why, why_len, "%s", msg);
        return code;
    };
    std::memset(p, 0, sizeof(*p));
    if (!data) return say(STRIDE_ERR_ARG, "null stream");
    if (len < kHeaderBytes) return say(STRIDE_ERR_TRUNCATED, "stream shorter than the 86-byte DPR4 header");
    if (be32(data) != kMagic) {
        char m[96];
        snprintf(m, sizeof(m), "bad magic 0x%08X (expected DPR4 0x44505234)", be32(data));
        return say(STRIDE_ERR_MAGIC, m);
    }
    if (data[4] != kVersion) {
        char m[64];
        snprintf(m, sizeof(m), "DPR4 version %u (expected 3)", data[4]);
        return say(STRIDE_ERR_VERSION, m);
    }
    float center[3], gmin[3], grange[3];
    for (int i = 0; i < 3; i++) center[i] = bef32(data + 6 + 4 * i);
    const float scale = bef32(data + 18);
    for (int i = 0; i < 3; i++) gmin[i] = bef32(data + 26 + 4 * i);
    for (int i = 0; i < 3; i++) grange[i] = bef32(data + 38 + 4 * i);
    for (int i = 0; i < 3; i++) p->g_bits[i] = data[50 + i];
    for (int i = 0; i < 9; i++) {
        const uint32_t v = (static_cast<uint32_t>(data[53 + 2 * i]) << 8) | data[54 + 2 * i];
        p->pred_n[i] = (v & 0x8000u) ? static_cast<int32_t>(v) - 0x10000 : static_cast<int32_t>(v);
    }
    for (int i = 0; i < 3; i++) p->pred_k[i] = data[71 + i];
    p->n_v = be32(data + 74);
    p->n_t = be32(data + 78);
    p->n_meshlets = be32(data + 82);
    const unsigned long long table_end = kHeaderBytes + 4ull * p->n_meshlets;
    if (table_end > len) return say(STRIDE_ERR_TRUNCATED, "offset table runs past the end of the stream");
    if (len * 8ull >= (1ull << 32) - 4096) return say(STRIDE_ERR_UNSUPPORTED, "stream longer than 512 MB");
    if (p->n_meshlets == 0) return say(STRIDE_ERR_CORRUPT, "stream has no meshlets");
    for (int d = 0; d < 3; d++) {
        if (p->g_bits[d] > static_cast<uint32_t>(kMaxGBits))
            return say(STRIDE_ERR_UNSUPPORTED, "more than 24 bits per axis");
        if (p->pred_k[d] > 30) return say(STRIDE_ERR_UNSUPPORTED, "predictor shift K above 30");
        p->code_max[d] = (1u << p->g_bits[d]) - 1u;
        p->pred_half[d] = p->pred_k[d] ? (1 << (p->pred_k[d] - 1)) : 0;
        // the int32 IRLP sum of in-range codes must not overflow
        long long bound = 0;
        for (int j = 0; j < 3; j++) bound += std::llabs(static_cast<long long>(p->pred_n[3 * d + j]));
        bound = bound * static_cast<long long>(p->code_max[d]) + p->pred_half[d];
        if (bound >= (1ll << 31)) return say(STRIDE_ERR_UNSUPPORTED, "IRLP weights overflow int32 arithmetic");
        stride_dequant_setup(&p->dq[d], center[d], scale, gmin[d], grange[d], p->g_bits[d]);
    }
    p->nbits = len * 8ull;
    p->body_bit = static_cast<uint32_t>(table_end * 8ull);
    p->anchor_bits = p->g_bits[0] + p->g_bits[1] + p->g_bits[2];
    p->meshlet_begin = 0;
    p->blob_off = 0;
    p->v_offset = 0;
    p->t_offset = 0;
    return STRIDE_OK;
}

size_t blob_alloc_bytes(size_t len) { return (len + kBlobPad + 255) & ~static_cast<size_t>(255); }

int status_to_code(const Status& st, uint32_t* bad_meshlet) {
    if (st.err == 0ull) return STRIDE_OK;
    const int code = static_cast<int>(st.err >> 32);
    if (bad_meshlet) *bad_meshlet = static_cast<uint32_t>(st.err & 0xFFFFFFFFull);
    switch (code) {
        case kErrOffset: return STRIDE_ERR_OFFSET;
        case kErrCorrupt: return STRIDE_ERR_CORRUPT;
        case kErrUnsupported: return STRIDE_ERR_UNSUPPORTED;
        case kErrTimeout: return STRIDE_ERR_TIMEOUT;
        default: return STRIDE_ERR_CORRUPT;
    }
}

const char* status_message(int code) {
    switch (code) {
        case STRIDE_ERR_OFFSET: return "meshlet offset table out of order or out of range";
        case STRIDE_ERR_CORRUPT: return "meshlet payload inconsistent with its header or the offset table";
        case STRIDE_ERR_UNSUPPORTED: return "meshlet outside this decoder's limits (>256 vertices/triangles, k>24)";
        case STRIDE_ERR_TIMEOUT: return "a bounded device wait gave up";
        default: return "decode failed";
    }
}

}  // namespace stride

using namespace stride;

namespace stride {

unsigned long long plan_luts(MeshParams* p, uint32_t n, uint32_t* meshes, uint32_t max_meshes, uint32_t* n_lut,
                             uint32_t* lut_max) {
    unsigned long long total = 0;
    uint32_t k = 0, mx = 0;
    for (uint32_t i = 0; i < n; i++) {
        p[i].has_lut = 0;
        p[i].lut_off = 0;
        const unsigned long long e = lut_entries(p[i]);
        if (!e || k >= max_meshes || k >= 65535u) continue;  // bounds the table blocks of the scan launch
        p[i].has_lut = 1;
        p[i].lut_off = total;
        total += e;
        if (meshes) meshes[k] = i;
        k++;
        mx = std::max<uint32_t>(mx, static_cast<uint32_t>(e));
    }
    *n_lut = k;
    *lut_max = mx;
    return total;
}

}  // namespace stride

struct stride_handle {
    int device = 0;
    size_t len = 0, cap_bytes = 0;
    uint32_t cap_meshlets = 0;
    uint8_t* d_blob = nullptr;
    MeshParams params;
    MeshParams* d_params = nullptr;
    MeshletDesc* d_descs = nullptr;
    uint4* d_blk_sums = nullptr;
    BlockPrefix* d_blk_prefix = nullptr;
    uint32_t* d_walk_scratch = nullptr;
    unsigned long long walk_cap = 0;
    Status* d_status = nullptr;
    uint32_t* d_idx = nullptr;
    float* d_pos = nullptr;
    size_t cap_v = 0, cap_t = 0;
    float* d_lut = nullptr;             // dequantisation tables
    unsigned long long lut_cap = 0;     // floats
    uint32_t* d_lut_mesh = nullptr;     // the one-entry mesh list {0}
    uint32_t n_lut = 0, lut_max = 0;
    cudaEvent_t done = nullptr;
    bool launched = false;
    LaunchCfg cfg;
    bool cfg_set = false;               // stride_set_config called: keep cfg across reloads
    long long wait_clocks = 1ll << 31;  // DecodeArgs::wait_clocks of this handle's decodes
    uint32_t launch_smem = 0, launch_grid = 0;  // the last decode's main kernel
    HostLink link;          // stride_decode_host, and a reload that uploads by parts
    bool up_parts = false;  // the last reload uploaded by parts (link.bytes_in)
};

// A reload that uploaded by parts: the decode stream waits for all of it
// (decodes that do not go by parts).
static cudaError_t wait_upload(stride_handle* h, cudaStream_t s) {
    return h->up_parts ? cudaStreamWaitEvent(s, h->link.bytes_in[kHostParts - 1], 0) : cudaSuccess;
}

namespace stride {

static void for_link_events(HostLink& L, void (*f)(cudaEvent_t*, cudaError_t*), cudaError_t* e) {
    for (cudaEvent_t* ev : {&L.conn_done, &L.vert_done, &L.done, &L.copied[0], &L.copied[1], &L.before_up})
        f(ev, e);
    for (int p = 0; p < kHostParts; p++)
        for (cudaEvent_t* ev : {&L.part_done[p], &L.scan_done[p], &L.end_in[p], &L.bytes_in[p]}) f(ev, e);
}

void host_link_free(HostLink& L) {
    for (cudaStream_t* c : {&L.copy[0], &L.copy[1], &L.up})
        if (*c) cudaStreamDestroy(*c), *c = nullptr;
    for_link_events(L, [](cudaEvent_t* ev, cudaError_t*) { if (*ev) cudaEventDestroy(*ev), *ev = nullptr; }, nullptr);
    cudaFreeHost(L.h_end);
    L.h_end = nullptr;
    cudaFreeHost(L.h_status);
    L.h_status = nullptr;
}

cudaError_t host_link_init(HostLink& L) {
    if (L.copy[0]) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    for (cudaStream_t* c : {&L.copy[0], &L.copy[1], &L.up})
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(c, cudaStreamNonBlocking);
    for_link_events(L, [](cudaEvent_t* ev, cudaError_t* err) {
        if (*err == cudaSuccess) *err = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    }, &e);
    if (e == cudaSuccess) e = cudaHostAlloc(&L.h_status, sizeof(Status), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(&L.h_end, kHostParts * sizeof(PartEnd), cudaHostAllocDefault);
    if (e != cudaSuccess) host_link_free(L);
    return e;
}

void host_part_groups(uint32_t total_meshlets, uint32_t* part_g) {
    const uint32_t n_groups = (total_meshlets + 31u) / 32u;
    const uint32_t n_win = (n_groups + 7u) / 8u;
    for (int p = 0; p < kHostParts; p++)
        part_g[p] = 8u * static_cast<uint32_t>(static_cast<uint64_t>(n_win) * p / kHostParts);
    part_g[kHostParts] = n_groups;
}

int decode_to_host(HostLink& L, const DecodeArgs& a, LaunchCfg cfg, void* stream, uint64_t n_t, uint64_t n_v,
                   uint32_t* h_idx, float* h_pos, const cudaEvent_t* bytes_in, uint32_t* bad, bool* ran) {
    *ran = false;
    cudaError_t e = host_link_init(L);
    if (e != cudaSuccess) return cuda_fail(e, "copy streams");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // a failure once work is queued: nothing may still run on the buffers
    // or write the host outputs when this returns
    auto drain = [&]() {
        cudaStreamSynchronize(s);
        cudaStreamSynchronize(L.copy[0]);
        cudaStreamSynchronize(L.copy[1]);
    };
    auto bail = [&](cudaError_t err, const char* what) {
        drain();
        return cuda_fail(err, what);
    };
    if (cfg.persistent == 2) cfg.persistent = 1;
    const size_t ib = 12 * n_t, pb = 12 * n_v;
    const bool parts = cfg.persistent < 2 && host_parts(n_t, a.total_meshlets);
    if (parts) {
        // Part by part: its scan, the read-back of its end (the next part's
        // first triangle row), its connectivity; then, once its end is
        // known, the copy of its triangles, queued before the next part's
        // kernels so that it starts as soon as the part's connectivity ends.
        // A corrupt stream's ends are clamped (its status reports it).
        uint32_t part_g[kHostParts + 1];
        host_part_groups(a.total_meshlets, part_g);
        int rc = enqueue_parts_begin(a, cfg, stream);
        size_t from = 0;
        for (int p = 0; p < kHostParts && rc == STRIDE_OK && e == cudaSuccess; p++) {
            rc = enqueue_part(a, cfg, stream, part_g[p], part_g[p + 1], p == 0, bytes_in ? bytes_in[p] : nullptr,
                              L.scan_done[p], L.part_done[p]);
            if (rc) break;
            size_t to = ib;
            if (p + 1 < kHostParts) {
                const uint32_t last = part_g[p + 1] / 8u - 1u;  // the part's last window
                if ((e = cudaStreamWaitEvent(L.copy[1], L.scan_done[p], 0)) != cudaSuccess ||
                    (e = cudaMemcpyAsync(&L.h_end[p].prefix, a.blk_prefix + last, sizeof(BlockPrefix),
                                         cudaMemcpyDeviceToHost, L.copy[1])) != cudaSuccess ||
                    (e = cudaMemcpyAsync(&L.h_end[p].sums, a.blk_sums + last, sizeof(uint4), cudaMemcpyDeviceToHost,
                                         L.copy[1])) != cudaSuccess ||
                    (e = cudaEventRecord(L.end_in[p], L.copy[1])) != cudaSuccess ||
                    (e = cudaEventSynchronize(L.end_in[p])) != cudaSuccess)
                    break;
                const PartEnd& pe = L.h_end[p];
                to = std::max(from, 12 * std::min<size_t>(pe.prefix.t + pe.sums.y, n_t));
            }
            if ((e = cudaStreamWaitEvent(L.copy[0], L.part_done[p], 0)) == cudaSuccess && to > from)
                e = cudaMemcpyAsync(reinterpret_cast<uint8_t*>(h_idx) + from,
                                    reinterpret_cast<const uint8_t*>(a.idx) + from, to - from,
                                    cudaMemcpyDeviceToHost, L.copy[0]);
            from = to;
        }
        if (rc == STRIDE_OK && e == cudaSuccess) rc = enqueue_parts_end(a, cfg, stream, L.vert_done);
        if (e != cudaSuccess) return bail(e, "decode to host: parts");
        if (rc) {
            drain();
            return fail(rc, "decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        }
    } else {
        if (bytes_in && (e = cudaStreamWaitEvent(s, bytes_in[kHostParts - 1], 0)) != cudaSuccess)
            return cuda_fail(e, "decode to host: upload");
        void* ev[4] = {nullptr, nullptr, L.conn_done, L.vert_done};
        const int rc = enqueue_decode(a, cfg, stream, ev);
        if (rc) return fail(rc, "decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    }
    // each output (the triangles unless they went by parts) in two halves,
    // one per copy stream
    const size_t ih = (ib / 2) & ~size_t(15), ph = (pb / 2) & ~size_t(15);
    const size_t ioff[2] = {0, ih}, ilen[2] = {ih, ib - ih};
    const size_t poff[2] = {0, ph}, plen[2] = {ph, pb - ph};
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        cudaStream_t c = L.copy[k];
        if (!parts && (e = cudaStreamWaitEvent(c, L.conn_done, 0)) == cudaSuccess && ilen[k])
            e = cudaMemcpyAsync(reinterpret_cast<uint8_t*>(h_idx) + ioff[k],
                                reinterpret_cast<const uint8_t*>(a.idx) + ioff[k], ilen[k], cudaMemcpyDeviceToHost, c);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c, L.vert_done, 0);
        if (e == cudaSuccess && plen[k])
            e = cudaMemcpyAsync(reinterpret_cast<uint8_t*>(h_pos) + poff[k],
                                reinterpret_cast<const uint8_t*>(a.pos) + poff[k], plen[k], cudaMemcpyDeviceToHost, c);
        // the status is final with the vertex kernel: it comes back with the
        // positions, and no synchronous read follows the decode
        if (e == cudaSuccess && k == 1)
            e = cudaMemcpyAsync(L.h_status, a.status, sizeof(Status), cudaMemcpyDeviceToHost, c);
        if (e == cudaSuccess) e = cudaEventRecord(L.copied[k], c);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, L.copied[k], 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(L.done, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(L.done);
    if (e != cudaSuccess) return bail(e, "decode to host: copies");
    *ran = true;
    return status_to_code(*L.h_status, bad);
}

}  // namespace stride

static void free_buffers(stride_handle* h) {
    cudaFree(h->d_blob);
    cudaFree(h->d_params);
    cudaFree(h->d_descs);
    cudaFree(h->d_blk_sums);
    cudaFree(h->d_blk_prefix);
    cudaFree(h->d_walk_scratch);
    cudaFree(h->d_status);
    cudaFree(h->d_idx);
    cudaFree(h->d_pos);
    cudaFree(h->d_lut);
    cudaFree(h->d_lut_mesh);
    h->d_lut = nullptr;
    h->d_lut_mesh = nullptr;
    h->lut_cap = 0;
    h->d_walk_scratch = nullptr;
    h->walk_cap = 0;
    h->d_blob = nullptr;
    h->d_params = nullptr;
    h->d_descs = nullptr;
    h->d_blk_sums = nullptr;
    h->d_blk_prefix = nullptr;
    h->d_status = nullptr;
    h->d_idx = nullptr;
    h->d_pos = nullptr;
}

// Buffers for a stream of this size; also plans the dequantisation tables
// of `p` (has_lut, lut_off) and sizes their buffer.
static int ensure_capacity(stride_handle* h, size_t len, MeshParams& p) {
    const uint32_t n_meshlets = p.n_meshlets;
    const uint64_t n_v = p.n_v;
    cudaError_t e;
    const unsigned long long lut = plan_luts(&p, 1, nullptr, 1, &h->n_lut, &h->lut_max);
    if (!h->d_lut_mesh) {
        const uint32_t zero = 0u;
        if ((e = cudaMalloc(&h->d_lut_mesh, sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaMemcpy(h->d_lut_mesh, &zero, sizeof(zero), cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(table list)");
    }
    if (lut > h->lut_cap) {
        cudaFree(h->d_lut);
        h->d_lut = nullptr;
        if ((e = cudaMalloc(&h->d_lut, 4ull * lut)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
        h->lut_cap = lut;
    }
    const unsigned long long ww = walk_scratch_words(n_v, n_meshlets);
    if (ww > h->walk_cap) {
        cudaFree(h->d_walk_scratch);
        h->d_walk_scratch = nullptr;
        if ((e = cudaMalloc(&h->d_walk_scratch, 4ull * ww)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
        h->walk_cap = ww;
    }
    if (blob_alloc_bytes(len) > h->cap_bytes) {
        cudaFree(h->d_blob);
        h->d_blob = nullptr;
        h->cap_bytes = blob_alloc_bytes(len);
        if ((e = cudaMalloc(&h->d_blob, h->cap_bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(stream)");
    }
    if (n_meshlets > h->cap_meshlets) {
        cudaFree(h->d_descs);
        cudaFree(h->d_blk_sums);
        cudaFree(h->d_blk_prefix);
        h->d_descs = nullptr;
        h->d_blk_sums = nullptr;
        h->d_blk_prefix = nullptr;
        const uint32_t nb = scan_blocks(n_meshlets);
        if ((e = cudaMalloc(&h->d_descs, sizeof(MeshletDesc) * n_meshlets)) != cudaSuccess ||
            (e = cudaMalloc(&h->d_blk_sums, sizeof(uint4) * nb)) != cudaSuccess ||
            (e = cudaMalloc(&h->d_blk_prefix, sizeof(BlockPrefix) * nb)) != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(scratch)");
        h->cap_meshlets = n_meshlets;
    }
    return STRIDE_OK;
}

extern "C" {

const char* stride_last_error_message(void) { return g_last_error.c_str(); }

const char* stride_error_string(int code) {
    switch (code) {
        case STRIDE_OK: return "ok";
        case STRIDE_ERR_ARG: return "bad argument";
        case STRIDE_ERR_MAGIC: return "bad magic";
        case STRIDE_ERR_VERSION: return "unsupported version";
        case STRIDE_ERR_TRUNCATED: return "truncated stream";
        case STRIDE_ERR_OFFSET: return "bad meshlet offset table";
        case STRIDE_ERR_CORRUPT: return "corrupt meshlet payload";
        case STRIDE_ERR_UNSUPPORTED: return "unsupported stream parameters";
        case STRIDE_ERR_CUDA: return "CUDA error";
        case STRIDE_ERR_TIMEOUT: return "timeout";
        case STRIDE_ERR_NOMEM: return "out of memory";
        case STRIDE_ERR_BUSY: return "busy";
        default: return "unknown error";
    }
}

int stride_device_info(int* sm_count, int* arch) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (sm_count) *sm_count = device_sm_count();
    if (arch) *arch = 103;
    return STRIDE_OK;
}

static void fill_info(const MeshParams& p, size_t len, int persistent, stride_info_t* info) {
    std::memset(info, 0, sizeof(*info));
    info->n_meshlets = p.n_meshlets;
    for (int i = 0; i < 3; i++) {
        info->g_bits[i] = p.g_bits[i];
        info->center[i] = static_cast<float>(p.dq[i].center);
        info->g_min[i] = static_cast<float>(p.dq[i].gmin);
        info->g_range[i] = static_cast<float>(p.dq[i].grange);
        info->pred_k[i] = p.pred_k[i];
    }
    for (int i = 0; i < 9; i++) info->pred_n[i] = p.pred_n[i];
    info->scale = static_cast<float>(p.dq[0].scale);
    info->n_v = p.n_v;
    info->n_t = p.n_t;
    info->nbytes = len;
    // scan (+ tables), then one kernel (group or fused) or the connectivity and vertex kernels
    info->kernels = p.n_meshlets ? (persistent >= 2 ? 2u : 3u) : 0u;
}

int stride_inspect(const uint8_t* data, size_t len, stride_info_t* info) {
    if (!info) return fail(STRIDE_ERR_ARG, "null info");
    MeshParams p;
    char why[256] = {0};
    const int rc = parse_header(data, len, &p, why, sizeof(why));
    if (rc) return fail(rc, "%s", why);
    fill_info(p, len, default_config(p.n_meshlets).persistent, info);
    return STRIDE_OK;
}

int stride_open(const uint8_t* data, size_t len, stride_handle** out) {
    if (!out) return fail(STRIDE_ERR_ARG, "null output handle");
    *out = nullptr;
    MeshParams p;
    char why[256] = {0};
    int rc = parse_header(data, len, &p, why, sizeof(why));
    if (rc) return fail(rc, "%s", why);
    stride_handle* h = new stride_handle();
    cudaGetDevice(&h->device);
    h->len = len;
    cudaError_t e;
    rc = ensure_capacity(h, len, p);
    h->params = p;
    h->cfg = default_config(p.n_meshlets);
    if (rc != STRIDE_OK) {
        free_buffers(h);
        delete h;
        return rc;
    }
    if ((e = cudaMalloc(&h->d_params, sizeof(MeshParams))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_status, sizeof(Status))) != cudaSuccess ||
        (e = cudaMemcpy(h->d_blob, data, len, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(h->d_blob + len, 0, h->cap_bytes - len)) != cudaSuccess ||
        (e = cudaMemcpy(h->d_params, &h->params, sizeof(MeshParams), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(h->d_status, 0, sizeof(Status))) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming)) != cudaSuccess) {
        free_buffers(h);
        delete h;
        return cuda_fail(e, "stride_open");
    }
    *out = h;
    return STRIDE_OK;
}

int stride_reload(stride_handle* h, const uint8_t* data, size_t len, void* stream) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    MeshParams p;
    char why[256] = {0};
    int rc = parse_header(data, len, &p, why, sizeof(why));
    if (rc) return fail(rc, "%s", why);
    if ((rc = ensure_capacity(h, len, p)) != STRIDE_OK) return rc;
    h->params = p;
    h->len = len;
    if (!h->cfg_set) h->cfg = default_config(p.n_meshlets);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    const size_t pad = std::min<size_t>(h->cap_bytes - len, kBlobPad);
    // an earlier upload by parts may still be writing the arena
    if ((e = wait_upload(h, s)) != cudaSuccess) return cuda_fail(e, "stride_reload");
    h->up_parts = false;
    if (host_parts(p.n_t, p.n_meshlets) && host_link_init(h->link) == cudaSuccess) {
        // A stream large enough for a host decode by parts goes up in the
        // same parts (whole windows of meshlets, cut where the offset table
        // says the part's first meshlet starts), one event per part, on
        // the handle's upload stream after the work already queued on
        // `stream` (a decode there may still read the arena).
        uint32_t part_g[kHostParts + 1];
        host_part_groups(p.n_meshlets, part_g);
        size_t cut[kHostParts + 1];
        cut[0] = 0;
        cut[kHostParts] = len;
        for (int q = 1; q < kHostParts; q++) {
            const uint8_t* t = data + kHeaderBytes + 4ull * (32ull * part_g[q]);  // inside the table
            const uint64_t bit = (uint64_t(t[0]) << 24) | (uint64_t(t[1]) << 16) | (uint64_t(t[2]) << 8) | t[3];
            cut[q] = std::min(len, std::max(cut[q - 1], static_cast<size_t>((bit + 7) / 8)));
        }
        HostLink& L = h->link;
        if ((e = cudaEventRecord(L.before_up, s)) != cudaSuccess || (e = cudaStreamWaitEvent(L.up, L.before_up, 0)))
            return cuda_fail(e, "stride_reload");
        // the mesh record first: a copy queued on `stream` would go after
        // every part on the copy engine, and the first part's scan needs it
        if ((e = cudaMemcpyAsync(h->d_params, &h->params, sizeof(MeshParams), cudaMemcpyHostToDevice, L.up)) !=
            cudaSuccess)
            return cuda_fail(e, "stride_reload");
        for (int q = 0; q < kHostParts; q++) {
            if (cut[q + 1] > cut[q] &&
                (e = cudaMemcpyAsync(h->d_blob + cut[q], data + cut[q], cut[q + 1] - cut[q], cudaMemcpyHostToDevice,
                                     L.up)) != cudaSuccess)
                return cuda_fail(e, "stride_reload");
            if (q + 1 == kHostParts && (e = cudaMemsetAsync(h->d_blob + len, 0, pad, L.up)) != cudaSuccess)
                return cuda_fail(e, "stride_reload");
            if ((e = cudaEventRecord(L.bytes_in[q], L.up)) != cudaSuccess) return cuda_fail(e, "stride_reload");
        }
        h->up_parts = true;
    } else if ((e = cudaMemcpyAsync(h->d_blob, data, len, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemsetAsync(h->d_blob + len, 0, pad, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(h->d_params, &h->params, sizeof(MeshParams), cudaMemcpyHostToDevice, s)) !=
                   cudaSuccess) {
        return cuda_fail(e, "stride_reload");
    }
    return STRIDE_OK;
}

int stride_info(const stride_handle* h, stride_info_t* info) {
    if (!h || !info) return fail(STRIDE_ERR_ARG, "null argument");
    fill_info(h->params, h->len, h->cfg.persistent, info);
    info->shared_bytes = h->launch_smem;
    info->persistent_blocks = h->launch_grid;
    return STRIDE_OK;
}

static DecodeArgs handle_args(stride_handle* h, uint32_t* d_idx, float* d_pos, int32_t* d_codes) {
    DecodeArgs a;
    a.wait_clocks = h->wait_clocks;
    a.arena = h->d_blob;
    a.meshes = h->d_params;
    a.meshlet_mesh = nullptr;
    a.total_meshlets = h->params.n_meshlets;
    a.n_meshes = 1;
    a.descs = h->d_descs;
    a.blk_sums = h->d_blk_sums;
    a.blk_prefix = h->d_blk_prefix;
    a.walk_scratch = h->d_walk_scratch;
    a.walk_cap = h->walk_cap;
    a.status = h->d_status;
    a.idx = d_idx;
    a.pos = d_pos;
    a.codes = d_codes;
    a.wide_codes = h->params.g_bits[0] > 16 || h->params.g_bits[1] > 16 || h->params.g_bits[2] > 16;
    a.lut = h->d_lut;
    a.lut_meshes = h->d_lut_mesh;
    a.n_lut_meshes = h->n_lut;
    a.lut_max = h->lut_max;
    return a;
}

int stride_decode_timed(stride_handle* h, void* stream, uint32_t* d_idx, float* d_pos, float* kernel_ms) {
    if (!h || !d_idx || !d_pos) return fail(STRIDE_ERR_ARG, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions 4-byte aligned");
    cudaEvent_t ev[4];
    for (auto& e : ev) cudaEventCreate(&e);
    void* evp[4] = {ev[0], ev[1], ev[2], ev[3]};
    int rc = wait_upload(h, static_cast<cudaStream_t>(stream)) == cudaSuccess
                 ? enqueue_decode(handle_args(h, d_idx, d_pos, nullptr), h->cfg, stream, evp)
                 : STRIDE_ERR_CUDA;
    if (rc == STRIDE_OK) {
        last_launch(&h->launch_smem, &h->launch_grid);
        cudaEventRecord(h->done, static_cast<cudaStream_t>(stream));
        h->launched = true;
        cudaError_t e = cudaEventSynchronize(ev[3]);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "stride_decode_timed");
        } else if (kernel_ms) {
            for (int i = 0; i < 3; i++) cudaEventElapsedTime(&kernel_ms[i], ev[i], ev[i + 1]);
        }
    } else {
        rc = fail(rc, "decode launch failed");
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

int stride_decode(stride_handle* h, void* stream, uint32_t* d_idx, float* d_pos, int32_t* d_codes) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    if ((!d_idx && h->params.n_t) || (!d_pos && h->params.n_v)) return fail(STRIDE_ERR_ARG, "null output pointer");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u) ||
        (reinterpret_cast<uintptr_t>(d_codes) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions and codes 4-byte aligned");
    if (wait_upload(h, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return fail(STRIDE_ERR_CUDA, "decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    const int rc = enqueue_decode(handle_args(h, d_idx, d_pos, d_codes), h->cfg, stream);
    if (rc) return fail(rc, "decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    last_launch(&h->launch_smem, &h->launch_grid);
    cudaError_t e = cudaEventRecord(h->done, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    h->launched = true;
    return STRIDE_OK;
}

int stride_status(stride_handle* h, int wait, uint32_t* bad_meshlet) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    if (!h->launched) return STRIDE_OK;
    cudaError_t e = wait ? cudaEventSynchronize(h->done) : cudaEventQuery(h->done);
    if (e == cudaErrorNotReady) return STRIDE_ERR_BUSY;
    if (e != cudaSuccess) return cuda_fail(e, "decode");
    Status st;
    if ((e = cudaMemcpy(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(status)");
    uint32_t bad = 0;
    const int rc = status_to_code(st, &bad);
    if (bad_meshlet) *bad_meshlet = bad;
    if (rc) return fail(rc, "%s (meshlet %u)", status_message(rc), bad);
    return STRIDE_OK;
}

int stride_side_table(stride_handle* h, void* stream, uint64_t* d_resid_bit, uint16_t* d_sub_offs) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    const uint32_t n = h->params.n_meshlets;
    if (n && (!d_resid_bit || !d_sub_offs)) return fail(STRIDE_ERR_ARG, "null output pointer");
    if (!h->launched) return fail(STRIDE_ERR_ARG, "no decode yet");
    const int rc = stride_status(h, 1, nullptr);
    if (rc) return rc;
    const int r2 = enqueue_side_table(h->d_descs, n, reinterpret_cast<unsigned long long*>(d_resid_bit), d_sub_offs,
                                      stream);
    return r2 ? fail(r2, "side table launch failed") : STRIDE_OK;
}

int stride_meshlet_ranges(stride_handle* h, void* stream, uint64_t* d_v_first, uint64_t* d_t_first) {
    if (!h || !d_v_first || !d_t_first) return fail(STRIDE_ERR_ARG, "null argument");
    if (!h->launched) return fail(STRIDE_ERR_ARG, "no decode yet");
    const int rc = stride_status(h, 1, nullptr);
    if (rc) return rc;
    const uint32_t n = h->params.n_meshlets;
    if (n == 0u) {
        const uint64_t z[1] = {0};
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (cudaMemcpyAsync(d_v_first, z, 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(d_t_first, z, 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return cuda_fail(cudaGetLastError(), "meshlet ranges");
        return STRIDE_OK;
    }
    const int r2 = enqueue_meshlet_ranges(h->d_descs, h->d_blk_prefix, n,
                                          reinterpret_cast<unsigned long long*>(d_v_first),
                                          reinterpret_cast<unsigned long long*>(d_t_first), stream);
    return r2 ? fail(r2, "meshlet ranges launch failed") : STRIDE_OK;
}

int stride_meshlet_bounds(stride_handle* h, void* stream, const float* d_pos, float* d_bounds) {
    if (!h || (!d_pos && h->params.n_v) || (!d_bounds && h->params.n_meshlets)) return fail(STRIDE_ERR_ARG, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_pos) & 3u) || (reinterpret_cast<uintptr_t>(d_bounds) & 3u))
        return fail(STRIDE_ERR_ARG, "positions and bounds must be 4-byte aligned");
    if (!h->launched) return fail(STRIDE_ERR_ARG, "no decode yet");
    const int rc = stride_status(h, 1, nullptr);
    if (rc) return rc;
    const int r2 = enqueue_meshlet_bounds(h->d_descs, h->d_blk_prefix, h->params.n_meshlets, d_pos, d_bounds, stream);
    return r2 ? fail(r2, "meshlet bounds launch failed") : STRIDE_OK;
}

int stride_cull_meshlets(const float* d_bounds, uint32_t n, const float* planes, void* stream, uint32_t* d_visible,
                         uint32_t* d_count) {
    if (!planes || !d_count || (n && (!d_bounds || !d_visible))) return fail(STRIDE_ERR_ARG, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_bounds) & 3u) || (reinterpret_cast<uintptr_t>(d_visible) & 3u) ||
        (reinterpret_cast<uintptr_t>(d_count) & 3u))
        return fail(STRIDE_ERR_ARG, "bounds, visibility and count must be 4-byte aligned");
    Planes pl;
    for (int i = 0; i < 24; i++) pl.p[i] = planes[i];
    const int r2 = enqueue_cull(d_bounds, n, pl, d_visible, d_count, stream);
    return r2 ? fail(r2, "cull launch failed") : STRIDE_OK;
}

int stride_decode_host(stride_handle* h, void* stream, uint32_t* h_idx, float* h_pos) {
    if (!h || (!h_idx && h->params.n_t) || (!h_pos && h->params.n_v)) return fail(STRIDE_ERR_ARG, "null argument");
    cudaError_t e;
    if (h->params.n_v > h->cap_v) {
        cudaFree(h->d_pos);
        h->d_pos = nullptr;
        if ((e = cudaMalloc(&h->d_pos, 12 * h->params.n_v)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(pos)");
        h->cap_v = h->params.n_v;
    }
    if (h->params.n_t > h->cap_t) {
        cudaFree(h->d_idx);
        h->d_idx = nullptr;
        if ((e = cudaMalloc(&h->d_idx, 12 * h->params.n_t)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(idx)");
        h->cap_t = h->params.n_t;
    }
    uint32_t bad = 0;
    bool ran = false;
    // after a reload by parts, each part of the decode starts when its
    // bytes are in.  With a valid offset table a part's meshlets lie inside
    // the bytes up to its cut; a table that decreases is rejected by the
    // scan, whatever the bytes not yet in hold (which of its faults the
    // error names can then differ from a decode after the whole upload)
    const cudaEvent_t* bytes_in = h->up_parts ? h->link.bytes_in : nullptr;
    const int rc = decode_to_host(h->link, handle_args(h, h->d_idx, h->d_pos, nullptr), h->cfg, stream,
                                  h->params.n_t, h->params.n_v, h_idx, h_pos, bytes_in, &bad, &ran);
    if (!ran) return rc;
    h->launched = true;  // later status queries see this decode
    cudaEventRecord(h->done, static_cast<cudaStream_t>(stream));
    return rc ? fail(rc, "%s (meshlet %u)", status_message(rc), bad) : STRIDE_OK;
}

int stride_set_wait_limit(stride_handle* h, uint64_t clocks) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    h->wait_clocks = static_cast<long long>(clocks > (1ull << 62) ? (1ull << 62) : clocks);
    return STRIDE_OK;
}

int stride_set_config(stride_handle* h, const stride_launch_cfg* c) {
    if (!h || !c) return fail(STRIDE_ERR_ARG, "null argument");
    LaunchCfg cfg;
    cfg.warps_per_cta = c->warps_per_cta;
    cfg.persistent = c->persistent;
    cfg.ctas_per_sm = c->ctas_per_sm;
    cfg.stage_bytes = c->stage_bytes;
    cfg.code_bytes = c->code_bytes;
    const bool wide = h->params.g_bits[0] > 16 || h->params.g_bits[1] > 16 || h->params.g_bits[2] > 16;
    if (check_config(cfg, wide)) return fail(STRIDE_ERR_ARG, "launch configuration not launchable");
    h->cfg = cfg;
    h->cfg_set = true;
    return STRIDE_OK;
}

void stride_close(stride_handle* h) {
    if (!h) return;
    if (h->launched) cudaEventSynchronize(h->done);
    if (h->done) cudaEventDestroy(h->done);
    host_link_free(h->link);
    free_buffers(h);
    delete h;
}

}  // extern "C"
