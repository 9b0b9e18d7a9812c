// Many meshes in one launch: a device arena holding every stream, one mesh
// table, one meshlet->mesh map, and the same parse + decode kernels run over
// the concatenated meshlet space (work stealing across meshes when the
// persistent grid is selected).  CUDA-graph capture and an autotuner over
// the launch shape sit on top.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "stride_common.cuh"
#include "stride_gb300.h"
#include "stride_internal.h"

using namespace stride;

struct stride_batch {
    uint32_t n_meshes = 0;
    uint32_t total_meshlets = 0;
    uint64_t arena_bytes = 0;
    uint64_t total_v = 0, total_t = 0;
    std::vector<MeshParams> params;
    uint8_t* d_arena = nullptr;
    MeshParams* d_params = nullptr;
    uint32_t* d_meshlet_mesh = nullptr;
    MeshletDesc* d_descs = nullptr;
    uint4* d_blk_sums = nullptr;
    BlockPrefix* d_blk_prefix = nullptr;
    uint32_t* d_walk_scratch = nullptr;
    unsigned long long walk_cap = 0;
    Status* d_status = nullptr;
    float* d_lut = nullptr;
    uint32_t* d_lut_meshes = nullptr;
    uint32_t n_lut = 0, lut_max = 0;
    bool wide = false;
    LaunchCfg cfg;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
    bool launched = false;
    HostLink link;          // stride_batch_decode_to_host, and an upload by parts
    bool up_parts = false;  // the last stride_batch_upload went by parts (link.bytes_in)
};

// After an upload by parts, a decode that does not go by parts waits for
// all of it.
static cudaError_t batch_wait_upload(stride_batch* b, cudaStream_t s) {
    return b->up_parts ? cudaStreamWaitEvent(s, b->link.bytes_in[kHostParts - 1], 0) : cudaSuccess;
}

namespace stride {

// Builds the device side of a batch from host streams (also used by the
// serving engine, which owns its arena separately).
int build_mesh_table(const uint8_t* const* blobs, const size_t* lens, uint32_t n, std::vector<MeshParams>& params,
                     std::vector<uint64_t>& arena_off, uint64_t& arena_bytes, uint32_t& total_meshlets,
                     uint64_t& total_v, uint64_t& total_t, bool& wide) {
    params.resize(n);
    arena_off.resize(n);
    arena_bytes = 0;
    total_meshlets = 0;
    total_v = total_t = 0;
    wide = false;
    for (uint32_t i = 0; i < n; i++) {
        char why[256] = {0};
        const int rc = parse_header(blobs[i], lens[i], &params[i], why, sizeof(why));
        if (rc) return fail(rc, "mesh %u: %s", i, why);
        MeshParams& p = params[i];
        arena_off[i] = arena_bytes;
        p.blob_off = arena_bytes;
        arena_bytes += blob_alloc_bytes(lens[i]);
        if (static_cast<uint64_t>(total_meshlets) + p.n_meshlets > 0xFFFFFFF0ull)
            return fail(STRIDE_ERR_UNSUPPORTED, "more than 2^32 meshlets in one batch");
        p.meshlet_begin = total_meshlets;
        total_meshlets += p.n_meshlets;
        p.v_offset = total_v;
        p.t_offset = total_t;
        total_v += p.n_v;
        total_t += p.n_t;
        wide = wide || p.g_bits[0] > 16 || p.g_bits[1] > 16 || p.g_bits[2] > 16;
    }
    return STRIDE_OK;
}

}  // namespace stride

static void batch_free(stride_batch* b) {
    host_link_free(b->link);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->done) cudaEventDestroy(b->done);
    cudaFree(b->d_arena);
    cudaFree(b->d_params);
    cudaFree(b->d_meshlet_mesh);
    cudaFree(b->d_descs);
    cudaFree(b->d_blk_sums);
    cudaFree(b->d_blk_prefix);
    cudaFree(b->d_walk_scratch);
    cudaFree(b->d_status);
    cudaFree(b->d_lut);
    cudaFree(b->d_lut_meshes);
}

static DecodeArgs batch_args(const stride_batch* b, uint32_t* d_idx, float* d_pos) {
    DecodeArgs a;
    a.arena = b->d_arena;
    a.meshes = b->d_params;
    a.meshlet_mesh = b->d_meshlet_mesh;
    a.total_meshlets = b->total_meshlets;
    a.n_meshes = b->n_meshes;
    a.descs = b->d_descs;
    a.blk_sums = b->d_blk_sums;
    a.blk_prefix = b->d_blk_prefix;
    a.walk_scratch = b->d_walk_scratch;
    a.walk_cap = b->walk_cap;
    a.status = b->d_status;
    a.idx = d_idx;
    a.pos = d_pos;
    a.codes = nullptr;
    a.wide_codes = b->wide;
    a.lut = b->d_lut;
    a.lut_meshes = b->d_lut_meshes;
    a.n_lut_meshes = b->n_lut;
    a.lut_max = b->lut_max;
    return a;
}

static LaunchCfg to_cfg(const stride_launch_cfg* c) {
    LaunchCfg cfg;
    cfg.warps_per_cta = c->warps_per_cta;
    cfg.persistent = c->persistent;
    cfg.ctas_per_sm = c->ctas_per_sm;
    cfg.stage_bytes = c->stage_bytes;
    cfg.code_bytes = c->code_bytes;
    return cfg;
}

static void from_cfg(const LaunchCfg& cfg, stride_launch_cfg* c) {
    c->warps_per_cta = cfg.warps_per_cta;
    c->persistent = cfg.persistent;
    c->ctas_per_sm = cfg.ctas_per_sm;
    c->stage_bytes = cfg.stage_bytes;
    c->code_bytes = cfg.code_bytes;
}

extern "C" {

int stride_batch_create(const uint8_t* const* blobs, const size_t* lens, uint32_t n_meshes, stride_batch** out) {
    if (!out || !blobs || !lens || n_meshes == 0) return fail(STRIDE_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    stride_batch* b = new stride_batch();
    b->n_meshes = n_meshes;
    std::vector<uint64_t> off;
    uint64_t arena_bytes = 0;
    int rc = build_mesh_table(blobs, lens, n_meshes, b->params, off, arena_bytes, b->total_meshlets, b->total_v,
                              b->total_t, b->wide);
    if (rc) {
        delete b;
        return rc;
    }
    b->cfg = default_config(b->total_meshlets);
    if (b->wide) b->cfg.code_bytes = std::max<uint32_t>(b->cfg.code_bytes, kMaxLocal * 4u);
    b->arena_bytes = arena_bytes;
    b->walk_cap = walk_scratch_words(b->total_v, b->total_meshlets);
    std::vector<uint32_t> lut_meshes(n_meshes);
    const unsigned long long lut_floats =
        plan_luts(b->params.data(), n_meshes, lut_meshes.data(), n_meshes, &b->n_lut, &b->lut_max);
    std::vector<uint8_t> arena(arena_bytes, 0);
    for (uint32_t i = 0; i < n_meshes; i++) std::memcpy(arena.data() + off[i], blobs[i], lens[i]);
    std::vector<uint32_t> mm(b->total_meshlets);
    for (uint32_t i = 0; i < n_meshes; i++)
        std::fill(mm.begin() + b->params[i].meshlet_begin,
                  mm.begin() + b->params[i].meshlet_begin + b->params[i].n_meshlets, i);
    const uint32_t nb = scan_blocks(b->total_meshlets);
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_arena, arena_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&b->d_params, sizeof(MeshParams) * n_meshes)) != cudaSuccess ||
        (e = cudaMalloc(&b->d_meshlet_mesh, sizeof(uint32_t) * std::max<uint32_t>(1u, b->total_meshlets))) !=
            cudaSuccess ||
        (e = cudaMalloc(&b->d_descs, sizeof(MeshletDesc) * std::max<uint32_t>(1u, b->total_meshlets))) !=
            cudaSuccess ||
        (e = cudaMalloc(&b->d_blk_sums, sizeof(uint4) * std::max<uint32_t>(1u, nb))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_blk_prefix, sizeof(BlockPrefix) * std::max<uint32_t>(1u, nb))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_walk_scratch, 4ull * b->walk_cap)) != cudaSuccess ||
        (e = cudaMalloc(&b->d_status, sizeof(Status))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_lut, 4ull * std::max<unsigned long long>(1ull, lut_floats))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_lut_meshes, 4ull * std::max<uint32_t>(1u, b->n_lut))) != cudaSuccess ||
        (b->n_lut && (e = cudaMemcpy(b->d_lut_meshes, lut_meshes.data(), 4ull * b->n_lut,
                                     cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (e = cudaMemcpy(b->d_arena, arena.data(), arena_bytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_params, b->params.data(), sizeof(MeshParams) * n_meshes, cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(b->d_meshlet_mesh, mm.data(), sizeof(uint32_t) * b->total_meshlets,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(b->d_status, 0, sizeof(Status))) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming)) != cudaSuccess) {
        batch_free(b);
        delete b;
        return cuda_fail(e, "stride_batch_create");
    }
    *out = b;
    return STRIDE_OK;
}

int stride_batch_info(const stride_batch* b, uint64_t* n_meshlets, uint64_t* n_v, uint64_t* n_t) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if (n_meshlets) *n_meshlets = b->total_meshlets;
    if (n_v) *n_v = b->total_v;
    if (n_t) *n_t = b->total_t;
    return STRIDE_OK;
}

int stride_batch_offsets(const stride_batch* b, uint64_t* v_offset, uint64_t* t_offset) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    for (uint32_t i = 0; i < b->n_meshes; i++) {
        if (v_offset) v_offset[i] = b->params[i].v_offset;
        if (t_offset) t_offset[i] = b->params[i].t_offset;
    }
    return STRIDE_OK;
}

int stride_batch_set_config(stride_batch* b, const stride_launch_cfg* c) {
    if (!b || !c) return fail(STRIDE_ERR_ARG, "null argument");
    const LaunchCfg cfg = to_cfg(c);
    if (check_config(cfg, b->wide)) return fail(STRIDE_ERR_ARG, "launch configuration not launchable");
    b->cfg = cfg;
    return STRIDE_OK;
}

int stride_batch_get_config(const stride_batch* b, stride_launch_cfg* c) {
    if (!b || !c) return fail(STRIDE_ERR_ARG, "null argument");
    from_cfg(b->cfg, c);
    return STRIDE_OK;
}

int stride_batch_decode(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if ((!d_idx && b->total_t) || (!d_pos && b->total_v)) return fail(STRIDE_ERR_ARG, "null output pointer");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions 4-byte aligned");
    if (batch_wait_upload(b, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return fail(STRIDE_ERR_CUDA, "batch decode: %s", cudaGetErrorString(cudaGetLastError()));
    const int rc = enqueue_decode(batch_args(b, d_idx, d_pos), b->cfg, stream);
    if (rc) return fail(rc, "batch decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    cudaError_t e = cudaEventRecord(b->done, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    b->launched = true;
    return STRIDE_OK;
}

// A decode error's message, with the batch meshlet turned into mesh and
// meshlet.
static int batch_error(const stride_batch* b, int rc, uint32_t bad, uint32_t* bad_mesh, uint32_t* bad_meshlet) {
    uint32_t mesh = 0;
    for (uint32_t i = 0; i < b->n_meshes; i++)
        if (b->params[i].meshlet_begin <= bad) mesh = i;
    if (bad_mesh) *bad_mesh = mesh;
    if (bad_meshlet) *bad_meshlet = bad - b->params[mesh].meshlet_begin;
    return fail(rc, "%s (mesh %u, meshlet %u)", status_message(rc), mesh, bad - b->params[mesh].meshlet_begin);
}

int stride_batch_decode_to_host(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos, uint32_t* h_idx,
                                float* h_pos) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if ((!d_idx || !h_idx) && b->total_t) return fail(STRIDE_ERR_ARG, "null index output");
    if ((!d_pos || !h_pos) && b->total_v) return fail(STRIDE_ERR_ARG, "null position output");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions 4-byte aligned");
    uint32_t bad = 0;
    bool ran = false;
    // after an upload by parts each part of the decode starts when its bytes are in
    const int rc = decode_to_host(b->link, batch_args(b, d_idx, d_pos), b->cfg, stream, b->total_t, b->total_v,
                                  h_idx, h_pos, b->up_parts ? b->link.bytes_in : nullptr, &bad, &ran);
    if (!ran) return rc;
    b->launched = true;  // later status queries see this decode
    cudaEventRecord(b->done, static_cast<cudaStream_t>(stream));
    return rc ? batch_error(b, rc, bad, nullptr, nullptr) : STRIDE_OK;
}

int stride_batch_image(const stride_batch* b, uint64_t* blob_offsets, uint64_t* image_bytes) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if (blob_offsets)
        for (uint32_t i = 0; i < b->n_meshes; i++) blob_offsets[i] = b->params[i].blob_off;
    if (image_bytes) *image_bytes = b->arena_bytes;
    return STRIDE_OK;
}

int stride_batch_upload(stride_batch* b, void* stream, const void* image, size_t bytes) {
    if (!b || !image) return fail(STRIDE_ERR_ARG, "null argument");
    if (bytes != b->arena_bytes)
        return fail(STRIDE_ERR_ARG, "image is %zu bytes, the batch's arena %llu", bytes,
                    static_cast<unsigned long long>(b->arena_bytes));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = batch_wait_upload(b, s);  // an earlier upload by parts may still be writing
    if (e != cudaSuccess) return cuda_fail(e, "stride_batch_upload");
    b->up_parts = false;
    if (host_parts(b->total_t, b->total_meshlets) && host_link_init(b->link) == cudaSuccess) {
        // As a handle's reload: the image goes up in the parts of a host
        // decode, cut where the offset table of the mesh holding a part's
        // first meshlet puts that meshlet, one event per part, on the
        // batch's upload stream after the work already queued on `stream`.
        const uint8_t* img = static_cast<const uint8_t*>(image);
        uint32_t part_g[kHostParts + 1];
        host_part_groups(b->total_meshlets, part_g);
        size_t cut[kHostParts + 1];
        cut[0] = 0;
        cut[kHostParts] = bytes;
        for (int q = 1; q < kHostParts; q++) {
            const uint32_t m = 32u * part_g[q];
            uint32_t i = 0;  // the mesh holding meshlet m
            while (i + 1 < b->n_meshes && b->params[i + 1].meshlet_begin <= m) i++;
            const MeshParams& P = b->params[i];
            const uint8_t* t = img + P.blob_off + kHeaderBytes + 4ull * (m - P.meshlet_begin);  // its table
            const uint64_t bit = (uint64_t(t[0]) << 24) | (uint64_t(t[1]) << 16) | (uint64_t(t[2]) << 8) | t[3];
            cut[q] = std::min<size_t>(bytes, std::max<size_t>(cut[q - 1], P.blob_off + (bit + 7) / 8));
        }
        HostLink& L = b->link;
        if ((e = cudaEventRecord(L.before_up, s)) != cudaSuccess || (e = cudaStreamWaitEvent(L.up, L.before_up, 0)))
            return cuda_fail(e, "stride_batch_upload");
        for (int q = 0; q < kHostParts; q++) {
            if (cut[q + 1] > cut[q] && (e = cudaMemcpyAsync(b->d_arena + cut[q], img + cut[q], cut[q + 1] - cut[q],
                                                            cudaMemcpyHostToDevice, L.up)) != cudaSuccess)
                return cuda_fail(e, "stride_batch_upload");
            if ((e = cudaEventRecord(L.bytes_in[q], L.up)) != cudaSuccess) return cuda_fail(e, "stride_batch_upload");
        }
        b->up_parts = true;
        return STRIDE_OK;
    }
    e = cudaMemcpyAsync(b->d_arena, image, bytes, cudaMemcpyHostToDevice, s);
    return e == cudaSuccess ? STRIDE_OK : cuda_fail(e, "stride_batch_upload");
}

int stride_batch_decode_timed(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos, float* kernel_ms) {
    if (!b || !d_idx || !d_pos) return fail(STRIDE_ERR_ARG, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions 4-byte aligned");
    cudaEvent_t ev[4];
    for (auto& e : ev) cudaEventCreate(&e);
    void* evp[4] = {ev[0], ev[1], ev[2], ev[3]};
    int rc = batch_wait_upload(b, static_cast<cudaStream_t>(stream)) == cudaSuccess
                 ? enqueue_decode(batch_args(b, d_idx, d_pos), b->cfg, stream, evp)
                 : STRIDE_ERR_CUDA;
    if (rc == STRIDE_OK) {
        cudaEventRecord(b->done, static_cast<cudaStream_t>(stream));
        b->launched = true;
        const cudaError_t e = cudaEventSynchronize(ev[3]);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "stride_batch_decode_timed");
        } else if (kernel_ms) {
            for (int i = 0; i < 3; i++) cudaEventElapsedTime(&kernel_ms[i], ev[i], ev[i + 1]);
        }
    } else {
        rc = fail(rc, "batch decode launch failed");
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

int stride_batch_capture_graph(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!s) return fail(STRIDE_ERR_ARG, "graph capture needs a non-default stream");
    // one eager decode first: kernel attributes are set outside the capture
    int rc = stride_batch_decode(b, stream, d_idx, d_pos);
    if (rc) return rc;
    cudaError_t e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamBeginCapture");
    rc = enqueue_decode(batch_args(b, d_idx, d_pos), b->cfg, stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return fail(rc, "capture of the decode sequence failed");
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    b->graph = g;
    if ((e = cudaGraphInstantiate(&b->exec, g, 0)) != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return STRIDE_OK;
}

int stride_batch_launch_graph(stride_batch* b, void* stream) {
    if (!b || !b->exec) return fail(STRIDE_ERR_ARG, "no captured graph");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if ((e = batch_wait_upload(b, s)) != cudaSuccess || (e = cudaGraphLaunch(b->exec, s)) != cudaSuccess)
        return cuda_fail(e, "cudaGraphLaunch");
    if ((e = cudaEventRecord(b->done, s)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    b->launched = true;
    return STRIDE_OK;
}

int stride_batch_autotune(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos, int iters,
                          stride_launch_cfg* best, float* best_ms) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if (iters < 1) iters = 3;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (batch_wait_upload(b, s) != cudaSuccess) return fail(STRIDE_ERR_CUDA, "autotune: upload");
    std::vector<LaunchCfg> cands;
    // the vertex kernel stages half of stage_bytes
    const uint32_t stage_opts[] = {8u * 1024u, 10u * 1024u, 12u * 1024u, 16u * 1024u, 24u * 1024u};
    // code plane per warp: 2 bytes per vertex (4 above 16-bit codes), 32
    // meshlets of up to 256 vertices fill 16 KiB; 10.5 KiB planes with a
    // 5 KiB stage are the largest that fit six vertex CTAs on an SM
    const uint32_t code_opts[] = {6u * 1024u, 8u * 1024u, 10u * 1024u, 10752u, 11u * 1024u, 12u * 1024u, 16u * 1024u};
    for (int w : {1, 2, 4})
        for (uint32_t st : stage_opts)
            for (uint32_t cb : code_opts)
                for (int pers : {0, 1, 2}) {
                    LaunchCfg c;
                    c.warps_per_cta = w;
                    c.stage_bytes = st;
                    c.code_bytes = b->wide ? 2u * cb : cb;
                    c.persistent = pers;
                    c.ctas_per_sm = 0;  // persistent grid sized by the occupancy calculator
                    if (check_config(c, b->wide)) continue;
                    cands.push_back(c);
                }
    for (int w : {1, 2}) {  // the group kernel: no stage or plane sizes to choose
        LaunchCfg c;
        c.warps_per_cta = w;
        c.persistent = 3;
        c.ctas_per_sm = 0;
        cands.push_back(c);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_t = 1e30f;
    LaunchCfg best_c = b->cfg;
    const LaunchCfg saved = b->cfg;
    for (const LaunchCfg& c : cands) {
        b->cfg = c;
        if (stride_batch_decode(b, stream, d_idx, d_pos)) continue;  // warm-up
        cudaEventRecord(e0, s);
        bool ok = true;
        for (int i = 0; i < iters && ok; i++) ok = stride_batch_decode(b, stream, d_idx, d_pos) == STRIDE_OK;
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess || !ok) {
            cudaGetLastError();
            continue;
        }
        uint32_t bm = 0, bl = 0;
        if (stride_batch_status(b, 1, &bm, &bl) != STRIDE_OK) {
            b->cfg = saved;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return STRIDE_ERR_CORRUPT;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= static_cast<float>(iters);
        if (ms < best_t) {
            best_t = ms;
            best_c = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = best_c;
    if (best) from_cfg(best_c, best);
    if (best_ms) *best_ms = best_t;
    return best_t < 1e29f ? STRIDE_OK : fail(STRIDE_ERR_CUDA, "no launch configuration ran");
}

int stride_batch_status(stride_batch* b, int wait, uint32_t* bad_mesh, uint32_t* bad_meshlet) {
    if (!b) return fail(STRIDE_ERR_ARG, "null batch");
    if (!b->launched) return STRIDE_OK;
    cudaError_t e = wait ? cudaEventSynchronize(b->done) : cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) return STRIDE_ERR_BUSY;
    if (e != cudaSuccess) return cuda_fail(e, "batch decode");
    Status st;
    if ((e = cudaMemcpy(&st, b->d_status, sizeof(st), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(status)");
    uint32_t bad = 0;
    const int rc = status_to_code(st, &bad);
    return rc ? batch_error(b, rc, bad, bad_mesh, bad_meshlet) : STRIDE_OK;
}

void stride_batch_destroy(stride_batch* b) {
    if (!b) return;
    if (b->launched) cudaEventSynchronize(b->done);
    batch_free(b);
    delete b;
}

}  // extern "C"
