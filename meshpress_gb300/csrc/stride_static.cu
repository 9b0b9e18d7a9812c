// Decode entry point that performs no device allocation.
//
// Who needs it: code that runs where cudaMalloc/cudaFree are off limits --
// a renderer's per-frame streaming loop (both calls synchronise the whole
// device and would stall every other stream mid-frame), a plugin living
// inside a host application that owns all device memory through its own
// pool, or a service that must not grow its footprint after start-up.  Such
// callers allocate their output buffers once from their own pool and then
// decode any stream that fits the fixed scratch below, with zero calls into
// the CUDA allocator.
//
// The scratch is one file-scope __device__ array of kStaticScratchBytes.
// Every GPU that loads this library reserves it until the process exits.
// All calls share it and it keeps the previous call's contents; the decode
// clears the only part that must start at zero (the status word) itself.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on this array and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "stride_common.cuh"
#include "stride_gb300.h"
#include "stride_internal.h"

namespace stride {
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB per device

__device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
uint8_t* g_static_addr[64] = {nullptr};

// Device address of the array on the current device.  The host-side symbol
// is only a stand-in for the device object, so the address must come from
// cudaGetSymbolAddress with the device current; it is looked up once per
// device and cached.  That first lookup is also where the runtime loads the
// library's device code on the device (lazy module loading) and so reserves
// the array's memory.  A cached address is checked on every call: after a
// cudaDeviceReset the device's context -- and the array with it -- is
// gone, and the address is looked up again in the new context.
int static_scratch(uint8_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(STRIDE_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_addr[dev]) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, g_static_addr[dev]) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
            at.device != dev) {
            cudaGetLastError();           // clear the query's error, if any
            g_static_addr[dev] = nullptr;  // the context was reset: look the address up again
        }
    }
    if (!g_static_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_static_addr[dev] = static_cast<uint8_t*>(p);
    }
    *out = g_static_addr[dev];
    return STRIDE_OK;
}

size_t up256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

struct StaticLayout {
    size_t blob, params, lut_list, descs, sums, prefix, walk, lut, status, total;
};

StaticLayout plan(size_t len, const MeshParams& p) {
    StaticLayout L;
    size_t o = 0;
    L.blob = o;
    o += up256(blob_alloc_bytes(len));
    L.params = o;
    o += up256(sizeof(MeshParams));
    L.lut_list = o;
    o += up256(sizeof(uint32_t));
    L.descs = o;
    o += up256(sizeof(MeshletDesc) * p.n_meshlets);
    L.sums = o;
    o += up256(sizeof(uint4) * scan_blocks(p.n_meshlets));
    L.prefix = o;
    o += up256(sizeof(BlockPrefix) * scan_blocks(p.n_meshlets));
    L.walk = o;
    o += up256(4ull * walk_scratch_words(p.n_v, p.n_meshlets));
    L.lut = o;
    o += up256(4ull * lut_entries(p));
    L.status = o;
    o += up256(sizeof(Status));
    L.total = o;
    return L;
}

}  // namespace
}  // namespace stride

using namespace stride;

extern "C" int stride_decode_static(const uint8_t* data, size_t len, void* stream, uint32_t* d_idx, float* d_pos) {
    MeshParams p;
    char why[256] = {0};
    int rc = parse_header(data, len, &p, why, sizeof(why));
    if (rc) return fail(rc, "%s", why);
    uint32_t n_lut = 0, lut_max = 0;
    plan_luts(&p, 1, nullptr, 1, &n_lut, &lut_max);
    const StaticLayout L = plan(len, p);
    if (L.total > kStaticScratchBytes)
        return fail(STRIDE_ERR_NOMEM,
                    "stream needs %zu bytes of decode scratch; the allocation-free entry point has a fixed "
                    "%zu-byte scratch (about 10 million triangles of a typical mesh); use stride_open/stride_decode instead",
                    L.total, kStaticScratchBytes);
    if ((!d_idx && p.n_t) || (!d_pos && p.n_v)) return fail(STRIDE_ERR_ARG, "null output pointer");
    if ((reinterpret_cast<uintptr_t>(d_idx) & 15u) || (reinterpret_cast<uintptr_t>(d_pos) & 3u))
        return fail(STRIDE_ERR_ARG, "index output must be 16-byte aligned, positions 4-byte aligned");
    uint8_t* base = nullptr;
    if ((rc = static_scratch(&base)) != STRIDE_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    // a pageable source is staged by the runtime before these calls return,
    // so `data` and `p` may go away afterwards
    if ((e = cudaMemcpyAsync(base + L.blob, data, len, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(base + L.blob + len, 0, kBlobPad, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(base + L.params, &p, sizeof(p), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(base + L.lut_list, 0, sizeof(uint32_t), s)) != cudaSuccess)
        return cuda_fail(e, "stride_decode_static upload");
    DecodeArgs a;
    a.arena = base + L.blob;
    a.meshes = reinterpret_cast<const MeshParams*>(base + L.params);
    a.meshlet_mesh = nullptr;
    a.total_meshlets = p.n_meshlets;
    a.n_meshes = 1;
    a.descs = reinterpret_cast<MeshletDesc*>(base + L.descs);
    a.blk_sums = reinterpret_cast<uint4*>(base + L.sums);
    a.blk_prefix = reinterpret_cast<BlockPrefix*>(base + L.prefix);
    a.walk_scratch = reinterpret_cast<uint32_t*>(base + L.walk);
    a.walk_cap = walk_scratch_words(p.n_v, p.n_meshlets);
    a.status = reinterpret_cast<Status*>(base + L.status);  // zeroed by enqueue_decode
    a.idx = d_idx;
    a.pos = d_pos;
    a.codes = nullptr;
    a.wide_codes = p.g_bits[0] > 16 || p.g_bits[1] > 16 || p.g_bits[2] > 16;
    a.lut = reinterpret_cast<float*>(base + L.lut);
    a.lut_meshes = reinterpret_cast<const uint32_t*>(base + L.lut_list);
    a.n_lut_meshes = n_lut;
    a.lut_max = lut_max;
    // always the fused shape: one set of kernels, loaded by the first call
    // (a shape used for the first time later would load its kernels then)
    LaunchCfg cfg;
    if (a.wide_codes) cfg.code_bytes = kMaxLocal * 4u > cfg.code_bytes ? kMaxLocal * 4u : cfg.code_bytes;
    rc = enqueue_decode(a, cfg, stream);
    if (rc) return fail(rc, "decode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "stride_decode_static");
    Status st;
    if ((e = cudaMemcpy(&st, a.status, sizeof(st), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(status)");
    uint32_t bad = 0;
    rc = status_to_code(st, &bad);
    if (rc) return fail(rc, "%s (meshlet %u)", status_message(rc), bad);
    return STRIDE_OK;
}
