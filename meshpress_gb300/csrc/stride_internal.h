// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <string>

#include "stride_common.cuh"

namespace stride {

extern thread_local std::string g_last_error;

// Record a message for stride_last_error_message() and return `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// Device bytes reserved for a stream of `len` bytes (256-aligned, zero pad).
size_t blob_alloc_bytes(size_t len);

// Device Status word -> STRIDE_OK / STRIDE_ERR_*.
int status_to_code(const Status& st, uint32_t* bad_meshlet);
const char* status_message(int code);

// Decodes whose outputs go to host memory.  The host link (about 190 GB/s
// each way on a GB300) is their bound, so the decode takes the two-kernel
// shape, whose connectivity ends first, and the triangles go out while the
// vertex kernel runs.  From kHostPartTris triangles the connectivity runs
// as kHostParts launches of whole windows and each part's triangles go out
// as soon as it ends (a part's connectivity takes less time than the copy
// of its triangles).
constexpr int kHostParts = 4;
constexpr uint64_t kHostPartTris = 3ull << 20;

// Copy streams, events and pinned scratch of such decodes (one per handle
// or batch; created on first use).
struct HostLink {
    cudaStream_t copy[2] = {nullptr, nullptr};
    cudaEvent_t conn_done = nullptr, vert_done = nullptr, scan_done = nullptr, prefix_in = nullptr, done = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, part_done[kHostParts] = {};
    BlockPrefix* h_prefix = nullptr;  // the scan's block prefixes
    uint32_t prefix_cap = 0;
    Status* h_status = nullptr;       // the decode's status, copied out with the outputs
};
void host_link_free(HostLink& L);

// Decode `a` (outputs at a.idx / a.pos, n_t and n_v rows) on `stream` and
// copy both to h_idx / h_pos; returns when they are there.  *ran says
// whether the decode ran to its end: then the result is its status code
// (STRIDE_OK or the error, the failing meshlet in *bad, the message left
// to the caller); otherwise a launch or copy failure, message recorded.
int decode_to_host(HostLink& L, const DecodeArgs& a, LaunchCfg cfg, void* stream, uint64_t n_t, uint64_t n_v,
                   uint32_t* h_idx, float* h_pos, uint32_t* bad, bool* ran);

}  // namespace stride
