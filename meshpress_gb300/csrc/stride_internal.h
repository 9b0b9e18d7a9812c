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

// The end of a part's windows: the last window's block prefix and sums
// (their sum is the next part's first rows).
struct PartEnd {
    BlockPrefix prefix;
    uint4 sums;
};

// Copy streams, events and pinned scratch of such decodes (one per handle
// or batch; created on first use).
struct HostLink {
    cudaStream_t copy[2] = {nullptr, nullptr};
    cudaStream_t up = nullptr;  // a handle's stream upload by parts
    cudaEvent_t conn_done = nullptr, vert_done = nullptr, done = nullptr, copied[2] = {nullptr, nullptr};
    cudaEvent_t part_done[kHostParts] = {}, scan_done[kHostParts] = {}, end_in[kHostParts] = {};
    cudaEvent_t bytes_in[kHostParts] = {}, before_up = nullptr;
    PartEnd* h_end = nullptr;   // pinned, kHostParts entries
    Status* h_status = nullptr; // pinned: the decode's status, copied out with the outputs
};
cudaError_t host_link_init(HostLink& L);
void host_link_free(HostLink& L);

// Whether a decode of this many triangles and groups goes by parts.
inline bool host_parts(uint64_t n_t, uint32_t total_meshlets) {
    const uint32_t n_win = ((total_meshlets + 31u) / 32u + 7u) / 8u;
    return n_t >= kHostPartTris && n_win >= static_cast<uint32_t>(kHostParts);
}
// Group bounds of the parts (kHostParts + 1 entries): whole windows.
void host_part_groups(uint32_t total_meshlets, uint32_t* part_g);

// Decode `a` (outputs at a.idx / a.pos, n_t and n_v rows) on `stream` and
// copy both to h_idx / h_pos; returns when they are there.  `bytes_in`,
// when given (kHostParts events), says when each part's bytes are in the
// arena (a decode by parts then starts each part when its bytes are).
// *ran says whether the decode ran to its end: then the result is its
// status code (STRIDE_OK or the error, the failing meshlet in *bad, the
// message left to the caller); otherwise a launch or copy failure, message
// recorded.
int decode_to_host(HostLink& L, const DecodeArgs& a, LaunchCfg cfg, void* stream, uint64_t n_t, uint64_t n_v,
                   uint32_t* h_idx, float* h_pos, const cudaEvent_t* bytes_in, uint32_t* bad, bool* ran);

}  // namespace stride
