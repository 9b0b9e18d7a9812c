// Shared definitions of the STRIDE (DPR4 v3) GPU decoder.
//
// Format facts (reference file:line in parentheses):
//   * every field is MSB-first, multi-byte fields big-endian
//     (utils/bit_codec.py:1-9);
//   * 86-byte global header, then a u32 table of absolute meshlet bit offsets
//     (encoder/paradelta_v5_dup.py:412-447);
//   * per meshlet: n_local, n_tris, n_strips (u16), strips of FIFO/raw
//     tokens, anchor, 6 (tag, k) pairs, then the residual substreams
//     dx, dy, dz, px, py, pz (paradelta_v5_dup.py:239-313, 507-579).
#pragma once

#include <cstdint>

#include "stride_dequant.h"

namespace stride {

constexpr uint32_t kMagic = 0x44505234u;
constexpr uint32_t kVersion = 3;
constexpr uint32_t kHeaderBytes = 86;
constexpr int kMaxLocal = 256;   // local vertices per meshlet handled on the GPU
constexpr int kMaxTris = 256;    // triangles per meshlet handled on the GPU
constexpr int kFifo = 16;        // REUSE_BUF_SIZE (encoder/paradelta_codec.py:104)
constexpr int kReuseBits = 5;    // _REUSE_BITS (encoder/paradelta_codec.py:128)
constexpr int kMaxResidK = 24;   // largest residual k this decoder accepts
constexpr int kMaxGBits = 24;    // largest per-axis code width this decoder accepts
constexpr int kScanThreads = 256;  // meshlets per parse block
constexpr int kRing = 32;          // triangles buffered per lane between flushes
constexpr int kRingStride = kRing + 1;
constexpr int kBlobPad = 64;       // zero bytes after every device copy of a stream

// Internal status codes (negated public STRIDE_ERR_* values).
constexpr int kErrOffset = 5;
constexpr int kErrCorrupt = 6;
constexpr int kErrUnsupported = 7;
constexpr int kErrTimeout = 9;

// One encoded mesh as the kernels see it.
struct MeshParams {
    uint64_t blob_off;       // byte offset of the stream inside the arena (256-aligned)
    uint64_t nbits;          // 8 * stream length (< 2^32)
    uint64_t v_offset;       // first output vertex of this mesh
    uint64_t t_offset;       // first output triangle of this mesh
    uint64_t n_v;            // header n_v_total (output extent)
    uint64_t n_t;            // header n_t
    uint32_t n_meshlets;
    uint32_t meshlet_begin;  // global index of the mesh's first meshlet
    uint32_t body_bit;       // first bit after the offset table
    uint32_t anchor_bits;    // g_bits[0] + g_bits[1] + g_bits[2]
    uint32_t g_bits[3];
    uint32_t code_max[3];    // 2^g_bits - 1
    int32_t pred_n[9];       // IRLP numerators, row = axis
    int32_t pred_k[3];
    int32_t pred_half[3];    // 2^(K-1), or 0 when K == 0
    uint32_t pad;
    stride_dequant_axis dq[3];
};

// Per-meshlet decode plan written by the parse kernel (64 bytes).
struct __align__(16) MeshletDesc {
    uint32_t conn_bit;     // first strip header
    uint32_t anchor_bit;   // anchor codes (end of connectivity)
    uint32_t res_bit[6];   // starts of dx, dy, dz, px, py, pz
    uint32_t counts0;      // n_local | n_tris << 16
    uint32_t counts1;      // n_strips | n_delta << 16
    uint32_t counts2;      // n_para
    uint32_t tk_delta;     // 3 x 8 bits: 0x80 = Exp-Golomb, low 6 bits = k
    uint32_t tk_para;
    uint32_t v_pref;       // exclusive prefix of n_local inside the parse block
    uint32_t t_pref;       // exclusive prefix of n_tris inside the parse block
    uint32_t end_bit;      // first bit after the meshlet
};

struct Status {
    unsigned long long err;  // ((uint64)code << 32) | meshlet; first error wins
    unsigned int ticket;     // parse blocks finished (last one scans block sums)
    unsigned int work;       // persistent decode work counter
};

struct LaunchCfg {
    int warps_per_cta = 1;
    int persistent = 0;
    int ctas_per_sm = 0;
    uint32_t stage_bytes = 20 * 1024;  // per-warp payload staging
    uint32_t code_bytes = 40 * 1024;   // per-warp integer code storage
};

struct DecodeArgs {
    const uint8_t* arena;            // device: all streams
    const MeshParams* meshes;        // device
    const uint32_t* meshlet_mesh;    // device, nullptr when there is one mesh
    uint32_t total_meshlets;
    uint32_t n_meshes;
    MeshletDesc* descs;              // device scratch, total_meshlets
    uint2* blk_sums;                 // device scratch, parse blocks
    ulonglong2* blk_prefix;          // device scratch, parse blocks
    Status* status;                  // device
    uint32_t* idx;                   // device outputs
    float* pos;
    int32_t* codes;                  // optional
    bool wide_codes;                 // some mesh has g_bits > 16
};

inline uint32_t parse_blocks(uint32_t total_meshlets) {
    return (total_meshlets + kScanThreads - 1) / kScanThreads;
}

// Host-side header parse + kernel parameters; returns 0 or a STRIDE_ERR_*.
int parse_header(const uint8_t* data, size_t len, MeshParams* p, char* why, size_t why_len);

// Enqueue parse + decode for `a` on `stream`.  When `ev` is non-null, the
// three events are recorded before the parse kernel, between the kernels and
// after the decode kernel.
int enqueue_decode(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* const* ev = nullptr);

// STRIDE_OK when `cfg` is a launchable shape (warps 1/2/4, budgets large
// enough for one 256-vertex meshlet, CTA shared memory <= 227 KB).
int check_config(const LaunchCfg& cfg, bool wide);

// Smem bytes one CTA of the decode kernel needs.
size_t decode_smem_bytes(const LaunchCfg& cfg, bool wide);

int device_sm_count();

}  // namespace stride
