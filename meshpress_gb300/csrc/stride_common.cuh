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
constexpr int kScanThreads = 256;  // meshlets per scan block
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
    uint32_t has_lut;        // positions come from a per-code table (see lut_entries)
    unsigned long long lut_off;  // first float of the mesh's tables in DecodeArgs::lut
    stride_dequant_axis dq[3];
};

// Dequantisation tables: a mesh with at least as many duplicated vertices as
// half its code space (all axes together) gets one float per code and axis,
// evaluated once per decode by extra blocks of the scan launch; axis d's table follows those of
// the axes before it.  Only for codes of up to kLutMaxBits bits.
constexpr uint32_t kLutMaxBits = 16;

inline unsigned long long lut_entries(const MeshParams& p) {
    unsigned long long e = 0;
    for (int d = 0; d < 3; d++) {
        if (p.g_bits[d] > kLutMaxBits) return 0;
        e += 1ull << p.g_bits[d];
    }
    return e <= 2ull * p.n_v ? e : 0;
}

// Per-meshlet record: the scan kernel writes the first part, the
// connectivity kernel the walk facts (64 bytes).
struct __align__(16) MeshletDesc {
    uint32_t start_bit;    // meshlet header (offset table entry)
    uint32_t end_bit;      // next meshlet's offset (or the stream end)
    uint32_t counts0;      // n_local | n_tris << 16
    uint32_t n_strips;
    uint32_t v_pref;       // exclusive prefixes inside the scan block:
    uint32_t t_pref;       //   n_local, n_tris,
    uint32_t wp_pref;      //   n_local rounded up to 4 (walk scratch)
    uint32_t pad0;
    uint32_t anchor_bit;   // end of connectivity = anchor codes
    uint32_t walk;         // n_kind0 | n_walk << 16
    uint32_t slot_meshlet; // meshlet decoded at slot i (= this record's index)
    uint16_t sub_offs[5];  // vertex kernel: starts of dy dz px py pz after anchor_bit (0xFFFF: too far)
    uint16_t pad16;
    uint32_t pad[2];
};
static_assert(sizeof(MeshletDesc) == 64, "meshlet records are four 16-byte loads");

struct BlockPrefix {
    unsigned long long v, t, wp, pad;
};

struct Status {
    unsigned long long err;  // ((uint64)code << 32) | meshlet; first error wins
    unsigned int ticket;     // scan blocks finished (the last one scans block sums)
    unsigned int work_conn;  // persistent work counters
    unsigned int work_vert;
    unsigned int done_tail;  // entries in the completion list (fused kernel)
    unsigned int pad[2];
};

struct LaunchCfg {
    int warps_per_cta = 4;
    int persistent = 2;  // 0: one vertex CTA per group, 1: persistent vertex grid, 2: one fused kernel,
                         // 3: group kernel (one warp per group, every phase; warps_per_cta 1 or 2)
    int ctas_per_sm = 0;
    uint32_t stage_bytes = 16 * 1024;  // per-warp payload staging (vertex kernel: half)
    uint32_t code_bytes = 12 * 1024;   // per-warp integer code plane (vertex kernel)
};

struct DecodeArgs {
    const uint8_t* arena;            // device: all streams
    const MeshParams* meshes;        // device
    const uint32_t* meshlet_mesh;    // device, nullptr when there is one mesh
    uint32_t total_meshlets;
    uint32_t n_meshes;
    MeshletDesc* descs;              // device scratch, total_meshlets
    uint4* blk_sums;                 // device scratch, scan blocks
    BlockPrefix* blk_prefix;         // device scratch, scan blocks
    uint32_t* walk_scratch;          // walk entries, 4-aligned per meshlet
    unsigned long long walk_cap;     // words in walk_scratch
    Status* status;                  // device
    uint32_t* idx;                   // device outputs (idx 16-byte aligned)
    float* pos;
    int32_t* codes;                  // optional
    bool wide_codes;                 // some mesh has g_bits > 16
    float* lut;                      // dequantisation tables (meshes with has_lut)
    const uint32_t* lut_meshes;      // device: indices of those meshes
    uint32_t n_lut_meshes;
    uint32_t lut_max;                // largest table set (floats) of one mesh
    // SM clocks a device wait (a bulk copy's mbarrier, the fused kernel's
    // completion list) spins before it gives up with STRIDE_ERR_TIMEOUT
    // (about a second by default; 0 gives up at the first unsuccessful check)
    long long wait_clocks = 1ll << 31;
    // groups [conn_g0, conn_g1) of the connectivity kernel (two-kernel
    // shape): whole 256-meshlet windows, i.e. multiples of eight; the
    // defaults take every group
    uint32_t conn_g0 = 0u, conn_g1 = 0xFFFFFFFFu;
};

// Host: assigns table offsets (has_lut, lut_off) to the meshes that get
// tables; returns the floats needed, fills `meshes` (at most max_meshes
// indices) and the largest per-mesh size.
unsigned long long plan_luts(MeshParams* p, uint32_t n, uint32_t* meshes, uint32_t max_meshes, uint32_t* n_lut,
                             uint32_t* lut_max);

inline uint32_t scan_blocks(uint32_t total_meshlets) {
    return (total_meshlets + kScanThreads - 1) / kScanThreads;
}

// Walk scratch words needed for a stream set with these totals.
inline unsigned long long walk_scratch_words(unsigned long long n_v, unsigned long long meshlets) {
    return n_v + 3ull * meshlets + 4ull;
}

// Host-side header parse + kernel parameters; returns 0 or a STRIDE_ERR_*.
int parse_header(const uint8_t* data, size_t len, MeshParams* p, char* why, size_t why_len);

// Enqueue the scan kernel and then the fused kernel (cfg.persistent == 2) or
// the connectivity and vertex kernels for `a` on `stream`.  When `ev` is
// non-null, its non-null entries of four are recorded: before the scan
// kernel, after it, after the connectivity (or fused) kernel and after the
// vertex kernel (right after the fused one).
int enqueue_decode(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* const* ev = nullptr);
// The two-kernel decode in parts of whole windows, enqueued on `stream`
// as: enqueue_parts_begin; per part (groups [g0, g1), `first` for the
// first), enqueue_part -- after `bytes_in` (when given: the part's bytes
// are in the arena), the scan of its windows (then `scan_done`: their
// block prefixes are final) and its connectivity (then `conn_done`);
// enqueue_parts_end -- the vertex kernel over every group (then
// `vert_done`).  Null events are skipped.
int enqueue_parts_begin(const DecodeArgs& a, const LaunchCfg& cfg, void* stream);
int enqueue_part(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, uint32_t g0, uint32_t g1, bool first,
                 void* bytes_in, void* scan_done, void* conn_done);
int enqueue_parts_end(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* vert_done);
// The launch shape a decode of this many meshlets takes unless one is set.
LaunchCfg default_config(uint32_t total_meshlets);

// Meshlet-native outputs of a finished decode: each meshlet's first vertex
// and triangle row (n + 1 entries, the last the totals); the bounds (min
// xyz, max xyz) of its rows of `pos`; frustum culling of such bounds into a
// visibility bit per meshlet and a visible count.
struct Planes {
    float p[24];  // six planes (a, b, c, d): inside where a x + b y + c z + d >= 0
};
int enqueue_meshlet_ranges(const MeshletDesc* descs, const BlockPrefix* bp, uint32_t n, unsigned long long* v_first,
                           unsigned long long* t_first, void* stream);
int enqueue_meshlet_bounds(const MeshletDesc* descs, const BlockPrefix* bp, uint32_t n, const float* pos,
                           float* bounds, void* stream);
int enqueue_cull(const float* bounds, uint32_t n, const Planes& planes, uint32_t* visible, uint32_t* count,
                 void* stream);

// Gathers the side table of a finished decode from its meshlet records:
// per meshlet the stream bit of its anchor and the five substream starts
// relative to it.
int enqueue_side_table(const MeshletDesc* descs, uint32_t n, unsigned long long* resid_bit, uint16_t* sub_offs,
                       void* stream);

// Geometry of the decode's main kernel (the fused, group or vertex kernel)
// as last launched by this host thread: dynamic shared memory per CTA and
// CTAs in the grid (the reference class exposes the same two numbers as
// _shared_bytes and _persistent_blocks, utils/paradelta_v5_cuda.py:656-683).
void note_launch(uint32_t smem_bytes, uint32_t grid);
void last_launch(uint32_t* smem_bytes, uint32_t* grid);

// The group kernel (stride_group.cu): launch for `a` on `stream`, and its
// shared memory per CTA.
cudaError_t launch_group(const DecodeArgs& a, const LaunchCfg& cfg, void* stream);
size_t group_smem_bytes(const LaunchCfg& cfg);

// STRIDE_OK when `cfg` is a launchable shape.
int check_config(const LaunchCfg& cfg, bool wide);

// Shared memory one CTA of each kernel needs.
size_t conn_smem_bytes(const LaunchCfg& cfg);
size_t vert_smem_bytes(const LaunchCfg& cfg);

int device_sm_count();

}  // namespace stride
