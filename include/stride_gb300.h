/*
 * stride_gb300.h -- C ABI of the GB300 (sm_103a) STRIDE "DPR4" v3 decoder.
 *
 * Plain pointers and sizes only (no torch or CUDA C++ types): `stream`
 * arguments are `cudaStream_t` values passed as `void*` (0 = legacy default
 * stream), device pointers are plain addresses in the current CUDA device.
 *
 * Every function returns 0 on success or a negative STRIDE_ERR_* code;
 * stride_last_error_message() gives a human-readable reason for the calling
 * thread's last failure.
 *
 * The reference decodes this format with the CPU function decode_dup
 * (encoder/paradelta_v5_dup.py:471-618) and exposes GPU decoding through
 * ParaDeltaV5GpuDecoder (utils/paradelta_v5_cuda.py:580-718), whose
 * constructor uploads the bytes and sizes the outputs (:597-684), whose
 * decode() enqueues the persistent decode kernel (:686-712) and whose
 * decode_to_host() copies the results back (:714-718).  The entry points
 * below replace that class's internals; the Python class
 * meshpress_gb300.ParaDeltaV5GpuDecoder binds them with ctypes.
 */
#ifndef STRIDE_GB300_H
#define STRIDE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define STRIDE_OK 0
#define STRIDE_ERR_ARG (-1)         /* bad argument (null pointer, size)            */
#define STRIDE_ERR_MAGIC (-2)       /* not a DPR4 stream (paradelta_v5_dup.py:520)  */
#define STRIDE_ERR_VERSION (-3)     /* DPR4 version != 3 (paradelta_v5_dup.py:523)  */
#define STRIDE_ERR_TRUNCATED (-4)   /* header / offset table past the end           */
#define STRIDE_ERR_OFFSET (-5)      /* offset table not increasing or out of range  */
#define STRIDE_ERR_CORRUPT (-6)     /* meshlet payload inconsistent (FIFO index,
                                       vertex id, triangle count, code range,
                                       payload end != next offset)                 */
#define STRIDE_ERR_UNSUPPORTED (-7) /* valid but outside this decoder's limits:
                                       > 256 local vertices or triangles per
                                       meshlet, g_bits > 24, K > 30, residual
                                       k > 24, IRLP sums beyond int32               */
#define STRIDE_ERR_CUDA (-8)        /* CUDA runtime error                           */
#define STRIDE_ERR_TIMEOUT (-9)     /* a bounded device/host wait gave up           */
#define STRIDE_ERR_NOMEM (-10)      /* allocation failed / admission budget          */
#define STRIDE_ERR_BUSY (-11)       /* server queue full                            */

typedef struct stride_handle stride_handle;

typedef struct {
    uint32_t n_meshlets;
    uint32_t g_bits[3];
    uint64_t n_v;        /* decoded (duplicated) vertices = sum of n_local      */
    uint64_t n_t;        /* triangles                                           */
    uint64_t nbytes;     /* length of the encoded stream                        */
    float center[3];
    float scale;
    int32_t pred_n[9];
    int32_t pred_k[3];
    uint32_t kernels;    /* kernel launches one decode makes: 2 with the
                            one-kernel shapes (scan, which also fills any
                            per-code dequantisation tables; then the fused
                            or the group kernel: persistent 2 or 3), 3 with
                            the two-kernel shapes (persistent 0 or 1), 0 for
                            an empty stream                                   */
    float g_min[3];      /* header g_min, g_range: a position's normalised   */
    float g_range[3];    /* value is g_min + q / (2^g_bits - 1) * g_range     */
    uint32_t shared_bytes;      /* stride_info only, after a decode: dynamic
                                   shared memory per CTA of the decode's main
                                   kernel (fused, group or vertex kernel)     */
    uint32_t persistent_blocks; /* ... and its CTAs; the reference's
                                   _shared_bytes / _persistent_blocks
                                   (utils/paradelta_v5_cuda.py:656-683)      */
} stride_info_t;

/* Launch shape of the decode kernel (the autotuner's search space). */
typedef struct {
    int32_t warps_per_cta;   /* 1, 2 or 4: connectivity kernel CTAs hold one
                                (1, 2) or two (4) parser/assembler warp pairs
                                of 32 meshlets each; the vertex kernel's CTA is
                                always three warps (one per axis)            */
    int32_t persistent;      /* 2 (default) = one persistent kernel for both
                                phases: CTAs of two pairs take connectivity
                                groups, then vertex work in the order groups
                                finish (warps_per_cta must be 4);
                                3 = group kernel: one warp decodes a group of
                                32 meshlets through every phase, lane per
                                meshlet (warps_per_cta 1 or 2; stage_bytes
                                and code_bytes unused);
                                1 = connectivity kernel, then a persistent
                                work-stealing vertex grid; 0 = connectivity
                                kernel, then one vertex CTA per group        */
    int32_t ctas_per_sm;     /* persistent grid = ctas_per_sm * SMs
                                (0 = as many as fit)                         */
    uint32_t stage_bytes;    /* the vertex kernel stages a round's residual
                                bits in half of this (the connectivity
                                kernel streams each meshlet through fixed
                                256-byte per-lane rings)                     */
    uint32_t code_bytes;     /* shared-memory code plane of one axis warp
                                (>= 516, or 1028 above 16-bit codes)        */
} stride_launch_cfg;

/* Thread-local description of the last error in this thread. */
const char* stride_last_error_message(void);
const char* stride_error_string(int code);

/* Library/device facts: number of SMs of the current device and the build's
 * target architecture (e.g. 103 for sm_103a). */
int stride_device_info(int* sm_count, int* arch);

/* Host-only: parse and validate the 86-byte global header and the size of the
 * offset table without touching the GPU.  Replaces the header part of
 * parse_globals_v5 (utils/paradelta_v5_cuda.py:515-577) for the DPR4 format
 * (header layout encoder/paradelta_v5_dup.py:412-447). */
int stride_inspect(const uint8_t* data, size_t len, stride_info_t* info);

/* ---- single mesh ---------------------------------------------------------
 * stride_open: parse + validate the global header on the host, allocate the
 * device copy of the bytes and the decoder's scratch, upload (synchronous).
 * Replaces ParaDeltaV5GpuDecoder.__init__ (utils/paradelta_v5_cuda.py:597-684)
 * and its CPU header parse parse_globals_v5 (:515-577).  The caller keeps
 * ownership of `data`. */
int stride_open(const uint8_t* data, size_t len, stride_handle** out);

/* Replace the handle's stream with new bytes (re-validates the header,
 * grows device buffers if needed, uploads asynchronously after the work
 * queued on `stream`; every later decode of the handle waits for it).
 * `data` must stay valid until the upload completes (the next decode or a
 * synchronisation); pinned host memory makes the upload asynchronous.  A
 * stream of about 3 million triangles or more goes up in four parts on a
 * copy stream of the handle's, so that stride_decode_host can start each
 * part of its decode as that part arrives. */
int stride_reload(stride_handle* h, const uint8_t* data, size_t len, void* stream);

int stride_info(const stride_handle* h, stride_info_t* info);

/* Enqueue one decode on `stream`: the header/meshlet-table parse kernel with
 * its device-wide scan, then the meshlet decode kernel.  Writes n_t x 3
 * uint32 triangle indices to d_idx and n_v x 3 float32 world-space positions
 * to d_pos (both device pointers, C-contiguous).  If d_codes is not NULL the
 * integer quantisation codes (n_v x 3 int32) are written too.  Asynchronous:
 * call stride_status() to learn whether the stream was valid.
 * Replaces ParaDeltaV5GpuDecoder.decode (utils/paradelta_v5_cuda.py:686-712)
 * plus the world-space transform of decode_to_host (:714-717). */
int stride_decode(stride_handle* h, void* stream, uint32_t* d_idx, float* d_pos,
                  int32_t* d_codes);

/* Decode with host buffers: enqueue decode into handle-owned device outputs,
 * copy them to h_idx / h_pos (host, n_t*3 uint32 and n_v*3 float32) and
 * synchronise.  Returns the decode status.  The triangle copy starts when
 * the connectivity kernel ends, beside the vertex kernel (a fused launch
 * shape is replaced by the persistent two-kernel one for this call); from
 * about 3 million triangles the connectivity runs in four parts and each
 * part's triangles are copied as soon as it ends, and after a
 * stride_reload of such a stream (uploaded in the same parts) each part
 * starts when its bytes are in.  Pinned host buffers make the copies
 * asynchronous to the host.
 * Replaces decode_to_host (utils/paradelta_v5_cuda.py:714-718). */
int stride_decode_host(stride_handle* h, void* stream, uint32_t* h_idx, float* h_pos);

/* Status of the last decode enqueued on this handle.  wait != 0 blocks until
 * it finished.  Returns STRIDE_OK, a STRIDE_ERR_* code for an invalid stream,
 * or STRIDE_ERR_BUSY when wait == 0 and the decode is still running.
 * *bad_meshlet (optional) receives the first failing meshlet. */
int stride_status(stride_handle* h, int wait, uint32_t* bad_meshlet);

/* The side table of the last decode, derived on the device: per meshlet the
 * stream bit where its anchor (residual part) starts (d_resid_bit, n_meshlets
 * uint64) and the starts of the dy, dz, px, py, pz substreams relative to it
 * (d_sub_offs, 5 x n_meshlets uint16, 0xFFFF when farther than 65,534 bits).
 * The reference GPU harness reads the same table from files its encoder
 * writes (scripts/dump_stride_dup_blob.py:120-160; there the anchor bit is
 * relative to the first meshlet).  Waits for the last decode; fails with its
 * status if that decode failed. */
int stride_side_table(stride_handle* h, void* stream, uint64_t* d_resid_bit, uint16_t* d_sub_offs);

/* ---- meshlet-native outputs (the consumer step after decode) ------------
 * No counterpart in the reference's decoder.  For a consumer that works per
 * meshlet (a renderer's meshlet pipeline): where each meshlet's rows lie in
 * the outputs, its bounds, and frustum culling of those bounds.  The first
 * two wait for the handle's last decode and fail with its status. */

/* Exclusive prefix sums, n_meshlets + 1 entries each (the last holds the
 * totals): meshlet m owns vertex rows [d_v_first[m], d_v_first[m+1]) and
 * triangle rows [d_t_first[m], d_t_first[m+1]) of the decode's outputs. */
int stride_meshlet_ranges(stride_handle* h, void* stream, uint64_t* d_v_first, uint64_t* d_t_first);

/* Axis-aligned bounds of each meshlet's rows of d_pos (the last decode's
 * positions): 6 floats per meshlet, min x y z then max x y z. */
int stride_meshlet_bounds(stride_handle* h, void* stream, const float* d_pos, float* d_bounds);

/* Frustum culling of n meshlet bounds (6 floats each, device) against six
 * planes (host, 24 floats: a b c d per plane, inside where
 * a x + b y + c z + d >= 0).  A meshlet is culled when its box lies wholly
 * outside one plane (or is empty).  Writes one visibility bit per meshlet
 * (d_visible, ceil(n / 32) uint32 words, bit m % 32 of word m / 32) and the
 * number of visible meshlets (*d_count, device).  Asynchronous. */
int stride_cull_meshlets(const float* d_bounds, uint32_t n, const float* planes, void* stream, uint32_t* d_visible,
                         uint32_t* d_count);

/* Measurement entry point (no reference counterpart): one decode like
 * stride_decode, with CUDA events recorded on `stream` between its
 * kernels; waits and writes their durations in milliseconds to
 * kernel_ms[0] (meshlet scan), kernel_ms[1] (connectivity) and
 * kernel_ms[2] (vertices + output).  With the fused kernel (persistent 2)
 * kernel_ms[1] is the fused kernel and kernel_ms[2] is 0. */
int stride_decode_timed(stride_handle* h, void* stream, uint32_t* d_idx, float* d_pos, float* kernel_ms);

/* Launch shape for this handle's decodes.  Until it is set the shape
 * follows the mesh's size: the two kernels (persistent 1) for 128 to 1,023
 * groups of 32 meshlets, the fused kernel (persistent 2) otherwise; a
 * reload keeps a shape that was set. */
int stride_set_config(stride_handle* h, const stride_launch_cfg* cfg);

/* No counterpart in the reference.  SM clocks each device wait of this
 * handle's decodes may spin -- a bulk copy's mbarrier, the fused kernel's
 * wait for a finished connectivity group -- before the decode gives up with
 * STRIDE_ERR_TIMEOUT (default 2^31, about a second; 0 gives up at the first
 * unsuccessful check).  The waits are bounded either way; a small limit
 * lets a test see the timeout path report its status while the context
 * stays usable for the next decode. */
int stride_set_wait_limit(stride_handle* h, uint64_t clocks);

void stride_close(stride_handle* h);

/* ---- decode without device allocation ------------------------------------
 * No counterpart in the reference.  For callers that must not call the CUDA
 * allocator after start-up -- e.g. a renderer's per-frame streaming loop,
 * where cudaMalloc/cudaFree synchronise the device and stall other streams,
 * or a plugin whose host application owns all device memory in its own
 * pool.  The caller passes the stream bytes on the host and its own device
 * output buffers (sizes from stride_inspect); the library uploads the bytes
 * into, and does all decode work in, one fixed 64 MiB device array that
 * every GPU loading the library reserves until process exit (enough for
 * streams of about 10 million triangles; larger ones are rejected with
 * STRIDE_ERR_NOMEM before any device work).  Calls nothing that allocates.
 * Synchronous: returns after the decode finished on `stream`, with its
 * status.  The first call on a device looks up the array's device address,
 * and that is where the runtime loads this library's device code on the
 * device and reserves the array (it can fail there with STRIDE_ERR_CUDA if
 * the device is out of memory): make that first call at start-up, before
 * any stream capture and before the frame loop.  A device reset
 * (cudaDeviceReset) releases the array; the next call on that device
 * reserves it again like a first call.  All calls share the array:
 * decodes that overlap on the GPU race and must be serialised. */
int stride_decode_static(const uint8_t* data, size_t len, void* stream, uint32_t* d_idx, float* d_pos);

/* ---- many meshes, one launch ---------------------------------------------
 * A batch holds the device copies of many streams and one device meshlet
 * queue over all of them.  Outputs are concatenated: mesh i writes its
 * triangles at d_idx + 3*t_offset[i] (indices local to mesh i) and its
 * positions at d_pos + 3*v_offset[i].  No reference counterpart: the
 * reference decodes one mesh per ParaDeltaV5GpuDecoder. */
typedef struct stride_batch stride_batch;


int stride_batch_create(const uint8_t* const* blobs, const size_t* lens, uint32_t n_meshes,
                        stride_batch** out);
int stride_batch_info(const stride_batch* b, uint64_t* n_meshlets, uint64_t* n_v, uint64_t* n_t);
/* Per-mesh output offsets (in vertices / triangles), n_meshes entries each. */
int stride_batch_offsets(const stride_batch* b, uint64_t* v_offset, uint64_t* t_offset);
int stride_batch_set_config(stride_batch* b, const stride_launch_cfg* cfg);
int stride_batch_get_config(const stride_batch* b, stride_launch_cfg* cfg);
int stride_batch_decode(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos);
/* Same decode, synchronous, with the device time of the scan, connectivity
 * and vertex kernels (CUDA events) in kernel_ms[0..2] (fused kernel: in
 * kernel_ms[1], kernel_ms[2] = 0, as for stride_decode_timed). */
int stride_batch_decode_timed(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos, float* kernel_ms);
/* Decode into d_idx / d_pos and copy both to h_idx / h_pos (host, the same
 * sizes; pinned for asynchronous copies), synchronously, overlapping the
 * copies with the decode as stride_decode_host does.  Returns the decode
 * status. */
int stride_batch_decode_to_host(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos, uint32_t* h_idx,
                                float* h_pos);
/* The arena image: stream i sits at blob_offsets[i] of an image_bytes-long
 * buffer (zero bytes elsewhere).  A caller that keeps such an image in
 * (pinned) host memory replaces every stream of the batch with one
 * asynchronous copy on `stream` through stride_batch_upload. */
int stride_batch_image(const stride_batch* b, uint64_t* blob_offsets, uint64_t* image_bytes);
/* The upload runs after the work queued on `stream`, and every later decode
 * of the batch waits for it; `image` must stay valid until then.  A batch
 * of about 3 million triangles or more goes up in four parts on a copy
 * stream of the batch's, so that stride_batch_decode_to_host can start each
 * part of its decode as that part arrives. */
int stride_batch_upload(stride_batch* b, void* stream, const void* image, size_t bytes);
/* Capture the decode sequence for these output pointers into a CUDA graph
 * (replaces any earlier graph) and replay it with stride_batch_launch_graph. */
int stride_batch_capture_graph(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos);
int stride_batch_launch_graph(stride_batch* b, void* stream);
/* Time every launch configuration on this batch (CUDA events, `iters` runs
 * each), keep the fastest, and report it. */
int stride_batch_autotune(stride_batch* b, void* stream, uint32_t* d_idx, float* d_pos,
                          int iters, stride_launch_cfg* best, float* best_ms);
int stride_batch_status(stride_batch* b, int wait, uint32_t* bad_mesh, uint32_t* bad_meshlet);
void stride_batch_destroy(stride_batch* b);

/* ---- serving: continuous batching over a device-resident arena ----------
 * Requests (encoded blobs) are submitted from any host thread.  A scheduler
 * thread admits queued requests while the arena (payload + output bytes)
 * stays under `hbm_budget_bytes`, packs whatever was admitted into one
 * persistent-kernel launch on one of `n_streams` streams, and keeps up to
 * n_streams launches in flight, so requests arriving while others decode are
 * admitted as soon as arena space frees.  Results stay in device memory until
 * the caller releases them.  No reference counterpart. */
typedef struct stride_server stride_server;

typedef struct {
    uint64_t hbm_budget_bytes;   /* arena limit for payloads + outputs        */
    uint32_t max_batch;          /* requests per launch (0 = 256)             */
    uint32_t n_streams;          /* launches in flight (0 = 2)                */
    uint32_t max_queue;          /* queued requests before submit is refused  */
    uint32_t copy_to_host;       /* 1 = also copy results to host buffers     */
    uint32_t pad0;
    uint64_t pinned_budget_bytes; /* pinned slab for payloads copied at submit, pinned
                                   * once at create (0 = 1 GiB); a payload that finds
                                   * no room in it is staged per launch             */
} stride_server_opts;

typedef struct {
    int32_t status;              /* STRIDE_OK or STRIDE_ERR_*                   */
    uint32_t pad;
    uint64_t n_v, n_t;
    const uint32_t* d_idx;       /* device results (valid until released)     */
    const float* d_pos;
    const uint32_t* h_idx;       /* host copies when copy_to_host             */
    const float* h_pos;
    double t_submit_us, t_admit_us, t_done_us; /* host steady clock, microseconds */
} stride_result;

int stride_server_create(const stride_server_opts* opts, stride_server** out);
/* Copies `data` (into pinned memory within the pinned budget, on the
 * calling thread); returns a request id. */
int stride_server_submit(stride_server* s, const uint8_t* data, size_t len, uint64_t* req_id);
/* Waits up to timeout_ms (<0 = forever) for the request to finish. */
int stride_server_wait(stride_server* s, uint64_t req_id, int timeout_ms, stride_result* out);
/* Frees the request's arena space. */
int stride_server_release(stride_server* s, uint64_t req_id);
/* hold != 0: keep admitting submissions to the queue but start no launch
 * (e.g. to collect a frame's requests into as few launches as possible);
 * hold == 0: resume.  Launches already running are not affected. */
int stride_server_hold(stride_server* s, int hold);
int stride_server_stats(stride_server* s, uint64_t* launches, uint64_t* completed,
                        uint64_t* arena_peak_bytes);
void stride_server_destroy(stride_server* s);

/* ---- PLDT v5 streams ------------------------------------------------------
 * The format the reference's CuPy decoder reads (magic 0x504C4454, version
 * 5: a global boundary table, per-meshlet boundary references, strip
 * connectivity, a float64 lin3 predictor).  Decoded bit-exactly like the
 * reference CPU decoder decode_paradelta_v5 (encoder/paradelta_v5.py:286-462);
 * rows are the boundary vertices, then every meshlet's interior vertices.
 * Stricter than that decoder on invalid streams: boundary references must
 * be rows of the boundary table, the strips must yield the header's triangle
 * count, and meshlets must lie back to back as the offset table says. */
typedef struct pldt5_handle pldt5_handle;

typedef struct {
    uint32_t n_meshlets;
    uint32_t n_boundary;
    uint32_t g_bits[3];
    uint64_t n_v;        /* decoded rows: boundary + interior vertices        */
    uint64_t n_t;
    uint64_t nbytes;
    float center[3];
    float scale;
    float lin3_w[3];
} pldt5_info_t;

/* Host parse of the header, the boundary table and the meshlet headers, then
 * a device copy.  Replaces parse_globals_v5 + ParaDeltaV5GpuDecoder.__init__
 * (utils/paradelta_v5_cuda.py:515-684). */
int pldt5_open(const uint8_t* data, size_t len, pldt5_handle** out);
/* The same host parse and validation without a device (sizes of the
 * outputs, header fields); like stride_inspect. */
int pldt5_inspect(const uint8_t* data, size_t len, pldt5_info_t* info);
int pldt5_info(const pldt5_handle* h, pldt5_info_t* info);
/* Enqueue the decode on `stream`: triangles (n_t x 3 uint32, global rows)
 * and world-space positions (n_v x 3 float32) into device buffers.
 * Replaces ParaDeltaV5GpuDecoder.decode (:686-712) plus the world transform
 * of decode_to_host (:714-717). */
int pldt5_decode(pldt5_handle* h, void* stream, uint32_t* d_idx, float* d_pos);
/* Like stride_status (wait != 0 blocks until the decode ends). */
int pldt5_status(pldt5_handle* h, int wait);
void pldt5_close(pldt5_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* STRIDE_GB300_H */
