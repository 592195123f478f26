/*
 * Host runtime shared by the livre_gb300 translation units: device buffers,
 * the context (streams, scratch, pinned staging), error handling.
 */
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include <cstdio>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "host_pool.h"
#include "lv_internal.h"

namespace lv
{
/* Owning device buffer that only grows. */
struct DeviceBuffer
{
    void* ptr = nullptr;
    size_t bytes = 0;

    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }

    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    /* Ensures at least `n` bytes; contents are not preserved on growth. */
    cudaError_t reserve(size_t n)
    {
        if (n <= bytes)
            return cudaSuccess;
        release();
        const size_t want = n < 256 ? 256 : n;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess)
            bytes = want;
        else
            ptr = nullptr;
        return e;
    }
    template <class T>
    T* as() const
    {
        return static_cast<T*>(ptr);
    }
};

/* Owning page-locked host buffer that only grows. It is mapped into the
 * device's address space: kernels may write it through `dev`. */
struct PinnedBuffer
{
    void* ptr = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    PinnedBuffer() = default;
    PinnedBuffer(const PinnedBuffer&) = delete;
    PinnedBuffer& operator=(const PinnedBuffer&) = delete;
    ~PinnedBuffer() { release(); }
    void release()
    {
        if (ptr)
            cudaFreeHost(ptr);
        ptr = nullptr;
        dev = nullptr;
        bytes = 0;
    }
    cudaError_t reserve(size_t n)
    {
        if (n <= bytes)
            return cudaSuccess;
        release();
        cudaError_t e = cudaHostAlloc(&ptr, n < 256 ? 256 : n, cudaHostAllocMapped);
        if (e != cudaSuccess)
        {
            ptr = nullptr;
            return e;
        }
        e = cudaHostGetDevicePointer(&dev, ptr, 0);
        if (e != cudaSuccess)
        {
            release();
            return e;
        }
        bytes = n < 256 ? 256 : n;
        return cudaSuccess;
    }
    template <class T>
    T* as() const
    {
        return static_cast<T*>(ptr);
    }
    /* the same memory as the device addresses it (mapped) */
    template <class T>
    T* as_dev() const
    {
        return static_cast<T*>(dev);
    }
};

/* Scratch of the LOD selection: two frontier queues + per-level counters. */
struct SelectScratch
{
    DeviceBuffer ids[2];
    DeviceBuffer view[2];
    DeviceBuffer counts;  /* kMaxLevels + 2 words, then the overflow word */
    DeviceBuffer views;   /* LodView array */
    DeviceBuffer sort;    /* range-slice sort keys/ids */
    PinnedBuffer staging; /* host copy of the LodView array */
    uint32_t frontier_capacity = 0;
    uint32_t generation = 0; /* bumped whenever the queues are reallocated */
    /* recorded after the last selection that used these queues, on whatever
     * stream it ran: the next user, on any stream, waits for it */
    cudaEvent_t free_event = nullptr;
    bool free_recorded = false;
    SelectScratch() = default;
    SelectScratch(const SelectScratch&) = delete;
    SelectScratch& operator=(const SelectScratch&) = delete;
    ~SelectScratch()
    {
        if (free_event)
            cudaEventDestroy(free_event);
    }
};

/* Orders a selection on stream s after the previous user of the scratch
 * (scratch_acquire), and the next user after it (scratch_release). */
lv_status scratch_acquire(lv_ctx* ctx, SelectScratch& S, cudaStream_t s);
lv_status scratch_release(lv_ctx* ctx, SelectScratch& S, cudaStream_t s);

struct Pool;
struct Renderer;

} // namespace lv

struct lv_ctx
{
    int device = 0;
    std::string error;
    cudaStream_t upload_stream = nullptr;
    lv::SelectScratch sel;
    lv::DeviceBuffer sel_host_out; /* lv_select_visible_host's device output */
    uint32_t test_barrier_polls = 0; /* lv_test_fail_grid_barrier */
    lv::Pool* pool = nullptr;
    lv::Renderer* renderer = nullptr;
    size_t pool_bytes = size_t(3072) << 20;
    uint32_t brick_layout = LV_BRICKS_QUADS; /* lv_pool_set_brick_layout */
    /* lv_render's ray cast */
    lv_render_launch launch{LV_LAUNCH_TILE_GRID, 8, 8, 0, LV_ORDER_LONGEST_FIRST, 1};
    /* host fetchers of callback sources (created on first use) */
    lv::HostPool* host_pool = nullptr;
    lv_ctx_totals totals{}; /* since creation, host-side (lv_get_totals) */
    /* bumped by every pool user other than lv_render (batches, the server)
     * whose work may still read pool slots when it returns */
    std::atomic<uint64_t> foreign_pool_use{0};
    std::mutex mutex;
};

namespace lv
{
inline lv_status fail(lv_ctx* ctx, lv_status st, const std::string& msg)
{
    if (ctx)
        ctx->error = msg;
    return st;
}

inline lv_status cuda_fail(lv_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(ctx, e == cudaErrorMemoryAllocation ? LV_ENOMEM : LV_EDEVICE,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define LV_CUDA(ctx, call)                                                    \
    do                                                                        \
    {                                                                         \
        cudaError_t lv_e_ = (call);                                           \
        if (lv_e_ != cudaSuccess)                                             \
            return ::lv::cuda_fail((ctx), lv_e_, #call);                      \
    } while (0)

/* Host-side derivation of the per-view selection constants. */
lv_status make_lod_view(lv_ctx* ctx, const lv_volume_info& vol,
                        const lv_camera& cam, const lv_lod_params& p,
                        LodView& out);

/* Runs the level-synchronous selection for n views (constants in
 * `host_views`, written to the device by this call) on `stream`.
 * Each view writes its visible ids to views[i].out_ids and its result words.
 * The device frontier holds at most `frontier_capacity` nodes per level. */
lv_status run_selection(lv_ctx* ctx, const LodView* host_views,
                        uint32_t n_views, uint32_t max_depth,
                        cudaStream_t stream, bool allow_fused = true);

/* The launch the ray cast of V really uses under L (other voxel types than
 * uint8 / uint16 always use one CTA per tile). */
lv_render_launch effective_launch(const RayView& V, const lv_render_launch& L);
/* lv_render's tile order for V under L, computed on `side` into the
 * renderer's tile scratch (null for raster order or the per-pixel grid). */
lv_status prepare_frame_order(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                              cudaStream_t side, const uint32_t*& order);

/* Kernels run_selection launches for n views of an octree of `depth` levels. */
uint32_t selection_launches(lv_ctx* ctx, uint32_t n_views, uint32_t depth,
                            bool allow_fused = true);

/* Enqueues the selection kernels for n views whose constants are already
 * on the device (capturable: no host synchronisation). */
lv_status enqueue_selection(lv_ctx* ctx, SelectScratch& S, const LodView* d_views,
                            uint32_t n_views, uint32_t total_roots, uint32_t max_depth,
                            cudaStream_t stream, const uint32_t* d_total_roots = nullptr);
/* Grows the frontier queues of S to hold `nodes` per level (synchronises `s`
 * when it reallocates). */
lv_status reserve_frontier(lv_ctx* ctx, SelectScratch& S, uint64_t nodes, cudaStream_t s);

/* Frontier size needed for a full traversal of a volume. */
uint64_t max_frontier(const lv_volume_info& vol);

/* Applies the sort-last range slice of SelectVisibles::visitPost to one
 * view (restores DFS order first). Synchronises `stream`. */
lv_status range_slice(lv_ctx* ctx, const lv_volume_info& vol,
                      const float range[2], uint64_t* d_ids, uint32_t* d_result,
                      cudaStream_t stream);

} // namespace lv

namespace lv
{
enum SourceKind
{
    SRC_CALLBACK = 0,
    SRC_BLOB_DEVICE = 1,
    SRC_BLOB_HOST = 2,
    SRC_FBM_DEVICE = 3
};

/* One resident brick. */
struct Resident
{
    lv_volume* vol;
    uint64_t node_idx;
    uint32_t unit;
    uint32_t units;
    uint64_t load; /* the stream_bricks call that placed it (Pool::loads) */
};

struct Pool
{
    DeviceBuffer arena;
    uint64_t capacity_units = 0;
    uint64_t bump = 0;
    std::map<uint32_t, std::vector<uint32_t>> free_by_units;
    std::list<Resident> lru; /* front = oldest load */
    uint64_t loads = 0;      /* stream_bricks calls so far */
    uint64_t resident_bytes = 0;
    /* per slot size: resident bricks and those pinned by server requests */
    std::map<uint32_t, uint64_t> resident_count, pinned_count;
};

struct Renderer
{
    DeviceBuffer visible, sel_result, render_ids, render_slots, missing,
        counters, leaf, pairs;
    DeviceBuffer tiles; /* longest-first tile order: bucket counts, keys, order */
    PinnedBuffer h_counters, h_missing, h_pairs;
    uint64_t visible_capacity = 0;
    uint32_t frame = 0;
    lv_frame_stats stats{};
    cudaStream_t last_stream = nullptr;
    bool have_last = false;
    /* the last frame's volume (null once destroyed) and description */
    lv_volume* last_vol = nullptr;
    lv_render_desc last_desc{};
    /* async mode: misses of the previous frame, copied back */
    cudaEvent_t pending_event = nullptr;
    lv_volume* pending_vol = nullptr;
    uint32_t pending_max = 0;
    uint32_t pending_frame = 0;
    cudaEvent_t render_event = nullptr;
    cudaEvent_t upload_event = nullptr;
    /* end of the last lv_render's work on its stream: lv_render returns
     * before its ray cast ends, so the next frame (on any stream) and any
     * brick streaming wait for it */
    cudaEvent_t frame_done = nullptr;
    /* the residency pass's counters have reached the host */
    cudaEvent_t resolve_done = nullptr;
    /* work a frame needs from the camera alone (the tile order, clearing
     * the leaf grid) runs on `side` while the selection runs: `fork` is
     * recorded before the selection, `join` after the side work */
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    const uint32_t* pre_order = nullptr; /* this frame's tile order (or null) */
    bool leaf_cleared = false;           /* the side stream cleared the leaf grid */
    /* the selection runs on its own high-priority stream once the previous
     * frame's residency pass has read the visible list (`visible_free`), so
     * a frame queued while the previous one still ray casts selects beside
     * it; `sel_done` orders the rest of the frame after it */
    cudaStream_t sel_stream = nullptr;
    cudaEvent_t sel_done = nullptr, visible_free = nullptr;
    bool visible_free_recorded = false;
    /* timing of the last frame: selection and ray cast */
    cudaEvent_t t_sel0 = nullptr, t_sel1 = nullptr, t_ray0 = nullptr, t_ray1 = nullptr;
    uint32_t launches = 0;
    /* multi-pass frames: the visible set split into pool-sized passes */
    PinnedBuffer h_pass;     /* visible ids in pass order */
    DeviceBuffer pass_count; /* visible ids of the current pass */
    uint32_t passes = 0;     /* passes of the last frame (0: one-pass frame) */
    lv_frame_stats pass_stats{}; /* summed over the passes */
    /* a frame queued while the previous one still ray casts looks its
     * visible bricks up beside it and streams the missing ones then */
    DeviceBuffer probe, probe_count; /* missing visible ids, their count */
    PinnedBuffer h_probe;
    uint64_t foreign_seen = 0; /* lv_ctx::foreign_pool_use after the last frame */
    /* device-generated bricks: ids and slot offsets */
    DeviceBuffer gen;
    PinnedBuffer h_gen;
    /* slot offsets of the uint8 bricks to expand into voxel quads, read by
     * the expansion kernel from mapped memory; free again once
     * expand_done has completed */
    PinnedBuffer h_expand;
    cudaEvent_t expand_done = nullptr;
    bool expand_recorded = false;
    /* (source, slot) offsets of the host-store bricks gather_bricks_kernel
     * reads, mapped; rewritten only once gather_done has completed */
    PinnedBuffer h_gather;
    cudaEvent_t gather_done = nullptr;
    bool gather_recorded = false;
};



/* Streams bricks `ids` of `vol` into the pool (allocate / evict bricks whose
 * node stamp is below protect_frame, fetch, copy on the upload stream,
 * publish page-table entries); `render` waits for the copies. The copies
 * wait for the work queued on `render` and for the last lv_render frame,
 * unless `beside_frame`: the caller then guarantees that protect_frame
 * spares every brick that queued work reads. */
lv_status stream_bricks(lv_ctx* ctx, lv_volume* vol, const uint64_t* ids,
                        uint32_t n, uint32_t protect_frame, cudaStream_t render,
                        uint32_t& n_loaded, uint64_t& bytes_loaded,
                        bool beside_frame = false);
lv_status ensure_renderer(lv_ctx* ctx);
/* Ray-cast constants of one view (shared by the plain and batched paths). */
lv_status make_ray_view(lv_ctx* ctx, const lv_volume* vol, const lv_tf* tf,
                        const lv_render_desc& desc, const lv_lod_params& lod, float* d_rgba,
                        uint32_t* leaf, uint32_t* counters, RayView& V);
/* Index of the ray-cast kernel instantiation for a view. */
int kernel_variant(uint32_t dtype, uint32_t filter, uint32_t edge);
/* Kernel groups of a batch's persistent queues: kernel_variant's 0..7, and
 * 8..13 for trilinear uint8 / uint16 bricks of pitch 34, 66 or 130 (the
 * pitch as immediates); >= kBatchGroups: a voxel type only the per-view
 * kernels render. */
constexpr int kBatchGroups = 14;
int batch_group(const RayView& V);
/* Per-view completion of a batch of per-view kernels (LV_QUEUE_VIEW_KERNELS):
 * called on a CUDA host-function thread once view `view`'s image is written,
 * with its counter words (FrameCounter words, then the selection result).
 * The callback must not call CUDA. */
typedef void (*BatchViewDone)(void* user, uint32_t view, const uint32_t* words);
void batch_set_view_hook(lv_batch* b, BatchViewDone fn, void* user);
/* Stream priority levels of a batch's ray casts: level 0 is one step below
 * the device's highest priority (kept for admission work), each further
 * level one step lower (clamped to the lowest). */
constexpr int kBatchPriorityLevels = 4;
/* Ray casts of the next launches at priority `level` (0 .. levels - 1): a
 * server launches each batch one level below the batches still rendering,
 * so older requests keep the SM slots first and a younger batch takes the
 * slots they leave free. */
void batch_set_priority_level(lv_batch* b, int level);
/* Frame statistics from a view's counter words. */
void batch_decode_stats(const uint32_t* words, lv_frame_stats& s);

/* One view's ray cast with launch shape L, its longest-first tile order (if
 * any) in `order_scratch` (tile_order_bytes; nullptr: the context's lv_render
 * scratch). The view's samples per ray must already be in its counters. */
lv_status launch_view_raycast(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                              uint8_t* order_scratch, cudaStream_t s);
size_t tile_order_bytes(const RayView& V, const lv_render_launch& L);
/* Longest-first order of a batched group's work items (memset + 2 kernels);
 * hist: 128 words, keys and order: max_items entries (an upper bound of the
 * group's items at every replay of a captured launch). */
/* fBm bricks for device ids d_ids into `out` (at d_offsets[i] when given,
 * else packed brick_bytes apart). */
lv_status launch_fbm_bricks(lv_ctx* ctx, const lv_volume_info& info, const lv_fbm_params& f,
                            const uint16_t* d_perm, const uint64_t* d_ids, uint32_t n,
                            uint8_t* out, const uint64_t* d_offsets, uint64_t brick_bytes,
                            cudaStream_t s);
std::vector<uint16_t> fbm_permutation(uint64_t seed);
lv_status volume_init(lv_ctx* ctx, lv_volume* v);
lv_status launch_batch_order(lv_ctx* ctx, const RayView* d_rays, const TileQueue& Q,
                             uint32_t max_items, uint8_t* keys, uint32_t* hist,
                             uint32_t* order, cudaStream_t s);
lv_status launch_persistent(lv_ctx* ctx, int variant, const lv_batch_config& cfg,
                            const RayView* d_rays, const TileQueue& Q, uint32_t tfn_max,
                            cudaStream_t s);
} // namespace lv

struct lv_tf
{
    lv_ctx* ctx;
    lv::DeviceBuffer rgba;
    uint32_t n;
};

struct lv_volume
{
    lv_ctx* ctx = nullptr;
    lv_volume_info info{};
    int kind = lv::SRC_CALLBACK;
    lv_get_data_fn fn = nullptr;
    void* user = nullptr;
    void (*user_free)(void*) = nullptr; /* built-in sources own `user` */
    lv_blob_desc blob{};
    lv::DeviceBuffer d_blobs;
    lv_fbm_params fbm{};
    lv::DeviceBuffer d_perm; /* fBm permutation (512 entries) */
    lv::PinnedBuffer host_store;
    uint64_t brick_bytes = 0;
    uint32_t slot_units = 0;
    /* uint8 volumes of quad_layout rows store their bricks as voxel quads
     * (lv_internal.h) unless the pool keeps them compact: a brick's
     * canonical bytes are written at slot + stage_off, then expanded in
     * place (or gathered straight into the quads); 0 for the others */
    uint64_t stage_off = 0;
    uint64_t level_offset[lv::kMaxLevels + 1] = {};
    uint64_t n_nodes = 0;
    lv::DeviceBuffer node_table, node_stamp;
    std::vector<int32_t> host_table;
    /* host pin counts per node: bricks of admitted, unfinished server
     * requests are never evicted (empty until a server uses the volume) */
    std::vector<uint16_t> pins;
    uint32_t time_step = 0;
    /* the last synchronous frame streamed bricks: the next one likely will
     * too, so it waits for its miss count before queueing the ray cast */
    bool streamed_last = false;
    /* pinned staging ring for callback sources: 2 * fetch_threads buffers
     * (at least 4), one group fetching while the previous one copies */
    std::vector<lv::PinnedBuffer*> staging;
    std::vector<cudaEvent_t> staging_ev;
    uint32_t fetch_threads = 1; /* > 1: get_data is called concurrently */
    ~lv_volume()
    {
        for (auto* p : staging)
            delete p;
        for (auto e : staging_ev)
            cudaEventDestroy(e);
    }
};

