/*
 * Batched rendering: many views (different volumes, transfer functions,
 * viewports and LOD thresholds) in one pass.
 *
 *  - one multi-view LOD selection (every view's frontier in the same queues),
 *  - one residency pass, prune and leaf-grid splat over all views
 *    (blockIdx.y = view),
 *  - one persistent ray-cast launch per voxel type / filter, whose CTAs pop
 *    (view, tile) items from a device work queue, or one ray-cast kernel per
 *    view on parallel streams (LV_QUEUE_VIEW_KERNELS),
 *  - the whole sequence runs as one CUDA graph launch: persistent queues are
 *    captured once and replayed (the per-view constants travel in one
 *    host->device copy inside the graph); per-view kernels, whose constants
 *    and grids are launch parameters, are captured on every call and applied
 *    to the cached executable graph by an update.
 *
 * Residency follows the reference's asynchronous mode (RenderPipeline::
 * renderAsync, livre/lib/pipeline/RenderPipeline.cpp:160-225): missing bricks
 * are replaced by their nearest resident ancestor and streamed before the next
 * launch (up to desc.max_uploads per view), since a graph cannot wait on the
 * host.
 *
 * An autotuner times the persistent kernel over tile shapes, CTAs per SM and
 * transfer-function staging (shared memory or L1) on the batch itself.
 */
#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "lv_runtime.h"

namespace lv
{
lv_status launch_views_pipeline(lv_ctx* ctx, const ResolveView* d_resolve,
                                const RayView* d_rays, uint32_t n, cudaStream_t s);
void type_range(uint32_t dt, float& lo, float& hi);
} // namespace lv

namespace
{
/* Views rendered by one instantiation of the persistent kernel. */
struct Group
{
    std::vector<uint32_t> views;
    uint32_t items = 0; /* work items (tiles) of the group's views */
};
constexpr int kGroups = lv::kBatchGroups;
/* streams the per-view kernels of a batch spread over */
constexpr uint32_t kViewStreams = 8;

/* byte offsets of one view's device regions */
struct ViewSlots
{
    uint64_t visible, render_ids, render_slots, missing, view_stamp, leaf;
};
} // namespace

struct lv_batch
{
    lv_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr, user_ready = nullptr;
    cudaEvent_t t_sel0 = nullptr, t_ray0 = nullptr, t_ray1 = nullptr;
    lv_batch_config cfg{8, 8, 0, 0, 1, LV_QUEUE_VIEW_KERNELS, 8, LV_ORDER_LONGEST_FIRST, 1};
    /* per-group longest-first order: hist (128 words) | keys | order, each
     * group at a fixed offset sized for order_cap items (grow-only) */
    lv::DeviceBuffer order_buf;
    uint32_t order_cap = 0;
    /* one stream per non-first group: the groups' persistent launches run
     * side by side, so one group's last tiles overlap the next group */
    /* at each priority level (batch_set_priority_level) */
    cudaStream_t aux[lv::kBatchPriorityLevels][kGroups] = {};
    int prio_level = 0;
    cudaEvent_t fork = nullptr, join[kGroups] = {};
    /* per-view kernels: tile-order scratch (offset of each view's region)
     * and ray-cast timing */
    lv::DeviceBuffer view_scratch;
    std::vector<uint64_t> view_offs;
    cudaEvent_t t_vk0 = nullptr, t_vk1 = nullptr;
    bool vk_timed = false;
    /* per-view completion hook (per-view kernels only) */
    lv::BatchViewDone hook = nullptr;
    void* hook_user = nullptr;
    lv::PinnedBuffer h_view_words;
    struct HookArg
    {
        lv_batch* b;
        uint32_t view;
    };
    std::vector<HookArg> hook_args;
    /* per-view region strides (grow-only) */
    uint64_t nodes_stride = 0, cells_stride = 0, missing_stride = 0;
    uint32_t views_cap = 0;
    uint32_t depth_max = 0;
    lv::DeviceBuffer params, zeroed, leafs, lists;
    lv::PinnedBuffer h_params, h_out;
    lv::SelectScratch sel; /* own frontier queues: independent of lv_render */
    uint64_t params_bytes = 0;
    uint32_t generation = 0;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t,
                        uint32_t, uintptr_t>,
             cudaGraphExec_t>
        graphs;
    uint32_t launch_id = 0;
    uint32_t frame = 0;
    /* previous launch, for the async misses and for statistics */
    std::vector<lv_batch_view> last;
    bool pending = false;
    uint64_t uploaded_bytes = 0;
    uint32_t uploaded = 0;
    uint32_t launches = 0;
    uint32_t last_n = 0;
    uint32_t sel_generation = 0; /* b->sel.generation the cached graphs use */
    uint64_t captures = 0, replays = 0;
    /* the last lv_batch_autotune: every candidate and its mean ray-cast ms */
    std::vector<lv_batch_config> tune_cfgs;
    std::vector<float> tune_ms;

    ~lv_batch()
    {
        for (auto& kv : graphs)
            cudaGraphExecDestroy(kv.second);
        if (done)
            cudaEventDestroy(done);
        if (user_ready)
            cudaEventDestroy(user_ready);
        if (t_sel0)
            cudaEventDestroy(t_sel0);
        if (t_ray0)
            cudaEventDestroy(t_ray0);
        if (t_ray1)
            cudaEventDestroy(t_ray1);
        if (fork)
            cudaEventDestroy(fork);
        if (t_vk0)
            cudaEventDestroy(t_vk0);
        if (t_vk1)
            cudaEventDestroy(t_vk1);
        for (int g = 0; g < kGroups; ++g)
        {
            if (join[g])
                cudaEventDestroy(join[g]);
            for (int l = 0; l < lv::kBatchPriorityLevels; ++l)
                if (aux[l][g])
                    cudaStreamDestroy(aux[l][g]);
        }
        if (stream)
            cudaStreamDestroy(stream);
    }
};

namespace
{
using namespace lv;

constexpr uint32_t kOutWords = FC_WORDS + LV_SELECT_RESULT_WORDS;

/* params layout: LodView[n] | ResolveView[n] | RayView[n] | queue tables */
struct ParamLayout
{
    uint64_t lod, resolve, ray, tables, bytes;
};

ParamLayout param_layout(uint32_t n)
{
    auto al = [](uint64_t x) { return (x + 255) & ~uint64_t(255); };
    ParamLayout L;
    L.lod = 0;
    L.resolve = al(L.lod + sizeof(LodView) * n);
    L.ray = al(L.resolve + sizeof(ResolveView) * n);
    L.tables = al(L.ray + sizeof(RayView) * n);
    /* kGroups x (view ids n + tile starts n + 1), then kGroups view counts
     * and the total root count: everything that changes between launches of
     * one captured graph lives in this copied block */
    L.bytes = al(L.tables + sizeof(uint32_t) * (kGroups * (2 * n + 1) + kGroups + 1));
    return L;
}

/* bytes of one view's id, slot and stamp lists */
uint64_t lists_per_view(const lv_batch* b) { return b->nodes_stride * (8 + 8 + 4 + 4); }

constexpr uint64_t kOrderHistBytes = 2 * 64 * sizeof(uint32_t);
uint64_t order_keys_bytes(uint32_t cap) { return (uint64_t(cap) + 255) & ~uint64_t(255); }
uint64_t order_region_bytes(uint32_t cap)
{
    return kOrderHistBytes + order_keys_bytes(cap) + sizeof(uint32_t) * uint64_t(cap);
}

/* Longest-first order buffers for groups of up to `items` work items; a
 * reallocation drops the captured graphs (they hold the old addresses). */
lv_status ensure_order(lv_batch* b, uint32_t items)
{
    /* per-view kernels order each view's tiles in their own scratch */
    if (b->cfg.order != LV_ORDER_LONGEST_FIRST || b->cfg.queue == LV_QUEUE_VIEW_KERNELS ||
        items <= b->order_cap)
        return LV_OK;
    lv_ctx* ctx = b->ctx;
    LV_CUDA(ctx, cudaStreamSynchronize(b->stream));
    uint32_t cap = std::max<uint32_t>(b->order_cap, 4096);
    while (cap < items)
        cap += cap / 2;
    b->order_buf.release();
    LV_CUDA(ctx, b->order_buf.reserve(order_region_bytes(cap) * kGroups));
    b->order_cap = cap;
    for (auto& kv : b->graphs)
        cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
    ++b->generation;
    return LV_OK;
}

lv_status ensure_regions(lv_batch* b, const lv_batch_view* views, uint32_t n,
                         cudaStream_t user, uint32_t n_run)
{
    lv_ctx* ctx = b->ctx;
    uint64_t nodes = b->nodes_stride, cells = b->cells_stride;
    uint32_t depth = b->depth_max;
    for (uint32_t i = 0; i < n; ++i)
    {
        const lv_volume_info& vi = views[i].volume->info;
        nodes = std::max(nodes, views[i].volume->n_nodes);
        uint64_t c = 1;
        for (int a = 0; a < 3; ++a)
            c *= uint64_t(vi.root_blocks[a]) << (vi.depth - 1);
        cells = std::max(cells, c);
        depth = std::max(depth, vi.depth);
    }
    const uint32_t vcap = std::max(b->views_cap, n_run);
    const bool grow = nodes > b->nodes_stride || cells > b->cells_stride ||
                      vcap > b->views_cap;
    b->depth_max = depth;
    if (!grow)
        return LV_OK;
    LV_CUDA(ctx, cudaStreamSynchronize(b->stream));
    LV_CUDA(ctx, cudaStreamSynchronize(user));
    b->nodes_stride = (nodes + 63) & ~uint64_t(63);
    b->cells_stride = (cells + 63) & ~uint64_t(63);
    b->missing_stride = std::min<uint64_t>(b->nodes_stride, 4096);
    b->views_cap = vcap;
    const ParamLayout PL = param_layout(vcap);
    b->params_bytes = PL.bytes;
    LV_CUDA(ctx, b->params.reserve(PL.bytes));
    LV_CUDA(ctx, b->h_params.reserve(PL.bytes));
    LV_CUDA(ctx, b->zeroed.reserve(sizeof(uint32_t) * (kOutWords * vcap + 64)));
    LV_CUDA(ctx, b->leafs.reserve(sizeof(uint32_t) * b->cells_stride * vcap));
    /* per view: visible + render ids (u64) + render slots + view stamps
     * (u32); then the missing lists of all views, contiguous (one
     * read-back kernel brings them to the host) */
    const uint64_t lists_bytes = lists_per_view(b) * vcap + b->missing_stride * 8 * vcap;
    b->lists.release();
    LV_CUDA(ctx, b->lists.reserve(lists_bytes));
    LV_CUDA(ctx, b->h_out.reserve(sizeof(uint32_t) * (kOutWords * vcap + 64) +
                                  sizeof(uint64_t) * b->missing_stride * vcap));
    /* view stamps start at 0; launch ids start at 1 */
    LV_CUDA(ctx, cudaMemset(b->lists.ptr, 0, lists_bytes));
    for (auto& kv : b->graphs)
        cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
    ++b->generation;
    return LV_OK;
}

ViewSlots view_slots(const lv_batch* b, uint32_t i)
{
    const uint64_t base = lists_per_view(b) * i;
    ViewSlots s;
    s.visible = base;
    s.render_ids = base + b->nodes_stride * 8;
    s.render_slots = s.render_ids + b->nodes_stride * 8;
    s.view_stamp = s.render_slots + b->nodes_stride * 4;
    s.missing = lists_per_view(b) * b->views_cap + b->missing_stride * 8 * i;
    s.leaf = uint64_t(i) * b->cells_stride * 4;
    return s;
}

/* Streams the previous launch's misses (async mode). */
lv_status process_misses(lv_batch* b)
{
    if (!b->pending)
        return LV_OK;
    lv_ctx* ctx = b->ctx;
    LV_CUDA(ctx, cudaEventSynchronize(b->done));
    b->pending = false;
    const uint32_t* out = b->h_out.as<uint32_t>();
    const uint64_t* miss = reinterpret_cast<const uint64_t*>(
        b->h_out.as<uint8_t>() + sizeof(uint32_t) * (kOutWords * b->views_cap + 64));
    for (uint32_t i = 0; i < b->last.size(); ++i)
    {
        const uint32_t* c = out + kOutWords * i;
        const uint32_t m = std::min<uint32_t>(
            std::min<uint32_t>(c[FC_MISSING], uint32_t(b->missing_stride)),
            b->last[i].desc.max_uploads);
        if (!m)
            continue;
        uint32_t loaded = 0;
        uint64_t bytes = 0;
        lv_status st = stream_bricks(ctx, b->last[i].volume, miss + b->missing_stride * i, m,
                                     b->frame, b->stream, loaded, bytes);
        b->uploaded += loaded;
        b->uploaded_bytes += bytes;
        if (st != LV_OK && st != LV_EAGAIN)
            return st;
    }
    return LV_OK;
}

lv_status fill_params(lv_batch* b, const lv_batch_view* views, uint32_t n, uint32_t n_run,
                      std::vector<Group>& groups, uint32_t& total_roots,
                      uint32_t& tfn_max)
{
    lv_ctx* ctx = b->ctx;
    const ParamLayout PL = param_layout(b->views_cap);
    uint8_t* h = b->h_params.as<uint8_t>();
    LodView* lods = reinterpret_cast<LodView*>(h + PL.lod);
    ResolveView* res = reinterpret_cast<ResolveView*>(h + PL.resolve);
    RayView* rays = reinterpret_cast<RayView*>(h + PL.ray);
    uint8_t* dlists = b->lists.as<uint8_t>();
    uint32_t* dz = b->zeroed.as<uint32_t>();
    uint32_t* dleaf = b->leafs.as<uint32_t>();
    total_roots = 0;
    tfn_max = 0;
    groups.assign(kGroups, Group{});
    for (uint32_t i = 0; i < n; ++i)
    {
        const lv_batch_view& bv = views[i];
        lv_volume* vol = bv.volume;
        const lv_volume_info& info = vol->info;
        const lv_render_desc& d = bv.desc;
        const ViewSlots S = view_slots(b, i);
        uint32_t* counters = dz + kOutWords * i;
        uint32_t* selres = counters + FC_WORDS;
        lv_lod_params lod = d.lod;
        if (lod.window_height == 0)
            lod.window_height = d.height;
        if (!(lod.range[0] == 0.0f && lod.range[1] == 1.0f))
            return fail(ctx, LV_EINVAL, "batched views render the full range {0, 1}");
        if (lod.time_step != vol->time_step)
            return fail(ctx, LV_EINVAL, "batched views render the volume's current time step");
        lv_status st = make_lod_view(ctx, info, d.camera, lod, lods[i]);
        if (st != LV_OK)
            return st;
        lods[i].out_ids = reinterpret_cast<uint64_t*>(dlists + S.visible);
        lods[i].capacity = uint32_t(b->nodes_stride);
        lods[i].result = selres;
        lods[i].root_offset = total_roots;
        total_roots += info.root_blocks[0] * info.root_blocks[1] * info.root_blocks[2];

        uint32_t dims[3];
        const uint32_t Lf = info.depth - 1u;
        for (int a = 0; a < 3; ++a)
            dims[a] = info.root_blocks[a] << Lf;
        ResolveView& R = res[i];
        std::memset(&R, 0, sizeof(R));
        R.visible = lods[i].out_ids;
        R.n_visible_ptr = selres + LV_SEL_WRITTEN;
        R.node_table = vol->node_table.as<int32_t>();
        R.node_stamp = vol->node_stamp.as<uint32_t>();
        R.view_stamp = reinterpret_cast<uint32_t*>(dlists + S.view_stamp);
        R.frame = b->frame;
        R.view_frame = b->launch_id;
        R.depth = info.depth;
        for (int a = 0; a < 3; ++a)
        {
            R.root_blocks[a] = info.root_blocks[a];
            R.dims[a] = dims[a];
        }
        std::memcpy(R.level_offset, vol->level_offset, sizeof(R.level_offset));
        R.synchronous = 0;
        R.render_ids = reinterpret_cast<uint64_t*>(dlists + S.render_ids);
        R.render_slots = reinterpret_cast<uint32_t*>(dlists + S.render_slots);
        R.render_capacity = uint32_t(b->nodes_stride);
        R.missing = reinterpret_cast<uint64_t*>(dlists + S.missing);
        R.missing_capacity = uint32_t(b->missing_stride);
        R.counters = counters;
        R.leaf = dleaf + S.leaf / 4;
        R.Lf = Lf;
        R.n_nodes = vol->n_nodes;

        RayView& V = rays[i];
        st = make_ray_view(ctx, vol, bv.tf, d, lod, bv.d_rgba, R.leaf, counters, V);
        if (st != LV_OK)
            return st;
        tfn_max = std::max(tfn_max, bv.tf->n);
        const int variant = batch_group(V);
        if (variant < kGroups)
            groups[variant].views.push_back(i);
        else if (b->cfg.queue != LV_QUEUE_VIEW_KERNELS)
            return fail(ctx, LV_EINVAL,
                        "the persistent batch kernels render uint8 and uint16 volumes; other "
                        "voxel types need the view-kernel queue");
    }
    /* views [n, n_run) pad the launch to a power of two so a few captured
     * graphs serve every batch size: no roots, no visible nodes, no tiles */
    for (uint32_t i = n; i < n_run; ++i)
    {
        const ViewSlots S = view_slots(b, i);
        uint32_t* counters = dz + kOutWords * i;
        uint32_t* selres = counters + FC_WORDS;
        std::memset(&lods[i], 0, sizeof(LodView));
        lods[i].out_ids = reinterpret_cast<uint64_t*>(dlists + S.visible);
        lods[i].result = selres;
        lods[i].depth = 1;
        lods[i].root_offset = total_roots;
        std::memset(&res[i], 0, sizeof(ResolveView));
        res[i].n_visible_ptr = selres + LV_SEL_WRITTEN;
        res[i].counters = counters;
        res[i].leaf = dleaf + S.leaf / 4;
        res[i].depth = 1;
        std::memset(&rays[i], 0, sizeof(RayView));
        rays[i].counters = counters;
        rays[i].depth = 1;
        rays[i].samples_fixed = 1;
    }
    /* queue tables */
    uint32_t* tables = reinterpret_cast<uint32_t*>(h + PL.tables);
    const uint32_t stride = 2 * b->views_cap + 1;
    for (int g = 0; g < kGroups; ++g)
    {
        uint32_t* ids = tables + stride * g;
        uint32_t* starts = ids + b->views_cap;
        uint32_t acc = 0;
        for (uint32_t k = 0; k < groups[g].views.size(); ++k)
        {
            const uint32_t v = groups[g].views[k];
            ids[k] = v;
            starts[k] = acc;
            const uint32_t tw = b->cfg.tile_w, th = b->cfg.tile_h;
            acc += ((rays[v].W + tw - 1) / tw) * ((rays[v].H + th - 1) / th);
        }
        starts[groups[g].views.size()] = acc;
        groups[g].items = acc;
    }
    uint32_t* counts = tables + stride * kGroups;
    for (int g = 0; g < kGroups; ++g)
        counts[g] = uint32_t(groups[g].views.size());
    counts[kGroups] = total_roots;
    return LV_OK;
}

/* Per-view kernels: each view's tile-order region in view_scratch and the
 * host words and hook arguments of its completion, sized before the launch
 * is enqueued (or captured: nothing here may run inside a capture). */
lv_status prepare_view_kernels(lv_batch* b, uint32_t n)
{
    lv_ctx* ctx = b->ctx;
    const ParamLayout PL = param_layout(b->views_cap);
    const RayView* h_rays = reinterpret_cast<const RayView*>(b->h_params.as<uint8_t>() + PL.ray);
    const lv_render_launch L{LV_LAUNCH_TILE_GRID, b->cfg.tile_w, b->cfg.tile_h, 0,
                             b->cfg.order, b->cfg.lookahead};
    b->view_offs.assign(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i)
        b->view_offs[i + 1] =
            b->view_offs[i] + ((tile_order_bytes(h_rays[i], L) + 255) & ~size_t(255));
    if (b->cfg.order == LV_ORDER_LONGEST_FIRST && b->view_scratch.bytes < b->view_offs[n])
    {
        LV_CUDA(ctx, cudaStreamSynchronize(b->stream));
        LV_CUDA(ctx, b->view_scratch.reserve(b->view_offs[n] + b->view_offs[n] / 2));
    }
    if (b->hook)
    {
        LV_CUDA(ctx, b->h_view_words.reserve(sizeof(uint32_t) * kOutWords * n));
        b->hook_args.resize(n);
        for (uint32_t i = 0; i < n; ++i)
            b->hook_args[i] = lv_batch::HookArg{b, i};
    }
    return LV_OK;
}

/* A timing event on `s`: inside a stream capture it becomes an event-record
 * node of the graph (recorded on every replay), else a plain record. */
cudaError_t record_time(cudaEvent_t e, cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        return cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    return cudaEventRecord(e, s);
}

/* The batch's parameter block from mapped page-locked host memory, by a
 * kernel rather than a copy (as the read-backs below): a copy waiting for
 * its stream would hold up the copy engine's queue. Grid-stride over
 * 16-byte words (the block is 256-byte aligned and sized). */
__global__ void params_from_host_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                        uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

/* Every kernel of a captured batch at the stream priority of the batch's
 * level (the graph is instantiated to run its kernels at their own
 * priorities, not the launch stream's): a server's older batches keep the
 * SM slots first, as without graphs. */
lv_status set_node_priority(lv_batch* b, cudaGraph_t g)
{
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const int high = greatest < least ? greatest + 1 : greatest;
    cudaLaunchAttributeValue v{};
    v.priority = std::min(high + b->prio_level, least);
    size_t n = 0;
    LV_CUDA(b->ctx, cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    LV_CUDA(b->ctx, cudaGraphGetNodes(g, nodes.data(), &n));
    for (cudaGraphNode_t node : nodes)
    {
        cudaGraphNodeType t;
        LV_CUDA(b->ctx, cudaGraphNodeGetType(node, &t));
        if (t == cudaGraphNodeTypeKernel)
            LV_CUDA(b->ctx, cudaGraphKernelNodeSetAttribute(node, cudaLaunchAttributePriority, &v));
    }
    return LV_OK;
}

/* One view's counter words to mapped page-locked host memory by a kernel
 * rather than a copy: a copy waiting for its stream's ray cast holds up the
 * copies queued behind it on the copy engine (other batches' read-backs, a
 * server's admission read-back); a kernel holds up only its own stream. */
__global__ void view_words_to_host_kernel(const uint32_t* __restrict__ src, uint32_t* dst,
                                          uint32_t n)
{
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
    __threadfence_system();
}

/* The batch's counter words and every view's missing list (its first
 * FC_MISSING entries, at most `stride`) to mapped host memory, the same
 * way: CTA v copies view v's list, CTA 0 also the words. */
__global__ void batch_to_host_kernel(const uint32_t* __restrict__ words, uint32_t n_words,
                                     const uint64_t* __restrict__ missing, uint32_t stride,
                                     uint32_t n_views, uint32_t* h_words, uint64_t* h_missing)
{
    const uint32_t v = blockIdx.x;
    if (v == 0)
        for (uint32_t i = threadIdx.x; i < n_words; i += blockDim.x)
            h_words[i] = words[i];
    if (v < n_views)
    {
        const uint32_t k = min(words[kOutWords * v + FC_MISSING], stride);
        for (uint32_t i = threadIdx.x; i < k; i += blockDim.x)
            h_missing[uint64_t(stride) * v + i] = missing[uint64_t(stride) * v + i];
    }
    __threadfence_system();
}

void CUDART_CB view_done_trampoline(void* p)
{
    const auto* a = static_cast<const lv_batch::HookArg*>(p);
    lv_batch* b = a->b;
    if (b->hook)
        b->hook(b->hook_user, a->view, b->h_view_words.as<uint32_t>() + kOutWords * a->view);
}

lv_status enqueue_batch(lv_batch* b, uint32_t n, const std::vector<Group>& groups,
                        uint32_t total_roots, uint32_t tfn_max)
{
    lv_ctx* ctx = b->ctx;
    cudaStream_t s = b->stream;
    const ParamLayout PL = param_layout(b->views_cap);
    uint8_t* d = b->params.as<uint8_t>();
    {
        const uint32_t n16 = uint32_t(PL.bytes / 16);
        params_from_host_kernel<<<std::min<uint32_t>((n16 + 255) / 256, 64u), 256, 0, s>>>(
            static_cast<const uint4*>(b->h_params.dev), reinterpret_cast<uint4*>(d), n16);
        LV_CUDA(ctx, cudaGetLastError());
    }
    LV_CUDA(ctx, cudaMemsetAsync(b->zeroed.ptr, 0, sizeof(uint32_t) * (kOutWords * n + 64), s));
    LV_CUDA(ctx, cudaMemsetAsync(b->leafs.ptr, 0xFF, sizeof(uint32_t) * b->cells_stride * n, s));
    const uint32_t* tables = reinterpret_cast<const uint32_t*>(d + PL.tables);
    const uint32_t stride = 2 * b->views_cap + 1;
    const uint32_t* group_counts = tables + stride * kGroups;
    /* the root frontier is sized for every view having all its roots */
    lv_status st = enqueue_selection(ctx, b->sel, reinterpret_cast<LodView*>(d + PL.lod), n,
                                     total_roots, b->depth_max, s, group_counts + kGroups);
    if (st != LV_OK)
        return st;
    st = launch_views_pipeline(ctx, reinterpret_cast<ResolveView*>(d + PL.resolve),
                               reinterpret_cast<RayView*>(d + PL.ray), n, s);
    if (st != LV_OK)
        return st;
    uint32_t* heads = b->zeroed.as<uint32_t>() + kOutWords * n; /* kGroups words */
    unsigned long long* clock = reinterpret_cast<unsigned long long*>(heads + kGroups);
    const RayView* d_rays = reinterpret_cast<RayView*>(d + PL.ray);
    b->vk_timed = false;
    cudaStream_t* aux = b->aux[b->prio_level];
    if (b->cfg.queue == LV_QUEUE_VIEW_KERNELS)
    {
        /* lv_render's ray cast per view, views spread over the aux streams */
        const RayView* h_rays = reinterpret_cast<const RayView*>(b->h_params.as<uint8_t>() + PL.ray);
        const lv_render_launch L{LV_LAUNCH_TILE_GRID, b->cfg.tile_w, b->cfg.tile_h, 0,
                                 b->cfg.order, b->cfg.lookahead};
        const std::vector<uint64_t>& offs = b->view_offs; /* prepare_view_kernels */
        if (offs.size() < size_t(n) + 1 || (b->hook && b->hook_args.size() < n))
            return fail(ctx, LV_EINVAL, "view-kernel batch not prepared");
        LV_CUDA(ctx, record_time(b->t_vk0, s));
        LV_CUDA(ctx, cudaEventRecord(b->fork, s));
        const uint32_t n_streams = std::min<uint32_t>(n, kViewStreams);
        for (uint32_t k = 0; k < n_streams; ++k)
            LV_CUDA(ctx, cudaStreamWaitEvent(aux[k], b->fork, 0));
        /* the views with the most pixels first, dealt round-robin over the
         * streams: the costliest views start at once instead of queueing
         * behind light ones, which shortens the batch and the latency of
         * its heaviest requests */
        std::vector<uint32_t> by_cost(n);
        for (uint32_t i = 0; i < n; ++i)
            by_cost[i] = i;
        std::stable_sort(by_cost.begin(), by_cost.end(), [&](uint32_t a, uint32_t c) {
            return uint64_t(h_rays[a].W) * h_rays[a].H > uint64_t(h_rays[c].W) * h_rays[c].H;
        });
        for (uint32_t j = 0; j < n; ++j)
        {
            const uint32_t i = by_cost[j];
            if (h_rays[i].W == 0) /* padding view */
                continue;
            uint8_t* scratch = b->cfg.order == LV_ORDER_LONGEST_FIRST
                                   ? b->view_scratch.as<uint8_t>() + offs[i]
                                   : nullptr;
            cudaStream_t vs = aux[j % n_streams];
            st = launch_view_raycast(ctx, h_rays[i], L, scratch, vs);
            if (st != LV_OK)
                return st;
            if (b->hook)
            {
                /* this view is done: its counters to the host, then the hook */
                view_words_to_host_kernel<<<1, 32, 0, vs>>>(
                    b->zeroed.as<uint32_t>() + kOutWords * i,
                    static_cast<uint32_t*>(b->h_view_words.dev) + kOutWords * i, kOutWords);
                LV_CUDA(ctx, cudaGetLastError());
                LV_CUDA(ctx, cudaLaunchHostFunc(vs, view_done_trampoline, &b->hook_args[i]));
            }
        }
        for (uint32_t k = 0; k < n_streams; ++k)
        {
            LV_CUDA(ctx, cudaEventRecord(b->join[k], aux[k]));
            LV_CUDA(ctx, cudaStreamWaitEvent(s, b->join[k], 0));
        }
        LV_CUDA(ctx, record_time(b->t_vk1, s));
        b->vk_timed = true;
    }
    const bool ordered = b->cfg.order == LV_ORDER_LONGEST_FIRST;
    bool first = true;
    if (!b->vk_timed)
        LV_CUDA(ctx, cudaEventRecord(b->fork, s));
    for (int g = 0; g < kGroups && !b->vk_timed; ++g)
    {
        if (groups[g].views.empty())
            continue;
        TileQueue Q;
        Q.view_ids = tables + stride * g;
        Q.tile_start = Q.view_ids + b->views_cap;
        Q.n_views = group_counts + g;
        Q.tile_w = b->cfg.tile_w;
        Q.tile_h = b->cfg.tile_h;
        Q.head = heads + g;
        Q.clock = clock;
        Q.order = nullptr;
        /* the first group on the batch stream, the others each on its own */
        cudaStream_t gs = first ? s : aux[g];
        if (!first)
            LV_CUDA(ctx, cudaStreamWaitEvent(gs, b->fork, 0));
        if (ordered)
        {
            const uint64_t region = order_region_bytes(b->order_cap);
            uint8_t* base = b->order_buf.as<uint8_t>() + region * g;
            uint32_t* hist = reinterpret_cast<uint32_t*>(base);
            uint8_t* keys = base + kOrderHistBytes;
            uint32_t* order = reinterpret_cast<uint32_t*>(keys + order_keys_bytes(b->order_cap));
            st = launch_batch_order(ctx, d_rays, Q, b->order_cap, keys, hist, order, gs);
            if (st != LV_OK)
                return st;
            Q.order = order;
        }
        st = launch_persistent(ctx, g, b->cfg, d_rays, Q, tfn_max, gs);
        if (st != LV_OK)
            return st;
        if (!first)
        {
            LV_CUDA(ctx, cudaEventRecord(b->join[g], gs));
            LV_CUDA(ctx, cudaStreamWaitEvent(s, b->join[g], 0));
        }
        first = false;
    }
    /* counter words and missing lists to the host */
    uint8_t* hmiss =
        static_cast<uint8_t*>(b->h_out.dev) + sizeof(uint32_t) * (kOutWords * b->views_cap + 64);
    batch_to_host_kernel<<<std::max(n, 1u), 128, 0, s>>>(
        b->zeroed.as<uint32_t>(), kOutWords * n + kGroups + 4,
        reinterpret_cast<const uint64_t*>(b->lists.as<uint8_t>() + view_slots(b, 0).missing),
        uint32_t(b->missing_stride), n, static_cast<uint32_t*>(b->h_out.dev),
        reinterpret_cast<uint64_t*>(hmiss));
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

} // namespace

namespace lv
{
void batch_set_priority_level(lv_batch* b, int level)
{
    std::lock_guard<std::mutex> lock(b->ctx->mutex);
    level = std::min(std::max(level, 0), kBatchPriorityLevels - 1);
    /* the streams of a level are created on its first use (only a server
     * uses levels above 0) */
    if (!b->aux[level][0])
    {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        const int high = greatest < least ? greatest + 1 : greatest;
        for (int g = 0; g < kGroups; ++g)
            if (cudaStreamCreateWithPriority(&b->aux[level][g], cudaStreamNonBlocking,
                                             std::min(high + level, least)) != cudaSuccess)
            {
                cudaGetLastError();
                for (int k = 0; k <= g; ++k)
                    if (b->aux[level][k])
                    {
                        cudaStreamDestroy(b->aux[level][k]);
                        b->aux[level][k] = nullptr;
                    }
                return; /* stays at its current level */
            }
    }
    b->prio_level = level;
}

void batch_set_view_hook(lv_batch* b, BatchViewDone fn, void* user)
{
    std::lock_guard<std::mutex> lock(b->ctx->mutex);
    b->hook = fn;
    b->hook_user = user;
}

void batch_decode_stats(const uint32_t* c, lv_frame_stats& s)
{
    const uint32_t* sel = c + FC_WORDS;
    s = lv_frame_stats{};
    s.n_visible = sel[LV_SEL_WRITTEN];
    s.n_visited = sel[LV_SEL_VISITED];
    s.n_rendered = c[FC_KEPT];
    s.n_available = c[FC_AVAILABLE];
    s.n_not_available = c[FC_NOT_AVAILABLE];
    s.max_level = c[FC_MAX_LEVEL] ? c[FC_MAX_LEVEL] - 1u : 0u;
    s.samples_per_ray = c[FC_SAMPLES_PER_RAY];
    s.n_samples = uint64_t(c[FC_SAMPLES_LO]) | (uint64_t(c[FC_SAMPLES_HI]) << 32);
    s.error_flags = c[FC_ERROR];
    s.n_passes = 1;
}
} // namespace lv

/* ================================================================ C ABI */
extern "C" lv_status lv_batch_create(lv_ctx* ctx, lv_batch** out)
{
    if (!ctx || !out)
        return fail(ctx, LV_EINVAL, "null argument");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    lv_status st = ensure_renderer(ctx);
    if (st != LV_OK)
        return st;
    lv_batch* b = new lv_batch();
    b->ctx = ctx;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->user_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t_sel0) != cudaSuccess || cudaEventCreate(&b->t_ray0) != cudaSuccess ||
        cudaEventCreate(&b->t_ray1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t_vk0) != cudaSuccess || cudaEventCreate(&b->t_vk1) != cudaSuccess)
    {
        delete b;
        return fail(ctx, LV_EDEVICE, "batch stream/events");
    }
    /* ray-cast streams from one step below the highest priority (kept for
     * admission work) down, one step per level (a smaller number is a
     * higher priority), clamped to the lowest */
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const int high = greatest < least ? greatest + 1 : greatest;
    for (int g = 0; g < kGroups; ++g)
    {
        /* level 0 now, the others on first use (batch_set_priority_level) */
        const bool ok =
            cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming) == cudaSuccess &&
            cudaStreamCreateWithPriority(&b->aux[0][g], cudaStreamNonBlocking, high) ==
                cudaSuccess;
        if (!ok)
        {
            delete b;
            return fail(ctx, LV_EDEVICE, "batch stream/events");
        }
    }
    *out = b;
    return LV_OK;
}

extern "C" void lv_batch_destroy(lv_batch* b)
{
    if (!b)
        return;
    {
        std::lock_guard<std::mutex> lock(b->ctx->mutex);
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->stream);
    }
    delete b;
}

extern "C" lv_status lv_batch_set_config(lv_batch* b, const lv_batch_config* cfg)
{
    if (!b || !cfg)
        return LV_EINVAL;
    const uint32_t pixels = cfg->tile_w * cfg->tile_h;
    if (cfg->ctas_per_sm > 16)
        return fail(b->ctx, LV_EINVAL, "ctas_per_sm in 0..16");
    if (cfg->queue == LV_QUEUE_CTA_TILES)
    {
        if (pixels == 0 || pixels > 256 || pixels % 32 != 0)
            return fail(b->ctx, LV_EINVAL,
                        "CTA tiles: tile_w * tile_h must be a multiple of 32 up to 256");
    }
    else if (cfg->queue == LV_QUEUE_WARP_REFILL)
    {
        if (pixels < 32 || pixels > 1024 || cfg->samples_per_check == 0 ||
            cfg->samples_per_check > 64 || cfg->tf_shared || cfg->order != LV_ORDER_RASTER)
            return fail(b->ctx, LV_EINVAL,
                        "warp refill: 32..1024 pixels per tile, samples_per_check in 1..64, "
                        "no shared transfer function, raster order");
    }
    else if (cfg->queue == LV_QUEUE_VIEW_KERNELS)
    {
        if (pixels == 0 || pixels > 256 || pixels % 32 != 0 || cfg->tf_shared)
            return fail(b->ctx, LV_EINVAL,
                        "view kernels: tile_w * tile_h a multiple of 32 up to 256, no shared "
                        "transfer function");
    }
    else
        return fail(b->ctx, LV_EINVAL, "unknown queue kind");
    if (cfg->order != LV_ORDER_RASTER && cfg->order != LV_ORDER_LONGEST_FIRST)
        return fail(b->ctx, LV_EINVAL, "unknown tile order");
    if (cfg->lookahead > 1 || (cfg->lookahead && cfg->queue != LV_QUEUE_VIEW_KERNELS))
        return fail(b->ctx, LV_EINVAL, "look-ahead 0 or 1, view kernels only");
    std::lock_guard<std::mutex> lock(b->ctx->mutex);
    b->cfg = *cfg;
    return LV_OK;
}

extern "C" lv_status lv_batch_get_config(const lv_batch* b, lv_batch_config* cfg)
{
    if (!b || !cfg)
        return LV_EINVAL;
    *cfg = b->cfg;
    return LV_OK;
}

extern "C" lv_status lv_batch_render(lv_batch* b, const lv_batch_view* views, uint32_t n,
                                     void* stream)
{
    if (!b || (n && !views))
        return fail(b ? b->ctx : nullptr, LV_EINVAL, "null argument");
    lv_ctx* ctx = b->ctx;
    ++ctx->foreign_pool_use; /* its kernels read pool slots after it returns */
    for (uint32_t i = 0; i < n; ++i)
        if (!views[i].volume || !views[i].tf || !views[i].d_rgba || views[i].volume->ctx != ctx ||
            views[i].tf->ctx != ctx || !views[i].desc.width || !views[i].desc.height)
            return fail(ctx, LV_EINVAL, "invalid batch view");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    b->uploaded = 0;
    b->uploaded_bytes = 0;
    lv_status st = process_misses(b);
    if (st != LV_OK)
        return st;
    if (n == 0)
        return LV_OK;
    /* the host staging is read by the previous launch until it completes */
    LV_CUDA(ctx, cudaEventSynchronize(b->done));
    uint32_t n_run = n;
    const bool graphed = b->cfg.use_graph != 0;
    const bool vk = b->cfg.queue == LV_QUEUE_VIEW_KERNELS;
    if (graphed && !vk)
        while (n_run & (n_run - 1))
            n_run += n_run & (~n_run + 1); /* round up to a power of two */
    st = ensure_regions(b, views, n, user, n_run);
    if (st != LV_OK)
        return st;
    uint64_t frontier = 0;
    for (uint32_t i = 0; i < n; ++i)
        frontier += max_frontier(views[i].volume->info);
    st = reserve_frontier(ctx, b->sel, frontier, b->stream);
    if (st != LV_OK)
        return st;
    if (b->sel.generation != b->sel_generation)
    {
        /* every buffer a cached graph references must still be the same:
         * the frontier queues moved, drop the graphs that used them */
        for (auto& kv : b->graphs)
            cudaGraphExecDestroy(kv.second);
        b->graphs.clear();
        b->sel_generation = b->sel.generation;
    }
    b->frame = ++ctx->renderer->frame;
    ++b->launch_id;
    std::vector<Group> groups;
    uint32_t total_roots = 0, tfn_max = 0;
    st = fill_params(b, views, n, n_run, groups, total_roots, tfn_max);
    if (st != LV_OK)
        return st;
    uint32_t max_items = 0;
    for (const Group& g : groups)
        max_items = std::max(max_items, g.items);
    st = ensure_order(b, max_items);
    if (st != LV_OK)
        return st;
    if (vk && (st = prepare_view_kernels(b, n)) != LV_OK)
        return st;
    if (b->cfg.tf_shared && tfn_max > 2048)
        return fail(ctx, LV_EINVAL, "shared-memory transfer functions hold at most 2048 entries");
    uint32_t mask = 0;
    for (int g = 0; g < kGroups; ++g)
        if (!groups[g].views.empty())
            mask |= 1u << g;
    LV_CUDA(ctx, cudaEventRecord(b->user_ready, user));
    LV_CUDA(ctx, cudaStreamWaitEvent(b->stream, b->user_ready, 0));
    LV_CUDA(ctx, cudaEventRecord(b->t_sel0, b->stream));
    if (graphed)
    {
        const auto key = std::make_tuple(
            n_run, mask, b->cfg.tile_w, b->cfg.tile_h,
            b->cfg.ctas_per_sm | (b->cfg.queue << 8) | (b->cfg.samples_per_check << 16) |
                (b->cfg.order << 24) | (uint32_t(b->prio_level) << 28),
            b->cfg.tf_shared ? tfn_max : 0u, b->depth_max, b->generation,
            uintptr_t(b->sel.generation));
        auto it = b->graphs.find(key);
        /* Persistent kernels read every per-launch value from the copied
         * parameter block, so a cached graph replays as captured. Per-view
         * kernels take their view's constants and grid as launch
         * parameters: the batch is captured on every call and the capture
         * applied to the cached executable graph (cudaGraphExecUpdate), which
         * keeps the instantiated graph while its topology (views, streams,
         * hooks) is unchanged; otherwise the graph is instantiated anew. */
        if (it == b->graphs.end() || vk)
        {
            cudaGraph_t g = nullptr;
            LV_CUDA(ctx, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            st = enqueue_batch(b, n_run, groups, total_roots, tfn_max);
            const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
            if (st != LV_OK)
            {
                if (g)
                    cudaGraphDestroy(g);
                return st;
            }
            LV_CUDA(ctx, ce);
            if (const lv_status ps = set_node_priority(b, g); ps != LV_OK)
            {
                cudaGraphDestroy(g);
                return ps;
            }
            if (it != b->graphs.end())
            {
                cudaGraphExecUpdateResultInfo info{};
                if (cudaGraphExecUpdate(it->second, g, &info) == cudaSuccess)
                    ++b->replays;
                else
                {
                    cudaGetLastError(); /* topology changed: instantiate anew */
                    cudaGraphExecDestroy(it->second);
                    b->graphs.erase(it);
                    it = b->graphs.end();
                }
            }
            if (it == b->graphs.end())
            {
                if (b->graphs.size() >= 32)
                {
                    cudaGraphExecDestroy(b->graphs.begin()->second);
                    b->graphs.erase(b->graphs.begin());
                }
                /* the kernels run at their node priority, the level's
                 * (an update cannot change it: the level is part of the
                 * cache key) */
                cudaGraphExec_t exec = nullptr;
                const cudaError_t ie =
                    cudaGraphInstantiate(&exec, g, cudaGraphInstantiateFlagUseNodePriority);
                if (ie != cudaSuccess)
                {
                    cudaGraphDestroy(g);
                    LV_CUDA(ctx, ie);
                }
                it = b->graphs.emplace(key, exec).first;
                ++b->captures;
            }
            cudaGraphDestroy(g);
        }
        else
            ++b->replays;
        LV_CUDA(ctx, cudaGraphLaunch(it->second, b->stream));
    }
    else
    {
        st = enqueue_batch(b, n, groups, total_roots, tfn_max);
        if (st != LV_OK)
            return st;
    }
    LV_CUDA(ctx, cudaEventRecord(b->t_ray1, b->stream));
    LV_CUDA(ctx, cudaEventRecord(b->done, b->stream));
    LV_CUDA(ctx, cudaStreamWaitEvent(user, b->done, 0));
    b->last_n = n_run;
    b->last.assign(views, views + n);
    b->pending = true;
    /* selection: roots + levels + finish; resolve, prune, leaf, step; per
     * non-empty group one persistent launch (+ key and order passes) */
    const uint32_t per = b->cfg.order == LV_ORDER_LONGEST_FIRST ? 3u : 1u;
    b->launches = b->depth_max + 2u + 4u +
                  (b->cfg.queue == LV_QUEUE_VIEW_KERNELS
                       ? n * per
                       : uint32_t(__builtin_popcount(mask)) * per);
    return LV_OK;
}

extern "C" lv_status lv_batch_stats(lv_batch* b, lv_frame_stats* out, uint32_t n,
                                    float* batch_ms, float* raycast_ms)
{
    if (!b || (n && !out))
        return LV_EINVAL;
    lv_ctx* ctx = b->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaEventSynchronize(b->done));
    const uint32_t m = std::min<uint32_t>(n, uint32_t(b->last.size()));
    const uint32_t* h = b->h_out.as<uint32_t>();
    for (uint32_t i = 0; i < m; ++i)
    {
        lv_frame_stats s;
        batch_decode_stats(h + kOutWords * i, s);
        if (i == 0)
        {
            s.n_uploaded = b->uploaded;
            s.bytes_uploaded = b->uploaded_bytes;
            s.n_launches = b->launches;
        }
        out[i] = s;
    }
    if (batch_ms)
    {
        if (cudaEventElapsedTime(batch_ms, b->t_sel0, b->t_ray1) != cudaSuccess)
        {
            cudaGetLastError();
            *batch_ms = 0.f;
        }
    }
    if (raycast_ms)
    {
        const unsigned long long* clock = reinterpret_cast<const unsigned long long*>(
            h + kOutWords * b->last_n + kGroups);
        *raycast_ms = clock[1] > clock[0] ? float(double(clock[1] - clock[0]) * 1e-6) : 0.f;
        if (b->vk_timed && cudaEventElapsedTime(raycast_ms, b->t_vk0, b->t_vk1) != cudaSuccess)
        {
            cudaGetLastError();
            *raycast_ms = 0.f;
        }
    }
    return LV_OK;
}

extern "C" lv_status lv_batch_graph_stats(lv_batch* b, uint64_t* captures, uint64_t* replays,
                                          uint32_t* cached)
{
    if (!b)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(b->ctx->mutex);
    if (captures)
        *captures = b->captures;
    if (replays)
        *replays = b->replays;
    if (cached)
        *cached = uint32_t(b->graphs.size());
    return LV_OK;
}

extern "C" lv_status lv_batch_autotune(lv_batch* b, const lv_batch_view* views, uint32_t n,
                                       void* stream, uint32_t reps, lv_batch_config* chosen)
{
    if (!b || !views || n == 0)
        return LV_EINVAL;
    /* CTA tiles: 6 tile shapes x TF staging x order, resident grid; view
     * kernels: 2 tile shapes x order x look-ahead; warp refill: 4 tile sizes
     * x 3 refill intervals */
    static const uint32_t cta_shapes[][2] = {{8, 8}, {16, 8}, {8, 16}, {16, 16}, {32, 4}, {32, 8}};
    static const uint32_t warp_shapes[][2] = {{8, 4}, {8, 8}, {16, 8}, {16, 16}};
    static const uint32_t checks[] = {2, 8, 32};
    std::vector<lv_batch_config> cands;
    const lv_batch_config start = b->cfg;
    for (const auto& sh : cta_shapes)
        for (uint32_t tfs = 0; tfs < 2; ++tfs)
            for (uint32_t ord = 0; ord < 2; ++ord)
            {
                lv_batch_config c = start;
                c.queue = LV_QUEUE_CTA_TILES;
                c.tile_w = sh[0];
                c.tile_h = sh[1];
                c.ctas_per_sm = 0;
                c.tf_shared = tfs;
                c.samples_per_check = 8;
                c.order = ord;
                c.lookahead = 0;
                cands.push_back(c);
            }
    static const uint32_t view_shapes[][2] = {{8, 8}, {8, 16}};
    for (const auto& sh : view_shapes)
        for (uint32_t ord = 0; ord < 2; ++ord)
            for (uint32_t la = 0; la < 2; ++la)
            {
                lv_batch_config c = start;
                c.queue = LV_QUEUE_VIEW_KERNELS;
                c.tile_w = sh[0];
                c.tile_h = sh[1];
                c.ctas_per_sm = 0;
                c.tf_shared = 0;
                c.samples_per_check = 8;
                c.order = ord;
                c.lookahead = la;
                cands.push_back(c);
            }
    for (const auto& sh : warp_shapes)
        for (uint32_t k : checks)
        {
            lv_batch_config c = start;
            c.queue = LV_QUEUE_WARP_REFILL;
            c.tile_w = sh[0];
            c.tile_h = sh[1];
            c.ctas_per_sm = 0;
            c.tf_shared = 0;
            c.samples_per_check = k;
            c.order = LV_ORDER_RASTER;
            c.lookahead = 0;
            cands.push_back(c);
        }
    lv_batch_config best = start;
    float best_ms = 1e30f;
    reps = reps ? reps : 3;
    b->tune_cfgs.clear();
    b->tune_ms.clear();
    for (const lv_batch_config& cfg : cands)
    {
        if (lv_batch_set_config(b, &cfg) != LV_OK)
            continue;
        float total = 0.f;
        bool ok = true;
        for (uint32_t r = 0; r <= reps && ok; ++r)
        {
            if (lv_batch_render(b, views, n, stream) != LV_OK)
            {
                ok = false;
                break;
            }
            float all = 0.f, ray = 0.f;
            lv_batch_stats(b, nullptr, 0, &all, &ray);
            if (r > 0)
                total += ray;
        }
        if (ok)
        {
            b->tune_cfgs.push_back(cfg);
            b->tune_ms.push_back(total / reps);
        }
        if (ok && total / reps < best_ms)
        {
            best_ms = total / reps;
            best = cfg;
        }
    }
    lv_batch_set_config(b, &best);
    if (chosen)
        *chosen = best;
    return best_ms < 1e30f ? LV_OK : fail(b->ctx, LV_EINVAL, "no configuration ran");
}

extern "C" lv_status lv_batch_autotune_results(const lv_batch* b, lv_batch_config* configs,
                                               float* raycast_ms, uint32_t capacity,
                                               uint32_t* n)
{
    if (!b || !n || (capacity && (!configs || !raycast_ms)))
        return LV_EINVAL;
    *n = uint32_t(b->tune_cfgs.size());
    const uint32_t k = std::min<uint32_t>(capacity, *n);
    for (uint32_t i = 0; i < k; ++i)
    {
        configs[i] = b->tune_cfgs[i];
        raycast_ms[i] = b->tune_ms[i];
    }
    return LV_OK;
}
