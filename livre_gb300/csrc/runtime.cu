/*
 * Host runtime of livre_gb300: context, HBM brick pool with LRU residency,
 * volumes and their data sources, transfer functions and the per-view frame
 * (select -> resolve -> stream misses -> leaf grid -> ray cast).
 *
 * Reference counterparts (paths inside BlueBrain/Livre):
 *  - brick pool + residency: TexturePool (livre/core/render/TexturePool.cpp:
 *    33-126), CacheT<TextureObject> with LRUCachePolicy (livre/core/cache/
 *    Cache.cpp:41-209), TextureObject upload (livre/lib/cache/
 *    TextureObject.cpp:76-120), DataUploadFilter (livre/lib/pipeline/
 *    DataUploadFilter.cpp:45-123);
 *  - frame: RenderPipeline::renderSync / renderAsync (livre/lib/pipeline/
 *    RenderPipeline.cpp:92-225) and Renderer::render (livre/core/render/
 *    Renderer.cpp:33-47).
 *
 * LRU semantics kept from the reference cache: residency order is load
 * order (a hit does not refresh it, Cache.cpp:111-123); when the pool is
 * full the oldest brick not in use by the frame being built is evicted
 * (objects still referenced are skipped, Cache.cpp:141-156).
 */
#include <chrono>
#include <algorithm>
#include <cmath>
#include <limits>
#include <list>
#include <map>
#include <functional>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "lv_runtime.h"

namespace lv
{
struct Blob
{
    float cx, cy, cz, inv2s2, cut2, amp;
};
std::vector<Blob> make_blobs(const lv_volume_info& v, const lv_blob_desc& d);
lv_status launch_blob_bricks(lv_ctx* ctx, const lv_volume_info& v,
                             const lv_blob_desc& d, const Blob* d_blobs,
                             const uint64_t* d_ids, uint32_t n, uint8_t* out,
                             const uint64_t* d_offsets, cudaStream_t stream);
lv_status launch_resolve(lv_ctx* ctx, const ResolveView& R, cudaStream_t s);
lv_status launch_leaf_fill(lv_ctx* ctx, const ResolveView& R, cudaStream_t s);
lv_status launch_raycast(lv_ctx* ctx, const RayView& V, cudaStream_t s);

namespace
{
__global__ void scatter_kernel(int32_t* __restrict__ table,
                               const int64_t* __restrict__ pairs, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        table[pairs[2 * i]] = int32_t(pairs[2 * i + 1]);
}

/* Copies a few result words into mapped page-locked host memory. A frame's
 * counters reach the host this way rather than by a copy-engine transfer: a
 * small copy queued behind a large one (the application's copy of the last
 * frame, say) would hold up the stream, and with it the frame's ray cast,
 * until the large one ends. */
__global__ void words_to_host_kernel(const uint32_t* __restrict__ src, uint32_t* dst, uint32_t n)
{
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
    __threadfence_system();
}

/* A synchronous frame's counters and its missing list (as many ids as the
 * residency pass appended, at most cap) into mapped page-locked host
 * memory: the host learns which bricks to stream when it learns how many,
 * without a copy queued behind the frame's first ray cast. */
__global__ void counters_to_host_kernel(const uint32_t* __restrict__ counters,
                                        const uint64_t* __restrict__ missing, uint32_t* words,
                                        uint64_t* ids, uint32_t cap)
{
    const uint32_t n = min(counters[FC_MISSING], cap);
    if (blockIdx.x == 0 && threadIdx.x < FC_WORDS)
        words[threadIdx.x] = counters[threadIdx.x];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        ids[i] = missing[i];
    __threadfence_system();
}

/* Voxel quads (quad_layout) of elements [j0, j0 + m) of a uint8 brick with
 * rows of n0 voxels and slices of n1 rows, from its canonical bytes c[i] =
 * byte j0 + i for i < min(voxels - j0, m + n0 + 1) (the elements' own bytes,
 * then one row and one byte more: every neighbour a quad takes), written as
 * 32-bit elements at q[j0 ..]. j0 is a multiple of 4 and q 16-byte aligned:
 * four elements per 16-byte store. A neighbour past the end of a row or
 * slice is the voxel itself. */
__device__ __forceinline__ void quads_from_bytes(const uint8_t* c, uint32_t* q, uint32_t j0,
                                                 uint32_t m, uint32_t n0, uint32_t n1)
{
    for (uint32_t k = 4u * threadIdx.x; k < m; k += 4u * blockDim.x)
    {
        uint32_t x = (j0 + k) % n0, y = ((j0 + k) / n0) % n1;
        uint32_t e[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (uint32_t t = 0; t < 4; ++t)
        {
            const uint32_t i = k + t;
            if (i < m)
            {
                const bool xr = x + 1u < n0, yr = y + 1u < n1;
                const uint32_t b0 = c[i];
                const uint32_t b1 = xr ? c[i + 1] : b0;
                const uint32_t b2 = yr ? c[i + n0] : b0;
                const uint32_t b3 = xr && yr ? c[i + n0 + 1] : xr ? b1 : b2;
                e[t] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
            }
            if (++x == n0)
            {
                x = 0u;
                y = y + 1u == n1 ? 0u : y + 1u;
            }
        }
        if (k + 4u <= m)
            *reinterpret_cast<uint4*>(q + j0 + k) = make_uint4(e[0], e[1], e[2], e[3]);
        else
            for (uint32_t t = 0; k + t < m; ++t)
                q[j0 + k + t] = e[t];
    }
}

/* Elements a block turns into quads per pass, and the canonical bytes it
 * stages for them (one row of at most kQuadMaxRow voxels and one byte more,
 * rounded up to whole 8-byte words). */
constexpr uint32_t kQuadRun = 4096;
constexpr uint32_t kQuadStage = kQuadRun + kQuadMaxRow + 8;

/* Expands uint8 bricks into voxel quads in place (quad_layout). Block b
 * takes the slot at arena + offsets[b], whose canonical bytes (`voxels` of
 * them, x fastest, rows of n0, slices of n1 rows) are at slot + stage_off,
 * stage_off >= 3 * voxels and 256-byte aligned. The block takes runs of
 * elements in increasing order, staging a run's canonical bytes (and the
 * row after them) in shared memory before any of its writes; the run ending
 * at element j writes slot bytes below 4j <= stage_off + j, so no later run
 * finds a canonical byte replaced. */
constexpr uint32_t kExpandThreads = 512;

__global__ void __launch_bounds__(kExpandThreads)
    expand_quads_kernel(uint8_t* __restrict__ arena, const uint64_t* __restrict__ offsets,
                        uint32_t n0, uint32_t n1, uint32_t voxels, uint32_t stage_off)
{
    __shared__ uint32_t s_c[kQuadStage / 4];
    uint8_t* sb = reinterpret_cast<uint8_t*>(s_c);
    uint8_t* slot = arena + offsets[blockIdx.x];
    const uint8_t* canon = slot + stage_off;
    for (uint32_t j0 = 0; j0 < voxels; j0 += kQuadRun)
    {
        const uint32_t m = min(kQuadRun, voxels - j0);
        const uint32_t L = min(voxels - j0, m + n0 + 1u);
        /* canon + j0 is 4-byte aligned (stage_off 256-aligned, j0 a
         * multiple of kQuadRun) */
        const uint32_t* cw = reinterpret_cast<const uint32_t*>(canon + j0);
        for (uint32_t i = threadIdx.x; i < L / 4u; i += blockDim.x)
            s_c[i] = cw[i];
        for (uint32_t i = (L / 4u) * 4u + threadIdx.x; i < L; i += blockDim.x)
            sb[i] = canon[j0 + i];
        __syncthreads(); /* the run staged before any of its writes */
        quads_from_bytes(sb, reinterpret_cast<uint32_t*>(slot), j0, m, n0, n1);
        __syncthreads(); /* the run written before the next one is staged */
    }
}

/* Copies bricks from mapped page-locked host memory straight into their
 * slots, in the pool's layout: voxel quads (quads != 0) or the bytes as they
 * are. One kernel reads every missing brick of a frame over the host link
 * at once, where a copy-engine transfer per brick (and an expansion pass
 * after it) costs a transfer's set-up per brick. Brick blockIdx.x is read at
 * src + offs[2b] and written at arena + offs[2b + 1] (a slot, 1 KiB
 * aligned); gridDim.y blocks share a brick, each a run of whole 8-byte
 * words. `bytes` is a multiple of 8 and every source offset a multiple of
 * `bytes`, so every word load is 8-byte aligned. For quads a block stages a
 * run's canonical bytes and the row after them in shared memory. */
constexpr uint32_t kGatherThreads = 256;

__global__ void __launch_bounds__(kGatherThreads)
    gather_bricks_kernel(uint8_t* __restrict__ arena, const uint8_t* __restrict__ src,
                         const uint64_t* __restrict__ offs, uint32_t bytes, uint32_t n0,
                         uint32_t n1, uint32_t quads)
{
    __shared__ uint2 s_w[kQuadStage / 8];
    const uint8_t* s = src + offs[2 * blockIdx.x];
    uint8_t* d = arena + offs[2 * blockIdx.x + 1];
    const uint32_t words = bytes / 8;
    const uint32_t per = (words + gridDim.y - 1) / gridDim.y;
    const uint32_t w0 = min(words, blockIdx.y * per), w1 = min(words, w0 + per);
    if (!quads)
    {
        for (uint32_t w = w0 + threadIdx.x; w < w1; w += kGatherThreads)
            *reinterpret_cast<uint2*>(d + 8ull * w) = *reinterpret_cast<const uint2*>(s + 8ull * w);
        return;
    }
    const uint32_t j1 = 8u * w1;
    for (uint32_t j0 = 8u * w0; j0 < j1; j0 += kQuadRun)
    {
        const uint32_t m = min(kQuadRun, j1 - j0);
        /* bytes - j0 is a multiple of 8, so whole words stay in the brick */
        const uint32_t nw = (min(bytes - j0, m + n0 + 1u) + 7u) / 8u;
        for (uint32_t i = threadIdx.x; i < nw; i += kGatherThreads)
            s_w[i] = *reinterpret_cast<const uint2*>(s + j0 + 8ull * i);
        __syncthreads();
        quads_from_bytes(reinterpret_cast<const uint8_t*>(s_w), reinterpret_cast<uint32_t*>(d), j0,
                         m, n0, n1);
        __syncthreads();
    }
}

lv_status words_to_host(lv_ctx* ctx, const void* d_src, const PinnedBuffer& host,
                        size_t word_offset, uint32_t n, cudaStream_t s)
{
    words_to_host_kernel<<<1, 32, 0, s>>>(static_cast<const uint32_t*>(d_src),
                                          static_cast<uint32_t*>(host.dev) + word_offset, n);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

/* The visible nodes of a frame queued while the previous frame still ray
 * casts: the ones not resident are collected (to stream beside that ray
 * cast), the resident ones stamped with the frame so that eviction spares
 * them. */
__global__ void probe_kernel(const __grid_constant__ ResolveView RV, uint64_t* __restrict__ out,
                             uint32_t* __restrict__ out_count, uint32_t capacity)
{
    const uint32_t n = *RV.n_visible_ptr;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint64_t id = RV.visible[i];
        if (nid_level(id) >= RV.depth)
            continue;
        const uint64_t idx = node_index(RV.level_offset, RV.root_blocks, id);
        if (idx >= RV.n_nodes)
            continue;
        if (RV.node_table[idx] >= 0)
            RV.node_stamp[idx] = RV.frame;
        else
        {
            const uint32_t k = atomicAdd(out_count, 1u);
            if (k < capacity)
                out[k] = id;
        }
    }
}

__global__ void fill_i32_kernel(int32_t* p, uint64_t n, int32_t v)
{
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        p[i] = v;
}

uint64_t round_units(uint64_t bytes)
{
    return (bytes + kSlotUnit - 1) / kSlotUnit;
}
} // namespace

} // namespace lv

namespace lv
{
uint32_t bytes_per_voxel(uint32_t dt)
{
    switch (dt)
    {
    case LV_DT_UINT8:
    case LV_DT_INT8:
        return 1;
    case LV_DT_UINT16:
    case LV_DT_INT16:
        return 2;
    case LV_DT_FLOAT:
    case LV_DT_UINT32:
    case LV_DT_INT32:
        return 4;
    default:
        return 0;
    }
}

/* dataSourceRange of a voxel type: its numeric_limits min and max
 * (RayCastRenderer.cpp:236-277; for float, the smallest positive normal and
 * the largest finite value, as the reference has it). */
void type_range(uint32_t dt, float& lo, float& hi)
{
    switch (dt)
    {
    case LV_DT_UINT16: lo = 0.0f; hi = 65535.0f; break;
    case LV_DT_UINT32: lo = 0.0f; hi = 4294967295.0f; break;
    case LV_DT_INT8: lo = -128.0f; hi = 127.0f; break;
    case LV_DT_INT16: lo = -32768.0f; hi = 32767.0f; break;
    case LV_DT_INT32: lo = -2147483648.0f; hi = 2147483647.0f; break;
    case LV_DT_FLOAT: lo = 1.17549435e-38f; hi = 3.40282347e+38f; break;
    default: lo = 0.0f; hi = 255.0f; break;
    }
}

lv_status ensure_pool(lv_ctx* ctx)
{
    if (ctx->pool)
        return LV_OK;
    Pool* p = new Pool();
    const uint64_t units = ctx->pool_bytes / kSlotUnit;
    if (units == 0 || units > (uint64_t(1) << kLeafSlotBits))
    {
        delete p;
        return fail(ctx, LV_EINVAL, "pool size must be in (0, 128 GiB]");
    }
    cudaError_t e = p->arena.reserve(units * kSlotUnit);
    if (e != cudaSuccess)
    {
        delete p;
        return cuda_fail(ctx, e, "brick pool allocation");
    }
    p->capacity_units = units;
    ctx->pool = p;
    return LV_OK;
}

lv_status ensure_renderer(lv_ctx* ctx)
{
    if (ctx->renderer)
        return LV_OK;
    Renderer* r = new Renderer();
    cudaEventCreateWithFlags(&r->pending_event, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->render_event, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->upload_event, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->expand_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->gather_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->frame_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->resolve_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->join, cudaEventDisableTiming);
    cudaStreamCreateWithFlags(&r->side, cudaStreamNonBlocking);
    {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        cudaStreamCreateWithPriority(&r->sel_stream, cudaStreamNonBlocking, greatest);
    }
    cudaEventCreateWithFlags(&r->sel_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&r->visible_free, cudaEventDisableTiming);
    cudaEventCreate(&r->t_sel0);
    cudaEventCreate(&r->t_sel1);
    cudaEventCreate(&r->t_ray0);
    cudaEventCreate(&r->t_ray1);
    ctx->renderer = r;
    LV_CUDA(ctx, r->sel_result.reserve(sizeof(uint32_t) * LV_SELECT_RESULT_WORDS));
    LV_CUDA(ctx, r->counters.reserve(sizeof(uint32_t) * FC_WORDS));
    LV_CUDA(ctx, r->h_counters.reserve(sizeof(uint32_t) * (FC_WORDS + LV_SELECT_RESULT_WORDS)));
    return LV_OK;
}

lv_status reserve_selection(lv_ctx* ctx, const lv_volume_info& info,
                            cudaStream_t s)
{
    return reserve_frontier(ctx, ctx->sel, max_frontier(info), s);
}

/* Frees one slot of `units` for a new brick, evicting the oldest resident
 * brick of the same size that is not in use (stamp < protect_frame).
 * Returns false when every candidate is in use. */
bool pool_alloc(lv_ctx* ctx, uint32_t units, uint32_t protect_frame,
                std::unordered_map<lv_volume*, std::vector<uint32_t>>& stamps,
                std::vector<std::pair<lv_volume*, std::pair<uint64_t, int32_t>>>& updates,
                uint32_t& out_unit, cudaStream_t stamp_stream)
{
    Pool& P = *ctx->pool;
    auto& fl = P.free_by_units[units];
    if (!fl.empty())
    {
        out_unit = fl.back();
        fl.pop_back();
        return true;
    }
    if (P.bump + units <= P.capacity_units)
    {
        out_unit = uint32_t(P.bump);
        P.bump += units;
        return true;
    }
    for (auto it = P.lru.begin(); it != P.lru.end(); ++it)
    {
        /* a brick placed by this very call is not stamped yet, and evicting
         * it would leave the call's page-table updates naming one node twice */
        if (it->units != units || it->load == P.loads)
            continue;
        lv_volume* v = it->vol;
        if (protect_frame == 0xFFFFFFFFu)
        {
            /* pins alone decide (server requests) */
            if (!v->pins.empty() && v->pins[it->node_idx] != 0)
                continue;
            out_unit = it->unit;
            v->host_table[it->node_idx] = -1;
            updates.push_back({v, {it->node_idx, -1}});
            P.resident_bytes -= uint64_t(units) * kSlotUnit;
            --P.resident_count[units];
            P.lru.erase(it);
            return true;
        }
        auto st = stamps.find(v);
        if (st == stamps.end())
        {
            std::vector<uint32_t> h(v->n_nodes);
            /* on a stream of the library's own when a frame may still run on
             * the caller's (the legacy default stream would wait for it) */
            if (stamp_stream)
            {
                if (cudaMemcpyAsync(h.data(), v->node_stamp.ptr, sizeof(uint32_t) * v->n_nodes,
                                    cudaMemcpyDeviceToHost, stamp_stream) != cudaSuccess ||
                    cudaStreamSynchronize(stamp_stream) != cudaSuccess)
                    return false;
            }
            else if (cudaMemcpy(h.data(), v->node_stamp.ptr, sizeof(uint32_t) * v->n_nodes,
                                cudaMemcpyDeviceToHost) != cudaSuccess)
                return false;
            st = stamps.emplace(v, std::move(h)).first;
        }
        const uint32_t stamp = st->second[it->node_idx];
        if ((stamp != 0 && stamp >= protect_frame) ||
            (!v->pins.empty() && v->pins[it->node_idx] != 0))
            continue; /* in use: Cache.cpp:148 skips referenced objects */
        out_unit = it->unit;
        v->host_table[it->node_idx] = -1;
        updates.push_back({v, {it->node_idx, -1}});
        P.resident_bytes -= uint64_t(units) * kSlotUnit;
        --P.resident_count[units];
        P.lru.erase(it);
        return true;
    }
    return false;
}

lv_status apply_updates(
    lv_ctx* ctx,
    std::vector<std::pair<lv_volume*, std::pair<uint64_t, int32_t>>>& updates,
    cudaStream_t s)
{
    if (updates.empty())
        return LV_OK;
    Renderer& R = *ctx->renderer;
    /* one pair per node, its last value: the scatter writes the pairs in no
     * particular order */
    std::map<lv_volume*, std::map<uint64_t, int32_t>> last;
    for (auto& u : updates)
        last[u.first][u.second.first] = u.second.second;
    std::map<lv_volume*, std::vector<int64_t>> per;
    for (auto& kv : last)
        for (auto& e : kv.second)
        {
            per[kv.first].push_back(int64_t(e.first));
            per[kv.first].push_back(int64_t(e.second));
        }
    size_t total = 0;
    for (auto& kv : per)
        total += kv.second.size();
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    LV_CUDA(ctx, R.h_pairs.reserve(sizeof(int64_t) * total));
    LV_CUDA(ctx, R.pairs.reserve(sizeof(int64_t) * total));
    size_t off = 0;
    for (auto& kv : per)
    {
        std::memcpy(R.h_pairs.as<int64_t>() + off, kv.second.data(),
                    sizeof(int64_t) * kv.second.size());
        off += kv.second.size();
    }
    LV_CUDA(ctx, cudaMemcpyAsync(R.pairs.ptr, R.h_pairs.ptr, sizeof(int64_t) * total,
                                 cudaMemcpyHostToDevice, s));
    off = 0;
    for (auto& kv : per)
    {
        const uint32_t n = uint32_t(kv.second.size() / 2);
        scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(
            kv.first->node_table.as<int32_t>(), R.pairs.as<int64_t>() + off, n);
        off += kv.second.size();
    }
    LV_CUDA(ctx, cudaGetLastError());
    updates.clear();
    return LV_OK;
}

/* The context's host fetchers: one worker per hardware thread but the
 * caller's, at most 63 (created on first use, under the context lock). */
HostPool* host_pool(lv_ctx* ctx)
{
    if (!ctx->host_pool)
    {
        const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
        ctx->host_pool = new HostPool(std::min(hw, 64u) - 1u);
    }
    return ctx->host_pool;
}

/* Streams bricks `ids` of `vol` into the pool (DataUploadFilter::load):
 * allocate / evict, fetch from the source, copy on the upload stream, then
 * publish the node-table entries; `render` waits for all of it. Callback
 * sources are fetched in groups of half the staging ring, by up to
 * fetch_threads host threads at once, while the previous group copies. */
lv_status stream_bricks(lv_ctx* ctx, lv_volume* vol, const uint64_t* ids,
                        uint32_t n, uint32_t protect_frame, cudaStream_t render,
                        uint32_t& n_loaded, uint64_t& bytes_loaded, bool beside_frame)
{
    Renderer& R = *ctx->renderer;
    Pool& P = *ctx->pool;
    cudaStream_t up = ctx->upload_stream;
    n_loaded = 0;
    bytes_loaded = 0;
    if (n == 0)
        return LV_OK;
    ++P.loads;
    /* new copies may overwrite evicted slots still read by queued work: the
     * caller's stream and the last lv_render frame (on any stream) */
    if (!beside_frame)
    {
        LV_CUDA(ctx, cudaEventRecord(R.render_event, render));
        LV_CUDA(ctx, cudaStreamWaitEvent(up, R.render_event, 0));
        if (R.have_last)
            LV_CUDA(ctx, cudaStreamWaitEvent(up, R.frame_done, 0));
    }
    const cudaStream_t stamp_stream = beside_frame ? R.sel_stream : nullptr;
    std::unordered_map<lv_volume*, std::vector<uint32_t>> stamps;
    std::vector<std::pair<lv_volume*, std::pair<uint64_t, int32_t>>> updates;
    std::vector<uint64_t> gen_ids, gen_offsets;
    std::vector<uint64_t> expand; /* slots to expand into voxel quads */
    /* host-store bricks read by gather_bricks_kernel: (source, slot) offsets */
    std::vector<uint64_t> gather;
    const bool gathered = vol->kind == SRC_BLOB_HOST && vol->brick_bytes % 8 == 0;
    uint8_t* arena = P.arena.as<uint8_t>();
    lv_status st = LV_OK;
    /* the bookkeeping of a brick placed in `unit` */
    const auto place = [&](uint64_t idx, uint32_t unit) {
        vol->host_table[idx] = int32_t(unit);
        updates.push_back({vol, {idx, int32_t(unit)}});
        P.lru.push_back(Resident{vol, idx, unit, vol->slot_units, P.loads});
        P.resident_bytes += uint64_t(vol->slot_units) * kSlotUnit;
        ++P.resident_count[vol->slot_units];
        ++n_loaded;
    };
    if (vol->kind == SRC_CALLBACK)
    {
        /* first occurrences of the bricks that are not resident */
        std::vector<std::pair<uint64_t, uint64_t>> todo; /* (id, table index) */
        std::unordered_set<uint64_t> seen;
        for (uint32_t i = 0; i < n; ++i)
        {
            if (nid_level(ids[i]) >= vol->info.depth)
                continue;
            const uint64_t idx = node_index(vol->level_offset, vol->info.root_blocks, ids[i]);
            if (idx < vol->n_nodes && vol->host_table[idx] < 0 && seen.insert(idx).second)
                todo.push_back({ids[i], idx});
        }
        const size_t ring_n = vol->staging.size();
        const size_t group = std::max<size_t>(1, ring_n / 2);
        const uint32_t threads = std::max(1u, vol->fetch_threads);
        HostPool* pool = threads > 1 ? host_pool(ctx) : nullptr;
        std::vector<int> rc(group);
        size_t ring = 0;
        for (size_t g0 = 0; g0 < todo.size() && st == LV_OK; g0 += group)
        {
            const size_t m = std::min(group, todo.size() - g0);
            /* these staging buffers are free once their last copies ended */
            for (size_t j = 0; j < m; ++j)
                LV_CUDA(ctx, cudaEventSynchronize(vol->staging_ev[(ring + j) % ring_n]));
            const std::function<void(uint32_t)> fetch = [&](uint32_t j) {
                rc[j] = vol->fn(vol->user, todo[g0 + j].first,
                                vol->staging[(ring + j) % ring_n]->ptr, vol->brick_bytes);
            };
            if (pool)
                pool->parallel_for(uint32_t(m), threads, fetch);
            else
                for (uint32_t j = 0; j < uint32_t(m); ++j)
                    fetch(j);
            for (size_t j = 0; j < m; ++j)
            {
                /* null MemoryUnitPtr: the brick is skipped
                 * (DataUploadFilter.cpp:56-64) */
                if (rc[j] != 0)
                    continue;
                uint32_t unit = 0;
                if (!pool_alloc(ctx, vol->slot_units, protect_frame, stamps, updates, unit,
                                stamp_stream))
                {
                    st = fail(ctx, LV_EAGAIN, "brick pool full of bricks in use");
                    break;
                }
                const size_t slot = (ring + j) % ring_n;
                LV_CUDA(ctx, cudaMemcpyAsync(arena + uint64_t(unit) * kSlotUnit + vol->stage_off,
                                             vol->staging[slot]->ptr, vol->brick_bytes,
                                             cudaMemcpyHostToDevice, up));
                if (vol->stage_off)
                    expand.push_back(uint64_t(unit) * kSlotUnit);
                LV_CUDA(ctx, cudaEventRecord(vol->staging_ev[slot], up));
                bytes_loaded += vol->brick_bytes;
                place(todo[g0 + j].second, unit);
            }
            ring = (ring + m) % ring_n;
        }
    }
    else
        for (uint32_t i = 0; i < n; ++i)
        {
            const uint64_t id = ids[i];
            if (nid_level(id) >= vol->info.depth)
                continue;
            const uint64_t idx = node_index(vol->level_offset, vol->info.root_blocks, id);
            if (idx >= vol->n_nodes || vol->host_table[idx] >= 0)
                continue;
            uint32_t unit = 0;
            if (!pool_alloc(ctx, vol->slot_units, protect_frame, stamps, updates, unit,
                                stamp_stream))
            {
                st = fail(ctx, LV_EAGAIN, "brick pool full of bricks in use");
                break;
            }
            if (gathered)
            {
                gather.push_back(idx * vol->brick_bytes);
                gather.push_back(uint64_t(unit) * kSlotUnit);
                bytes_loaded += vol->brick_bytes;
            }
            else if (vol->kind == SRC_BLOB_HOST)
            {
                const uint8_t* src = vol->host_store.as<uint8_t>() + idx * vol->brick_bytes;
                LV_CUDA(ctx, cudaMemcpyAsync(arena + uint64_t(unit) * kSlotUnit + vol->stage_off,
                                             src, vol->brick_bytes, cudaMemcpyHostToDevice, up));
                bytes_loaded += vol->brick_bytes;
            }
            else /* generated on the device below */
            {
                gen_ids.push_back(id);
                gen_offsets.push_back(uint64_t(unit) * kSlotUnit + vol->stage_off);
            }
            if (vol->stage_off && !gathered)
                expand.push_back(uint64_t(unit) * kSlotUnit);
            place(idx, unit);
        }
    if (!gen_ids.empty())
    {
        /* grow-only buffers: freeing device memory would wait for the whole
         * device, a frame still ray casting included */
        DeviceBuffer& dids = R.gen;
        PinnedBuffer& h = R.h_gen;
        LV_CUDA(ctx, cudaStreamSynchronize(up)); /* the last generation read them */
        LV_CUDA(ctx, dids.reserve(sizeof(uint64_t) * 2 * gen_ids.size()));
        LV_CUDA(ctx, h.reserve(sizeof(uint64_t) * 2 * gen_ids.size()));
        std::memcpy(h.ptr, gen_ids.data(), sizeof(uint64_t) * gen_ids.size());
        std::memcpy(h.as<uint64_t>() + gen_ids.size(), gen_offsets.data(),
                    sizeof(uint64_t) * gen_offsets.size());
        LV_CUDA(ctx, cudaMemcpyAsync(dids.ptr, h.ptr, sizeof(uint64_t) * 2 * gen_ids.size(),
                                     cudaMemcpyHostToDevice, up));
        lv_status g =
            vol->kind == SRC_FBM_DEVICE
                ? launch_fbm_bricks(ctx, vol->info, vol->fbm, vol->d_perm.as<uint16_t>(),
                                    dids.as<uint64_t>(), uint32_t(gen_ids.size()), arena,
                                    dids.as<uint64_t>() + gen_ids.size(), vol->brick_bytes, up)
                : launch_blob_bricks(ctx, vol->info, vol->blob, vol->d_blobs.as<Blob>(),
                                     dids.as<uint64_t>(), uint32_t(gen_ids.size()), arena,
                                     dids.as<uint64_t>() + gen_ids.size(), up);
        if (g != LV_OK)
            return g;
    }
    if (!gather.empty())
    {
        /* the offsets' buffer is read by the previous gather until it ends */
        if (R.gather_recorded)
            LV_CUDA(ctx, cudaEventSynchronize(R.gather_done));
        LV_CUDA(ctx, R.h_gather.reserve(sizeof(uint64_t) * gather.size()));
        std::memcpy(R.h_gather.ptr, gather.data(), sizeof(uint64_t) * gather.size());
        const uint32_t nb = uint32_t(gather.size() / 2);
        /* about four blocks per SM in all, at least one pass per block */
        int sms = 0;
        LV_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
        const uint32_t words = uint32_t(vol->brick_bytes / 8);
        const uint32_t split = std::max(
            1u, std::min((4u * uint32_t(sms) + nb - 1) / nb,
                         (words + kGatherThreads - 1) / kGatherThreads));
        gather_bricks_kernel<<<dim3(nb, split), kGatherThreads, 0, up>>>(
            arena, vol->host_store.as_dev<uint8_t>(), static_cast<const uint64_t*>(R.h_gather.dev),
            uint32_t(vol->brick_bytes), vol->info.max_block[0], vol->info.max_block[1],
            vol->stage_off != 0);
        LV_CUDA(ctx, cudaGetLastError());
        LV_CUDA(ctx, cudaEventRecord(R.gather_done, up));
        R.gather_recorded = true;
    }
    if (!expand.empty())
    {
        /* the offsets' buffer is read by the previous expansion until it ends */
        if (R.expand_recorded)
            LV_CUDA(ctx, cudaEventSynchronize(R.expand_done));
        LV_CUDA(ctx, R.h_expand.reserve(sizeof(uint64_t) * expand.size()));
        std::memcpy(R.h_expand.ptr, expand.data(), sizeof(uint64_t) * expand.size());
        const uint32_t voxels = uint32_t(vol->brick_bytes); /* uint8: one byte per voxel */
        expand_quads_kernel<<<uint32_t(expand.size()), kExpandThreads, 0, up>>>(
            arena, static_cast<const uint64_t*>(R.h_expand.dev), vol->info.max_block[0],
            vol->info.max_block[1], voxels, uint32_t(vol->stage_off));
        LV_CUDA(ctx, cudaGetLastError());
        LV_CUDA(ctx, cudaEventRecord(R.expand_done, up));
        R.expand_recorded = true;
    }
    lv_status u = apply_updates(ctx, updates, up);
    if (u != LV_OK)
        return u;
    LV_CUDA(ctx, cudaEventRecord(R.upload_event, up));
    LV_CUDA(ctx, cudaStreamWaitEvent(render, R.upload_event, 0));
    return st;
}

void volume_layout(lv_volume* v, uint32_t brick_layout)
{
    uint64_t off = 0;
    for (uint32_t L = 0; L <= kMaxLevels; ++L)
    {
        v->level_offset[L] = off;
        if (L < v->info.depth)
            off += (uint64_t(v->info.root_blocks[0]) << L) *
                   (uint64_t(v->info.root_blocks[1]) << L) *
                   (uint64_t(v->info.root_blocks[2]) << L);
    }
    v->n_nodes = off;
    v->brick_bytes = uint64_t(v->info.max_block[0]) * v->info.max_block[1] *
                     v->info.max_block[2] * bytes_per_voxel(v->info.dtype) *
                     v->info.comp_count;
    /* voxel quads: 4 bytes per voxel, the canonical bytes staged in the
     * slot's upper part (256-byte aligned, at or past three times the
     * brick's voxel count so that the in-place expansion never overwrites
     * bytes it has still to read): a slot of about 4 bytes per voxel */
    v->stage_off = brick_layout == LV_BRICKS_QUADS &&
                           quad_layout(v->info.dtype, v->info.max_block[0])
                       ? (3 * v->brick_bytes + 255) & ~uint64_t(255)
                       : 0;
    v->slot_units = uint32_t(round_units(v->stage_off + v->brick_bytes));
}

lv_status volume_init(lv_ctx* ctx, lv_volume* v)
{
    if (v->info.depth == 0 || v->info.depth > kMaxLevels)
        return fail(ctx, LV_EINVAL, "volume depth must be 1..15 (fill the info first)");
    if (bytes_per_voxel(v->info.dtype) == 0 || v->info.comp_count != 1)
        return fail(ctx, LV_EINVAL, "unsupported voxel type or component count");
    volume_layout(v, ctx->brick_layout);
    if (v->n_nodes > (uint64_t(1) << 28))
        return fail(ctx, LV_EINVAL, "octree too large for a dense page table");
    lv_status st = ensure_pool(ctx);
    if (st != LV_OK)
        return st;
    st = ensure_renderer(ctx);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, v->node_table.reserve(sizeof(int32_t) * v->n_nodes));
    LV_CUDA(ctx, v->node_stamp.reserve(sizeof(uint32_t) * v->n_nodes));
    fill_i32_kernel<<<256, 256, 0, ctx->upload_stream>>>(v->node_table.as<int32_t>(),
                                                         v->n_nodes, -1);
    LV_CUDA(ctx, cudaMemsetAsync(v->node_stamp.ptr, 0, sizeof(uint32_t) * v->n_nodes,
                                 ctx->upload_stream));
    LV_CUDA(ctx, cudaStreamSynchronize(ctx->upload_stream));
    v->host_table.assign(v->n_nodes, -1);
    return LV_OK;
}

void drop_volume_residency(lv_ctx* ctx, lv_volume* v)
{
    if (!ctx->pool)
        return;
    Pool& P = *ctx->pool;
    for (auto it = P.lru.begin(); it != P.lru.end();)
    {
        if (it->vol == v)
        {
            P.free_by_units[it->units].push_back(it->unit);
            P.resident_bytes -= uint64_t(it->units) * kSlotUnit;
            --P.resident_count[it->units];
            if (!v->pins.empty() && v->pins[it->node_idx])
                --P.pinned_count[it->units];
            it = P.lru.erase(it);
        }
        else
            ++it;
    }
}

/* Frame pixels whose centre ray can reach the box [lo, hi]: the bounding
 * rectangle of the projected box corners (P * MV, in double), widened by two
 * pixels so that FP32 rounding of a grazing ray cannot reach past it. A
 * corner at or behind the eye plane (w <= 1e-6) gives the whole frame. The
 * result is half-open: [r[0], r[2]) x [r[1], r[3]). */
void screen_rect(const lv_camera& cam, const float* lo, const float* hi, uint32_t W, uint32_t H,
                 uint32_t r[4])
{
    double pm[16];
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col)
        {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k)
                acc += double(cam.projection[k * 4 + row]) * double(cam.modelview[col * 4 + k]);
            pm[col * 4 + row] = acc;
        }
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int c = 0; c < 8; ++c)
    {
        const double p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1],
                             (c & 4) ? hi[2] : lo[2]};
        double q[4];
        for (int row = 0; row < 4; ++row)
            q[row] = pm[row] * p[0] + pm[4 + row] * p[1] + pm[8 + row] * p[2] + pm[12 + row];
        if (!(q[3] > 1e-6))
        {
            r[0] = r[1] = 0;
            r[2] = W;
            r[3] = H;
            return;
        }
        /* pixel index whose centre is at this position: (ndc + 1) / 2 * W - 1/2 */
        const double x = (q[0] / q[3] + 1.0) * 0.5 * W - 0.5;
        const double y = (q[1] / q[3] + 1.0) * 0.5 * H - 0.5;
        xmin = std::min(xmin, x);
        xmax = std::max(xmax, x);
        ymin = std::min(ymin, y);
        ymax = std::max(ymax, y);
    }
    auto clampi = [](double v, uint32_t n) {
        return uint32_t(std::min(std::max(v, 0.0), double(n)));
    };
    r[0] = clampi(std::floor(xmin) - 2.0, W);
    r[1] = clampi(std::floor(ymin) - 2.0, H);
    r[2] = clampi(std::ceil(xmax) + 3.0, W);
    r[3] = clampi(std::ceil(ymax) + 3.0, H);
}

lv_status make_ray_view(lv_ctx* ctx, const lv_volume* vol, const lv_tf* tf,
                        const lv_render_desc& desc, const lv_lod_params& lod, float* d_rgba,
                        uint32_t* leaf, uint32_t* counters, RayView& V)
{
    const lv_volume_info& info = vol->info;
    if (info.dtype > LV_DT_INT32)
        return fail(ctx, LV_EINVAL, "unknown voxel type");
    std::memset(&V, 0, sizeof(V));
    float lim[6], planes[6][4], eye[3], dir[3];
    bool ok = false;
    frustum_setup(desc.camera.modelview, desc.camera.projection, V.inv_mv, V.inv_p, lim,
                  planes, eye, dir, &ok);
    if (!ok)
        return fail(ctx, LV_EINVAL, "singular camera");
    const uint32_t Lf = info.depth - 1u;
    uint32_t dims[3];
    for (int a = 0; a < 3; ++a)
        dims[a] = info.root_blocks[a] << Lf;
    const uint32_t bm = std::max(dims[0], std::max(dims[1], dims[2]));
    V.edge = 0;
    for (int a = 0; a < 3; ++a)
    {
        V.eye[a] = eye[a];
        const float half = info.world_size[a] / 2.0f;
        V.gmin[a] = -half;
        V.gmax[a] = half;
        V.gscale[a] = float(bm) / info.world_size[a];
        V.goff[a] = half * V.gscale[a];
        V.dims[a] = dims[a];
        V.N[a] = info.max_block[a];
        V.O[a] = info.overlap[a];
        V.B[a] = info.max_block[a] - 2u * info.overlap[a];
        if (info.overlap[a] == 0 || V.N[a] < 2)
            V.edge = 1;
    }
    V.nearp = lim[4];
    V.n_clip = lod.n_clip_planes;
    std::memcpy(V.clip, lod.clip_planes, sizeof(V.clip));
    V.Lf = Lf;
    V.dtype = info.dtype;
    V.bpv = bytes_per_voxel(info.dtype);
    V.quads = vol->stage_off != 0;
    V.filter = desc.filter == LV_FILTER_TRILINEAR ? LV_FILTER_TRILINEAR : LV_FILTER_NEAREST;
    /* the transfer function's range when valid, else the type's
     * (RayCastRenderer.cpp:279-284) */
    float lo = desc.data_range[0], hi = desc.data_range[1];
    if (!(hi > 0.0f && hi - lo > 0.0f))
        type_range(info.dtype, lo, hi);
    V.dmul = 1.0f / (hi - lo);
    V.dadd = -lo / (hi - lo);
    V.early = desc.early_exit;
    V.FW = desc.width;
    V.FH = desc.height;
    screen_rect(desc.camera, V.gmin, V.gmax, desc.width, desc.height, V.cull);
    if (desc.rect[2] && desc.rect[3])
    {
        if (uint64_t(desc.rect[0]) + desc.rect[2] > desc.width ||
            uint64_t(desc.rect[1]) + desc.rect[3] > desc.height)
            return fail(ctx, LV_EINVAL, "render rect outside the frame");
        V.x0 = desc.rect[0];
        V.y0 = desc.rect[1];
        V.W = desc.rect[2];
        V.H = desc.rect[3];
    }
    else
    {
        V.W = desc.width;
        V.H = desc.height;
    }
    V.samples_fixed = desc.samples_per_ray;
    V.step_policy = desc.step_policy;
    V.max_voxel_dim = std::max(info.voxels[0], std::max(info.voxels[1], info.voxels[2]));
    V.depth = info.depth;
    V.leaf = leaf;
    V.pool = ctx->pool->arena.as<uint8_t>();
    V.pool_units = uint32_t(ctx->pool->capacity_units);
    V.brick_units = vol->slot_units;
    V.tf = tf->rgba.as<float4>();
    V.tfn = tf->n;
    V.tf_mul = V.dmul * float(tf->n);
    V.tf_add = V.dadd * float(tf->n) - 0.5f;
    V.tf_last = float(tf->n - 1u);
    V.accumulate = 0;
    V.max_base = V.edge ? 0u
                        : (V.N[2] - 2u) * V.N[1] * V.N[0] + (V.N[1] - 2u) * V.N[0] + V.N[0] - 2u;
    V.out = reinterpret_cast<float4*>(d_rgba);
    V.counters = counters;
    return LV_OK;
}

} // namespace lv

/* ================================================================ C ABI */
using namespace lv;

extern "C" uint32_t lv_abi_version(void) { return LV_ABI_VERSION; }

extern "C" lv_status lv_brick_slot_bytes(const lv_ctx* ctx, const lv_volume_info* info,
                                        uint64_t* bytes)
{
    if (!info || !bytes || bytes_per_voxel(info->dtype) == 0 || info->comp_count != 1)
        return LV_EINVAL;
    lv_volume v;
    v.info = *info;
    v.info.depth = 0; /* the layout of a brick only */
    volume_layout(&v, ctx ? ctx->brick_layout : uint32_t(LV_BRICKS_QUADS));
    *bytes = uint64_t(v.slot_units) * kSlotUnit;
    return LV_OK;
}

extern "C" lv_status lv_fill_regular_volume_info(lv_volume_info* info)
{
    /* livre/data/DataSourcePlugin.cpp:73-95 */
    if (!info)
        return LV_EINVAL;
    const uint32_t maxv =
        std::max(info->voxels[0], std::max(info->voxels[1], info->voxels[2]));
    if (maxv == 0)
        return LV_EINVAL;
    info->world_space_per_voxel = 1.0f / float(maxv);
    uint32_t bs[3], lod[3];
    for (int i = 0; i < 3; ++i)
    {
        info->world_size[i] = float(info->voxels[i]) * info->world_space_per_voxel;
        if (info->max_block[i] <= 2u * info->overlap[i])
            return LV_EINVAL;
        bs[i] = info->max_block[i] - 2u * info->overlap[i];
        const uint32_t nb = uint32_t(std::ceil(float(info->voxels[i]) / float(bs[i])));
        lod[i] = uint32_t(std::ceil(std::log2(double(nb))));
    }
    const uint32_t depth = std::min(lod[0], std::min(lod[1], lod[2]));
    for (int i = 0; i < 3; ++i)
        info->root_blocks[i] =
            uint32_t(std::ceil(float(info->voxels[i] >> depth) / float(bs[i])));
    info->depth = depth + 1;
    if (info->comp_count == 0)
        info->comp_count = 1;
    return LV_OK;
}

extern "C" lv_status lv_ctx_create(int device, lv_ctx** out)
{
    if (!out)
        return LV_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
        return LV_EDEVICE;
    if (cudaSetDevice(device) != cudaSuccess)
        return LV_EDEVICE;
    lv_ctx* ctx = new lv_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking) !=
        cudaSuccess)
    {
        delete ctx;
        return LV_EDEVICE;
    }
    *out = ctx;
    return LV_OK;
}

extern "C" void lv_ctx_destroy(lv_ctx* ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    if (ctx->renderer)
    {
        cudaEventDestroy(ctx->renderer->pending_event);
        cudaEventDestroy(ctx->renderer->render_event);
        cudaEventDestroy(ctx->renderer->upload_event);
        cudaEventDestroy(ctx->renderer->expand_done);
        cudaEventDestroy(ctx->renderer->gather_done);
        cudaEventDestroy(ctx->renderer->frame_done);
        cudaEventDestroy(ctx->renderer->resolve_done);
        cudaEventDestroy(ctx->renderer->fork);
        cudaEventDestroy(ctx->renderer->join);
        cudaStreamDestroy(ctx->renderer->side);
        cudaStreamDestroy(ctx->renderer->sel_stream);
        cudaEventDestroy(ctx->renderer->sel_done);
        cudaEventDestroy(ctx->renderer->visible_free);
        cudaEventDestroy(ctx->renderer->t_sel0);
        cudaEventDestroy(ctx->renderer->t_sel1);
        cudaEventDestroy(ctx->renderer->t_ray0);
        cudaEventDestroy(ctx->renderer->t_ray1);
        delete ctx->renderer;
    }
    delete ctx->pool;
    delete ctx->host_pool;
    if (ctx->upload_stream)
        cudaStreamDestroy(ctx->upload_stream);
    delete ctx;
}

extern "C" const char* lv_last_error(const lv_ctx* ctx)
{
    return ctx ? ctx->error.c_str() : "null context";
}

extern "C" lv_status lv_pool_configure(lv_ctx* ctx, size_t bytes)
{
    if (!ctx)
        return LV_EINVAL;
    if (ctx->pool)
        return fail(ctx, LV_EINVAL, "pool already allocated");
    if (bytes < kSlotUnit || bytes / kSlotUnit > (uint64_t(1) << kLeafSlotBits))
        return fail(ctx, LV_EINVAL, "pool size must be in [1 KiB, 128 GiB]");
    ctx->pool_bytes = bytes;
    return LV_OK;
}

extern "C" lv_status lv_pool_set_brick_layout(lv_ctx* ctx, uint32_t layout)
{
    if (!ctx)
        return LV_EINVAL;
    if (layout != LV_BRICKS_QUADS && layout != LV_BRICKS_COMPACT)
        return fail(ctx, LV_EINVAL, "unknown brick layout");
    if (ctx->pool)
        return fail(ctx, LV_EINVAL, "pool already allocated");
    ctx->brick_layout = layout;
    return LV_OK;
}

extern "C" lv_status lv_pool_purge(lv_ctx* ctx)
{
    if (!ctx)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (!ctx->pool)
        return LV_OK;
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    LV_CUDA(ctx, cudaDeviceSynchronize());
    Pool& P = *ctx->pool;
    std::vector<lv_volume*> vols;
    for (auto& r : P.lru)
        if (std::find(vols.begin(), vols.end(), r.vol) == vols.end())
            vols.push_back(r.vol);
    for (lv_volume* v : vols)
    {
        std::fill(v->host_table.begin(), v->host_table.end(), -1);
        fill_i32_kernel<<<256, 256, 0, ctx->upload_stream>>>(v->node_table.as<int32_t>(),
                                                             v->n_nodes, -1);
    }
    LV_CUDA(ctx, cudaStreamSynchronize(ctx->upload_stream));
    P.lru.clear();
    P.free_by_units.clear();
    P.bump = 0;
    P.resident_bytes = 0;
    P.resident_count.clear();
    P.pinned_count.clear();
    for (lv_volume* v : vols)
        std::fill(v->pins.begin(), v->pins.end(), uint16_t(0));
    if (ctx->renderer)
        ctx->renderer->pending_vol = nullptr;
    return LV_OK;
}

namespace
{
/* At least `count` pinned staging buffers of one brick each. */
lv_status grow_staging(lv_ctx* ctx, lv_volume* v, size_t count)
{
    while (v->staging.size() < count)
    {
        PinnedBuffer* b = new PinnedBuffer();
        if (b->reserve(v->brick_bytes) != cudaSuccess)
        {
            delete b;
            return fail(ctx, LV_ENOMEM, "pinned staging allocation");
        }
        cudaEvent_t e;
        LV_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        v->staging.push_back(b);
        v->staging_ev.push_back(e);
    }
    return LV_OK;
}
} // namespace

extern "C" lv_status lv_volume_set_fetch_threads(lv_volume* v, uint32_t threads)
{
    if (!v)
        return LV_EINVAL;
    lv_ctx* ctx = v->ctx;
    if (v->kind != SRC_CALLBACK)
        return fail(ctx, LV_EINVAL, "only callback sources are fetched on the host");
    if (threads == 0)
        threads = std::min(64u, std::max(1u, std::thread::hardware_concurrency()));
    if (threads > 64)
        return fail(ctx, LV_EINVAL, "at most 64 fetch threads");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    const lv_status st = grow_staging(ctx, v, std::max<size_t>(4, 2 * size_t(threads)));
    if (st != LV_OK)
        return st;
    v->fetch_threads = threads;
    return LV_OK;
}

extern "C" lv_status lv_volume_get_fetch_threads(const lv_volume* v, uint32_t* threads)
{
    if (!v || !threads)
        return LV_EINVAL;
    *threads = v->fetch_threads;
    return LV_OK;
}

extern "C" lv_status lv_volume_create(lv_ctx* ctx, const lv_volume_info* info,
                                      lv_get_data_fn get_data, void* user,
                                      lv_volume** out)
{
    if (!ctx || !info || !get_data || !out)
        return fail(ctx, LV_EINVAL, "null argument");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    lv_volume* v = new lv_volume();
    v->ctx = ctx;
    v->info = *info;
    v->kind = SRC_CALLBACK;
    v->fn = get_data;
    v->user = user;
    lv_status st = volume_init(ctx, v);
    if (st == LV_OK)
        st = grow_staging(ctx, v, 4);
    if (st != LV_OK)
    {
        delete v;
        return st;
    }
    *out = v;
    return LV_OK;
}

extern "C" lv_status lv_volume_create_blob(lv_ctx* ctx, const lv_volume_info* info,
                                           const lv_blob_desc* blob,
                                           uint32_t placement, lv_volume** out)
{
    if (!ctx || !info || !blob || !out)
        return fail(ctx, LV_EINVAL, "null argument");
    if (info->dtype != LV_DT_UINT8 && info->dtype != LV_DT_UINT16)
        return fail(ctx, LV_EINVAL, "blob volumes are uint8 or uint16");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    lv_volume* v = new lv_volume();
    v->ctx = ctx;
    v->info = *info;
    v->blob = *blob;
    v->kind = placement == LV_BLOB_HOST ? SRC_BLOB_HOST : SRC_BLOB_DEVICE;
    lv_status st = volume_init(ctx, v);
    if (st != LV_OK)
    {
        delete v;
        return st;
    }
    const std::vector<Blob> blobs = make_blobs(*info, *blob);
    cudaStream_t s = ctx->upload_stream;
    if (v->d_blobs.reserve(sizeof(Blob) * (blobs.size() + 1)) != cudaSuccess ||
        cudaMemcpy(v->d_blobs.ptr, blobs.data(), sizeof(Blob) * blobs.size(),
                   cudaMemcpyHostToDevice) != cudaSuccess)
    {
        delete v;
        return fail(ctx, LV_ENOMEM, "blob table");
    }
    if (v->kind == SRC_BLOB_HOST)
    {
        /* materialise every brick once into page-locked host memory */
        if (v->host_store.reserve(v->n_nodes * v->brick_bytes) != cudaSuccess)
        {
            delete v;
            return fail(ctx, LV_ENOMEM, "host brick store allocation");
        }
        const uint64_t batch = std::max<uint64_t>(1, (uint64_t(256) << 20) / v->brick_bytes);
        DeviceBuffer tmp, dids;
        PinnedBuffer hids;
        if (tmp.reserve(batch * v->brick_bytes) != cudaSuccess ||
            dids.reserve(sizeof(uint64_t) * batch) != cudaSuccess ||
            hids.reserve(sizeof(uint64_t) * batch) != cudaSuccess)
        {
            delete v;
            return fail(ctx, LV_ENOMEM, "generation buffers");
        }
        uint64_t idx = 0;
        for (uint32_t L = 0; L < info->depth; ++L)
        {
            const uint32_t bx = info->root_blocks[0] << L, by = info->root_blocks[1] << L,
                           bz = info->root_blocks[2] << L;
            const uint64_t nl = uint64_t(bx) * by * bz;
            for (uint64_t first = 0; first < nl; first += batch)
            {
                const uint64_t cnt = std::min(batch, nl - first);
                if (cudaStreamSynchronize(s) != cudaSuccess)
                {
                    delete v;
                    return fail(ctx, LV_EDEVICE, "generation");
                }
                for (uint64_t k = 0; k < cnt; ++k)
                {
                    const uint64_t lin = first + k; /* (x * by + y) * bz + z */
                    const uint32_t z = uint32_t(lin % bz), y = uint32_t((lin / bz) % by),
                                   x = uint32_t(lin / (uint64_t(by) * bz));
                    hids.as<uint64_t>()[k] = nid_make(L, x, y, z, 0);
                }
                cudaMemcpyAsync(dids.ptr, hids.ptr, sizeof(uint64_t) * cnt,
                                cudaMemcpyHostToDevice, s);
                st = launch_blob_bricks(ctx, *info, *blob, v->d_blobs.as<Blob>(),
                                        dids.as<uint64_t>(), uint32_t(cnt),
                                        tmp.as<uint8_t>(), nullptr, s);
                if (st != LV_OK)
                {
                    delete v;
                    return st;
                }
                cudaMemcpyAsync(v->host_store.as<uint8_t>() + (idx + first) * v->brick_bytes,
                                tmp.ptr, cnt * v->brick_bytes, cudaMemcpyDeviceToHost, s);
            }
            idx += nl;
        }
        if (cudaStreamSynchronize(s) != cudaSuccess)
        {
            delete v;
            return fail(ctx, LV_EDEVICE, "generation");
        }
    }
    *out = v;
    return LV_OK;
}

extern "C" void lv_volume_destroy(lv_volume* v)
{
    if (!v)
        return;
    lv_ctx* ctx = v->ctx;
    {
        std::lock_guard<std::mutex> lock(ctx->mutex);
        cudaSetDevice(ctx->device);
        cudaDeviceSynchronize();
        drop_volume_residency(ctx, v);
        if (ctx->renderer && ctx->renderer->pending_vol == v)
            ctx->renderer->pending_vol = nullptr;
        if (ctx->renderer && ctx->renderer->last_vol == v)
            ctx->renderer->last_vol = nullptr;
    }
    if (v->user_free)
        v->user_free(v->user);
    delete v;
}

extern "C" lv_status lv_volume_load(lv_volume* v, const uint64_t* ids, uint32_t n,
                                    uint32_t* n_loaded)
{
    if (!v || (n && !ids))
        return LV_EINVAL;
    lv_ctx* ctx = v->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->upload_stream;
    LV_CUDA(ctx, cudaDeviceSynchronize());
    uint32_t loaded = 0;
    uint64_t bytes = 0;
    /* nothing is in flight: no brick is protected from eviction */
    const uint32_t protect = ctx->renderer->frame + 1u;
    lv_status st = stream_bricks(ctx, v, ids, n, protect, s, loaded, bytes);
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    if (n_loaded)
        *n_loaded = loaded;
    return st;
}

extern "C" lv_status lv_volume_resident(const lv_volume* v, uint64_t* ids,
                                        uint32_t capacity, uint32_t* n)
{
    if (!v || !n || (capacity && !ids))
        return LV_EINVAL;
    lv_ctx* ctx = v->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    uint32_t k = 0;
    for (const Resident& r : ctx->pool->lru)
    {
        if (r.vol != v)
            continue;
        if (k < capacity)
        {
            uint32_t L = 0;
            while (L + 1 < v->info.depth && v->level_offset[L + 1] <= r.node_idx)
                ++L;
            const uint64_t local = r.node_idx - v->level_offset[L];
            const uint64_t by = uint64_t(v->info.root_blocks[1]) << L;
            const uint64_t bz = uint64_t(v->info.root_blocks[2]) << L;
            const uint32_t z = uint32_t(local % bz), y = uint32_t((local / bz) % by),
                           x = uint32_t(local / (by * bz));
            ids[k] = nid_make(L, x, y, z, v->time_step);
        }
        ++k;
    }
    *n = k;
    return k > capacity ? LV_ENOMEM : LV_OK;
}

extern "C" lv_status lv_volume_get_info(const lv_volume* v, lv_volume_info* out)
{
    if (!v || !out)
        return LV_EINVAL;
    *out = v->info;
    return LV_OK;
}

extern "C" lv_status lv_tf_create(lv_ctx* ctx, const float* rgba, uint32_t n,
                                  lv_tf** out)
{
    if (!ctx || !rgba || !out || n == 0)
        return fail(ctx, LV_EINVAL, "empty transfer function");
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    /* device layout: (value_i, value_{i+1} - value_i) pairs, last difference 0 */
    std::vector<float> pairs(size_t(8) * n);
    for (uint32_t i = 0; i < n; ++i)
        for (int c = 0; c < 4; ++c)
        {
            const float v = rgba[size_t(4) * i + c];
            const float nx = i + 1 < n ? rgba[size_t(4) * (i + 1) + c] : v;
            pairs[size_t(8) * i + c] = v;
            pairs[size_t(8) * i + 4 + c] = nx - v;
        }
    lv_tf* tf = new lv_tf();
    tf->ctx = ctx;
    tf->n = n;
    if (tf->rgba.reserve(sizeof(float) * pairs.size()) != cudaSuccess ||
        cudaMemcpy(tf->rgba.ptr, pairs.data(), sizeof(float) * pairs.size(),
                   cudaMemcpyHostToDevice) != cudaSuccess)
    {
        delete tf;
        return fail(ctx, LV_ENOMEM, "transfer function upload");
    }
    *out = tf;
    return LV_OK;
}

extern "C" void lv_tf_destroy(lv_tf* tf)
{
    if (!tf)
        return;
    cudaSetDevice(tf->ctx->device);
    cudaDeviceSynchronize();
    delete tf;
}

namespace lv
{
namespace
{
/* Streams up to `max` misses of the previous async frame. */
lv_status process_pending(lv_ctx* ctx, cudaStream_t s)
{
    Renderer& R = *ctx->renderer;
    if (!R.pending_vol)
        return LV_OK;
    LV_CUDA(ctx, cudaEventSynchronize(R.pending_event));
    lv_volume* v = R.pending_vol;
    R.pending_vol = nullptr;
    const uint32_t* hc = R.h_counters.as<uint32_t>();
    const uint32_t missing = std::min<uint32_t>(hc[FC_MISSING],
                                                uint32_t(R.h_missing.bytes / sizeof(uint64_t)));
    const uint32_t n = std::min(missing, R.pending_max);
    uint32_t loaded = 0;
    uint64_t bytes = 0;
    lv_status st = stream_bricks(ctx, v, R.h_missing.as<uint64_t>(), n, R.pending_frame,
                                 s, loaded, bytes);
    R.stats.n_uploaded += loaded;
    R.stats.bytes_uploaded += bytes;
    return st == LV_EAGAIN ? LV_OK : st;
}
} // namespace
} // namespace lv

namespace
{
/* Centre of node `id`'s world box, FP32 as LODNode's box
 * (DataSourcePlugin.cpp:40-71): bricks = rootBlocks << level, the largest
 * count scales every axis. */
void node_centre(const lv_volume_info& info, uint64_t id, float c[3])
{
    const uint32_t level = nid_level(id);
    uint32_t bricks[3];
    for (int i = 0; i < 3; ++i)
        bricks[i] = info.root_blocks[i] << level;
    int m = 0;
    for (int i = 1; i < 3; ++i)
        if (bricks[i] > bricks[m])
            m = i;
    const float denom = float(bricks[m]);
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    for (int i = 0; i < 3; ++i)
    {
        const float half = info.world_size[i] * 0.5f;
        const float lo = float(int32_t(pos[i])) / denom * info.world_size[i] - half;
        const float hi = float(int32_t(pos[i] + 1u)) / denom * info.world_size[i] - half;
        c[i] = (lo + hi) * 0.5f;
    }
}
} // namespace

extern "C" lv_status lv_set_render_launch(lv_ctx* ctx, const lv_render_launch* cfg)
{
    if (!ctx || !cfg)
        return LV_EINVAL;
    const uint32_t pixels = cfg->tile_w * cfg->tile_h;
    const bool ok = cfg->kind == LV_LAUNCH_WARP_TILES
                        ? pixels == 32
                    : cfg->kind == LV_LAUNCH_WARP_REFILL
                        ? pixels >= 32 && pixels <= 1024 && cfg->samples_per_check >= 1 &&
                              cfg->samples_per_check <= 64
                        : (cfg->kind == LV_LAUNCH_GRID || cfg->kind == LV_LAUNCH_TILE_QUEUE ||
                           cfg->kind == LV_LAUNCH_TILE_GRID) &&
                              pixels >= 32 && pixels <= 256 && pixels % 32 == 0;
    const bool order_ok = (cfg->order == LV_ORDER_RASTER ||
                           (cfg->order == LV_ORDER_LONGEST_FIRST && cfg->kind != LV_LAUNCH_GRID)) &&
                          (cfg->lookahead == 0 ||
                           (cfg->lookahead == 1 && cfg->kind != LV_LAUNCH_WARP_REFILL));
    if (!ok || !order_ok)
        return fail(ctx, LV_EINVAL,
                    "render launch: grid and tile-queue tiles of 32..256 threads (a multiple "
                    "of 32); warp-refill tiles of 32..1024 pixels, samples_per_check 1..64; "
                    "longest-first order only for the queue kinds; lookahead 0 or 1, not for "
                    "warp refill");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    ctx->launch = *cfg;
    return LV_OK;
}

extern "C" lv_status lv_get_render_launch(lv_ctx* ctx, lv_render_launch* cfg)
{
    if (!ctx || !cfg)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    *cfg = ctx->launch;
    return LV_OK;
}

extern "C" lv_status lv_render(lv_ctx* ctx, lv_volume* vol, lv_tf* tf,
                               const lv_render_desc* desc, float* d_rgba,
                               void* stream)
{
    if (!ctx || !vol || !tf || !desc || !d_rgba)
        return fail(ctx, LV_EINVAL, "null argument");
    if (desc->width == 0 || desc->height == 0)
        return fail(ctx, LV_EINVAL, "empty viewport");
    if (vol->ctx != ctx || tf->ctx != ctx)
        return fail(ctx, LV_EINVAL, "volume or transfer function of another context");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Renderer& R = *ctx->renderer;
    const lv_volume_info& info = vol->info;

    lv_frame_stats stats{};
    R.stats = stats;
    /* the previous frame's buffers are reused: its work (maybe on another
     * stream) comes first */
    if (R.have_last)
        LV_CUDA(ctx, cudaStreamWaitEvent(s, R.frame_done, 0));
    /* the side stream's work for this frame may start from here */
    LV_CUDA(ctx, cudaEventRecord(R.fork, s));
    R.pre_order = nullptr;
    R.leaf_cleared = false;
    struct ClearOrder
    {
        Renderer& r;
        ~ClearOrder() { r.pre_order = nullptr; }
    } clear_order{R};
    /* async: bricks missed by the previous frame are streamed now */
    if (!desc->synchronous)
    {
        lv_status st = process_pending(ctx, s);
        if (st != LV_OK)
            return st;
    }
    else
        R.pending_vol = nullptr;
    const uint32_t frame = ++R.frame;

    if (desc->lod.time_step != vol->time_step)
    {
        LV_CUDA(ctx, cudaStreamSynchronize(s));
        drop_volume_residency(ctx, vol);
        std::fill(vol->host_table.begin(), vol->host_table.end(), -1);
        fill_i32_kernel<<<256, 256, 0, s>>>(vol->node_table.as<int32_t>(), vol->n_nodes, -1);
        vol->time_step = desc->lod.time_step;
    }

    /* buffers */
    if (R.visible_capacity < vol->n_nodes)
    {
        LV_CUDA(ctx, cudaStreamSynchronize(s));
        const uint64_t cap = vol->n_nodes;
        LV_CUDA(ctx, R.visible.reserve(sizeof(uint64_t) * cap));
        LV_CUDA(ctx, R.render_ids.reserve(sizeof(uint64_t) * cap));
        LV_CUDA(ctx, R.render_slots.reserve(sizeof(uint32_t) * cap));
        LV_CUDA(ctx, R.missing.reserve(sizeof(uint64_t) * cap));
        LV_CUDA(ctx, R.h_missing.reserve(sizeof(uint64_t) * cap));
        R.visible_capacity = cap;
    }
    uint32_t dims[3];
    const uint32_t Lf = info.depth - 1u;
    for (int a = 0; a < 3; ++a)
        dims[a] = info.root_blocks[a] << Lf;
    const uint64_t cells = uint64_t(dims[0]) * dims[1] * dims[2];
    if (R.leaf.bytes < cells * sizeof(uint32_t))
    {
        LV_CUDA(ctx, cudaStreamSynchronize(s));
        LV_CUDA(ctx, R.leaf.reserve(cells * sizeof(uint32_t)));
    }
    lv_status st = reserve_selection(ctx, info, s);
    if (st != LV_OK)
        return st;

    /* 1. LOD selection */
    lv_lod_params lod = desc->lod;
    if (lod.window_height == 0)
        lod.window_height = desc->height;
    LodView LV;
    st = make_lod_view(ctx, info, desc->camera, lod, LV);
    if (st != LV_OK)
        return st;
    LV.out_ids = R.visible.as<uint64_t>();
    LV.capacity = uint32_t(std::min<uint64_t>(R.visible_capacity, 0xFFFFFFFFu));
    LV.result = R.sel_result.as<uint32_t>();
    /* kernels: the selection (one cooperative launch, or roots + one per
     * level + finish) and the copy of its result words to the host; then
     * resolve, the copy of its counters (synchronous mode) or prune
     * (asynchronous mode), leaf fill, ray cast (+ tile keys and order when
     * longest first) and the final copy of the counters. A synchronous frame
     * that streams misses resolves once more, and leaf fills and ray casts
     * again if its first ray cast was already queued. */
    const lv_render_launch& RL = ctx->launch;
    const uint32_t order_launches =
        RL.kind != LV_LAUNCH_GRID && RL.order == LV_ORDER_LONGEST_FIRST ? 2u : 0u;
    const uint32_t tail_launches = 3u + 1u + order_launches + 1u;
    /* the selection waits only for the previous frame's residency pass; while
     * that frame may still ray cast, the one-launch cooperative form (whose
     * CTAs must all be resident at once) gives way to the per-level form */
    cudaStream_t ss = R.sel_stream;
    bool overlap = false;
    if (R.have_last)
    {
        const cudaError_t q = cudaEventQuery(R.frame_done);
        overlap = q == cudaErrorNotReady;
        if (q != cudaSuccess)
            cudaGetLastError(); /* not ready is no error */
    }
    /* a frame queued behind one still in flight selects once that frame's
     * residency pass is done; otherwise in stream order */
    overlap = overlap && R.visible_free_recorded;
    LV_CUDA(ctx, cudaStreamWaitEvent(ss, overlap ? R.visible_free : R.fork, 0));
    st = scratch_acquire(ctx, ctx->sel, ss); /* after any lv_select_visible */
    if (st != LV_OK)
        return st;
    R.launches = selection_launches(ctx, 1, info.depth, !overlap) + 1u + tail_launches;
    LV_CUDA(ctx, cudaEventRecord(R.t_sel0, ss));
    st = run_selection(ctx, &LV, 1, info.depth, ss, !overlap);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaEventRecord(R.t_sel1, ss));
    if (!(lod.range[0] == 0.0f && lod.range[1] == 1.0f))
    {
        st = range_slice(ctx, info, lod.range, R.visible.as<uint64_t>(),
                         R.sel_result.as<uint32_t>(), ss);
        if (st != LV_OK)
            return st;
    }
    /* the frame's selection words for lv_last_stats, copied now: the next
     * frame's selection may overwrite them before this frame ends */
    st = scratch_release(ctx, ctx->sel, ss);
    if (st != LV_OK)
        return st;
    st = words_to_host(ctx, R.sel_result.ptr, R.h_counters, FC_WORDS, LV_SELECT_RESULT_WORDS, ss);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaEventRecord(R.sel_done, ss));
    LV_CUDA(ctx, cudaStreamWaitEvent(s, R.sel_done, 0));

    /* 2. residency */
    ResolveView RV;
    std::memset(&RV, 0, sizeof(RV));
    RV.visible = R.visible.as<uint64_t>();
    RV.n_visible_ptr = R.sel_result.as<uint32_t>() + LV_SEL_WRITTEN;
    RV.node_table = vol->node_table.as<int32_t>();
    RV.node_stamp = vol->node_stamp.as<uint32_t>();
    RV.view_stamp = vol->node_stamp.as<uint32_t>();
    RV.frame = frame;
    RV.view_frame = frame;
    RV.depth = info.depth;
    for (int a = 0; a < 3; ++a)
    {
        RV.root_blocks[a] = info.root_blocks[a];
        RV.dims[a] = dims[a];
    }
    std::memcpy(RV.level_offset, vol->level_offset, sizeof(RV.level_offset));
    RV.synchronous = desc->synchronous ? 1u : 0u;
    RV.render_ids = R.render_ids.as<uint64_t>();
    RV.render_slots = R.render_slots.as<uint32_t>();
    RV.render_capacity = uint32_t(R.visible_capacity);
    RV.missing = R.missing.as<uint64_t>();
    RV.missing_capacity = uint32_t(R.visible_capacity);
    RV.counters = R.counters.as<uint32_t>();
    RV.leaf = R.leaf.as<uint32_t>();
    RV.Lf = Lf;
    RV.n_nodes = vol->n_nodes;
    RayView V;
    st = make_ray_view(ctx, vol, tf, *desc, lod, d_rgba, R.leaf.as<uint32_t>(),
                       R.counters.as<uint32_t>(), V);
    if (st != LV_OK)
        return st;
    /* from the camera alone, beside the selection: the longest-first tile
     * order and the cleared leaf grid; the leaf fill waits for both */
    LV_CUDA(ctx, cudaStreamWaitEvent(R.side, R.fork, 0));
    LV_CUDA(ctx, cudaMemsetAsync(R.leaf.ptr, 0xFF, cells * sizeof(uint32_t), R.side));
    st = prepare_frame_order(ctx, V, ctx->launch, R.side, R.pre_order);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaEventRecord(R.join, R.side));
    R.leaf_cleared = true;
    /* residency pass, leaf grid and ray cast. The synchronous mode reads the
     * residency pass's miss count back while the rest runs, streams any
     * misses and renders again, and returns without waiting for the ray
     * cast. */
    auto timed_stream = [&](const uint64_t* ids, uint32_t n, uint32_t protect,
                            uint32_t& loaded, uint64_t& bytes, bool beside = false) -> lv_status {
        const auto t0 = std::chrono::steady_clock::now();
        const lv_status r = stream_bricks(ctx, vol, ids, n, protect, s, loaded, bytes, beside);
        R.stats.stream_ms += std::chrono::duration<float, std::milli>(
                                 std::chrono::steady_clock::now() - t0)
                                 .count();
        return r;
    };
    auto resolve = [&]() -> lv_status {
        LV_CUDA(ctx, cudaMemsetAsync(R.counters.ptr, 0, sizeof(uint32_t) * FC_WORDS, s));
        const lv_status t = launch_resolve(ctx, RV, s);
        if (t != LV_OK)
            return t;
        /* the next frame's selection may overwrite the visible list now */
        LV_CUDA(ctx, cudaEventRecord(R.visible_free, s));
        R.visible_free_recorded = true;
        return LV_OK;
    };
    auto after_resolve = [&]() -> lv_status {
        /* the first leaf fill of the frame waits for the side stream; a later
         * one (a frame rendered again, a later pass) clears the grid itself */
        if (R.leaf_cleared)
        {
            LV_CUDA(ctx, cudaStreamWaitEvent(s, R.join, 0));
            R.leaf_cleared = false;
        }
        else
            LV_CUDA(ctx, cudaMemsetAsync(R.leaf.ptr, 0xFF, cells * sizeof(uint32_t), s));
        lv_status t = launch_leaf_fill(ctx, RV, s);
        if (t != LV_OK)
            return t;
        LV_CUDA(ctx, cudaEventRecord(R.t_ray0, s));
        t = launch_raycast(ctx, V, s);
        if (t != LV_OK)
            return t;
        LV_CUDA(ctx, cudaEventRecord(R.t_ray1, s));
        return LV_OK;
    };
    auto frame_tail = [&]() -> lv_status {
        const lv_status t = resolve();
        return t != LV_OK ? t : after_resolve();
    };
    /* A visible set larger than the brick pool renders in passes of at most
     * a pool's worth of bricks, front to back by brick distance
     * (renderSync, RenderPipeline.cpp:92-158; DistanceOperator,
     * RayCastRenderer.cpp:57-81), each pass compositing on top of the
     * previous ones. The samples per ray come from the first pass's bricks,
     * as onFrameStart runs for the first pass only (Renderer.cpp,
     * RayCastRenderer.cpp:213-233). */
    auto multipass = [&](uint32_t n_vis, uint64_t per_pass, uint32_t first_frame) -> lv_status {
        const uint32_t m = uint32_t(std::min<uint64_t>(per_pass, 0xFFFFFFFFu));
        LV_CUDA(ctx, R.h_pass.reserve(sizeof(uint64_t) * n_vis));
        LV_CUDA(ctx, R.pass_count.reserve(sizeof(uint32_t)));
        std::vector<uint64_t> ids(n_vis);
        LV_CUDA(ctx, cudaMemcpyAsync(ids.data(), R.visible.ptr, sizeof(uint64_t) * n_vis,
                                     cudaMemcpyDeviceToHost, s));
        LV_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<float> dist(n_vis);
        std::vector<uint32_t> order(n_vis);
        const float* mv = desc->camera.modelview; /* column-major */
        for (uint32_t i = 0; i < n_vis; ++i)
        {
            float c[3], e[3];
            node_centre(info, ids[i], c);
            for (int k = 0; k < 3; ++k)
                e[k] = mv[k] * c[0] + mv[4 + k] * c[1] + mv[8 + k] * c[2] + mv[12 + k];
            dist[i] = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            order[i] = i;
        }
        /* equal distances: lower node id first, so the passes do not depend on
         * the order the selection emitted the ids in */
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            return dist[a] < dist[b] || (dist[a] == dist[b] && ids[a] < ids[b]);
        });
        uint64_t* hp = R.h_pass.as<uint64_t>();
        for (uint32_t i = 0; i < n_vis; ++i)
            hp[i] = ids[order[i]];
        const uint32_t passes = (n_vis + m - 1) / m;
        lv_frame_stats agg{};
        uint32_t n0 = 0;
        float ray_ms = 0.f;
        uint32_t* hc = R.h_counters.as<uint32_t>();
        RV.n_visible_ptr = R.pass_count.as<uint32_t>();
        RV.synchronous = 1;
        for (uint32_t p = 0; p < passes; ++p)
        {
            const uint32_t fp = p == 0 ? first_frame : ++R.frame;
            const uint32_t first = p * m, cnt = std::min(m, n_vis - first);
            RV.frame = RV.view_frame = fp;
            LV_CUDA(ctx, cudaMemcpyAsync(R.visible.ptr, hp + first, sizeof(uint64_t) * cnt,
                                         cudaMemcpyHostToDevice, s));
            LV_CUDA(ctx, cudaMemcpyAsync(R.pass_count.ptr, &cnt, sizeof(uint32_t),
                                         cudaMemcpyHostToDevice, s));
            /* this pass's misses: stream them, evicting earlier passes' bricks
             * (their stamps are older than fp) */
            LV_CUDA(ctx, cudaMemsetAsync(R.counters.ptr, 0, sizeof(uint32_t) * FC_WORDS, s));
            lv_status t = launch_resolve(ctx, RV, s);
            if (t != LV_OK)
                return t;
            LV_CUDA(ctx, cudaMemcpyAsync(hc, R.counters.ptr, sizeof(uint32_t) * FC_WORDS,
                                         cudaMemcpyDeviceToHost, s));
            LV_CUDA(ctx, cudaStreamSynchronize(s));
            const uint32_t missing = std::min<uint32_t>(hc[FC_MISSING], RV.missing_capacity);
            if (missing)
            {
                LV_CUDA(ctx, cudaMemcpyAsync(R.h_missing.ptr, R.missing.ptr,
                                             sizeof(uint64_t) * missing,
                                             cudaMemcpyDeviceToHost, s));
                LV_CUDA(ctx, cudaStreamSynchronize(s));
                uint32_t loaded = 0;
                uint64_t bytes = 0;
                t = timed_stream(R.h_missing.as<uint64_t>(), missing, fp, loaded, bytes);
                R.stats.n_uploaded += loaded;
                R.stats.bytes_uploaded += bytes;
                if (t != LV_OK && t != LV_EAGAIN)
                    return t;
            }
            V.accumulate = p > 0 ? 1u : 0u;
            V.samples_fixed = p > 0 ? n0 : desc->samples_per_ray;
            t = frame_tail();
            if (t != LV_OK)
                return t;
            LV_CUDA(ctx, cudaMemcpyAsync(hc, R.counters.ptr, sizeof(uint32_t) * FC_WORDS,
                                         cudaMemcpyDeviceToHost, s));
            LV_CUDA(ctx, cudaStreamSynchronize(s));
            if (p == 0)
                n0 = hc[FC_SAMPLES_PER_RAY];
            agg.n_rendered += hc[FC_KEPT];
            agg.n_available += hc[FC_AVAILABLE];
            agg.n_not_available += hc[FC_NOT_AVAILABLE];
            agg.max_level = std::max(agg.max_level, hc[FC_MAX_LEVEL]);
            agg.n_samples += uint64_t(hc[FC_SAMPLES_LO]) | (uint64_t(hc[FC_SAMPLES_HI]) << 32);
            agg.error_flags = agg.error_flags ? agg.error_flags : hc[FC_ERROR];
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, R.t_ray0, R.t_ray1) == cudaSuccess)
                ray_ms += ms;
            else
                cudaGetLastError();
        }
        agg.max_level = agg.max_level ? agg.max_level - 1u : 0u;
        agg.samples_per_ray = n0;
        agg.raycast_ms = ray_ms;
        agg.n_passes = passes;
        R.pass_stats = agg;
        R.passes = passes;
        /* per pass: a residency pass, then resolve, leaf fill and ray cast */
        R.launches = selection_launches(ctx, 1, info.depth, !overlap) + 1u + order_launches +
                     passes * 4u;
        return LV_OK;
    };
    /* A frame queued while the previous one still ray casts (a fly-through
     * rendered back to back) streams its missing bricks beside that ray cast:
     * its visible nodes are looked up on the selection stream, and eviction
     * spares the previous frame's bricks (stamped frame - 1 by its residency
     * passes) as well as this frame's resident ones (stamped by the lookup),
     * so no slot the running ray cast reads is overwritten. Only when the
     * previous frame was a one-pass synchronous lv_render of this volume and
     * no batch or server has used the pool since. */
    bool prefetched = false;
    if (overlap && desc->synchronous && R.last_desc.synchronous && R.passes == 0 &&
        R.last_vol == vol && vol->streamed_last && frame > 1u &&
        R.foreign_seen == ctx->foreign_pool_use.load())
    {
        const uint32_t cap = uint32_t(std::min<uint64_t>(R.visible_capacity, 0xFFFFFFFFu));
        LV_CUDA(ctx, R.probe.reserve(sizeof(uint64_t) * cap));
        LV_CUDA(ctx, R.probe_count.reserve(sizeof(uint32_t)));
        LV_CUDA(ctx, R.h_probe.reserve(sizeof(uint64_t) * (size_t(cap) + 1)));
        LV_CUDA(ctx, cudaMemsetAsync(R.probe_count.ptr, 0, sizeof(uint32_t), ss));
        probe_kernel<<<256, 256, 0, ss>>>(RV, R.probe.as<uint64_t>(), R.probe_count.as<uint32_t>(),
                                          cap);
        LV_CUDA(ctx, cudaGetLastError());
        ++R.launches;
        uint32_t* hcount = R.h_probe.as<uint32_t>();
        uint64_t* hids = R.h_probe.as<uint64_t>() + 1;
        LV_CUDA(ctx, cudaMemcpyAsync(hcount, R.probe_count.ptr, sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, ss));
        LV_CUDA(ctx, cudaStreamSynchronize(ss));
        const uint32_t n_probe = std::min(*hcount, cap);
        if (n_probe)
        {
            LV_CUDA(ctx, cudaMemcpyAsync(hids, R.probe.ptr, sizeof(uint64_t) * n_probe,
                                         cudaMemcpyDeviceToHost, ss));
            LV_CUDA(ctx, cudaStreamSynchronize(ss));
            uint32_t loaded = 0;
            uint64_t bytes = 0;
            st = timed_stream(hids, n_probe, frame - 1u, loaded, bytes, true);
            R.stats.n_uploaded += loaded;
            R.stats.bytes_uploaded += bytes;
            if (st != LV_OK && st != LV_EAGAIN)
                return st;
            prefetched = true;
        }
    }
    R.passes = 0;
    bool multi = false;
    /* bricks of this volume the pool holds at once: a visible set larger
     * than that renders in passes (renderSync) */
    const uint64_t per_pass = ctx->pool->capacity_units / vol->slot_units;
    if (desc->synchronous)
    {
        /* The residency pass's miss count (and the selection's visible
         * count, which reached the host before it) goes to the host while
         * the rest of the frame is already queued behind it; the host waits
         * for the counts only. A frame that missed bricks streams them and
         * renders again (the first ray cast lacked them), unless its volume
         * streamed in the previous frame too: then the ray cast is queued
         * only after the count is known. A visible set larger than the pool
         * cannot be resident at once, so it always misses: its queued ray
         * cast returns at once, and the frame renders in passes instead,
         * numbered after this residency pass so that the bricks it stamped
         * are not held in the pool. */
        uint32_t* hc = R.h_counters.as<uint32_t>();
        st = resolve();
        if (st != LV_OK)
            return st;
        /* the counters and the missing ids, through the host mapping */
        counters_to_host_kernel<<<8, 256, 0, s>>>(
            R.counters.as<uint32_t>(), R.missing.as<uint64_t>(), R.h_counters.as_dev<uint32_t>(),
            R.h_missing.as_dev<uint64_t>(), RV.missing_capacity);
        LV_CUDA(ctx, cudaGetLastError());
        LV_CUDA(ctx, cudaEventRecord(R.resolve_done, s));
        /* a volume that streamed last frame likely misses again: then the
         * ray cast waits for the streaming instead of running twice (unless
         * this frame's misses were streamed beside the previous frame).
         * Queued before the miss count is known, the ray cast returns at
         * once if there are misses (skip_if_missing). */
        const bool queued = !vol->streamed_last || prefetched;
        if (queued)
        {
            V.skip_if_missing = 1u;
            st = after_resolve();
            V.skip_if_missing = 0u;
            if (st != LV_OK)
                return st;
        }
        LV_CUDA(ctx, cudaEventSynchronize(R.resolve_done));
        const uint32_t n_vis = hc[FC_WORDS + LV_SEL_WRITTEN];
        if (per_pass > 0 && n_vis > per_pass)
        {
            multi = true;
            st = multipass(n_vis, per_pass, ++R.frame);
            if (st != LV_OK)
                return st;
            /* this residency pass and its counters' copy, and the leaf fill
             * and ray cast queued behind them */
            R.launches += queued ? 4u : 2u;
        }
        else
        {
            const uint32_t missing = std::min<uint32_t>(hc[FC_MISSING], RV.missing_capacity);
            if (!missing && !queued)
                st = after_resolve();
            else if (missing)
            {
                uint32_t loaded = 0;
                uint64_t bytes = 0;
                st = timed_stream(R.h_missing.as<uint64_t>(), missing, frame, loaded, bytes);
                R.stats.n_uploaded += loaded;
                R.stats.bytes_uploaded += bytes;
                if (st != LV_OK && st != LV_EAGAIN)
                    return st;
                /* resolve again with the streamed bricks; what still misses
                 * (pool too small) is not rendered */
                st = frame_tail();
                if (queued)
                    R.launches += 3u;
                else
                    R.launches += 1; /* one more residency pass */
            }
            vol->streamed_last = R.stats.n_uploaded > 0;
        }
    }
    else
        st = frame_tail();
    if (st != LV_OK)
        return st;

    /* 5. copy back counters (+ misses in async mode); the selection words
     * were copied after the selection */
    if (!multi)
    {
        st = words_to_host(ctx, R.counters.ptr, R.h_counters, 0, FC_WORDS, s);
        if (st != LV_OK)
            return st;
    }
    if (!desc->synchronous)
    {
        LV_CUDA(ctx, cudaMemcpyAsync(R.h_missing.ptr, R.missing.ptr,
                                     sizeof(uint64_t) * std::min<uint64_t>(R.visible_capacity, 4096),
                                     cudaMemcpyDeviceToHost, s));
        LV_CUDA(ctx, cudaEventRecord(R.pending_event, s));
        R.pending_vol = vol;
        R.pending_max = desc->max_uploads;
        R.pending_frame = frame;
    }
    LV_CUDA(ctx, cudaEventRecord(R.frame_done, s));
    R.last_stream = s;
    R.have_last = true;
    R.last_vol = vol;
    R.last_desc = *desc;
    R.foreign_seen = ctx->foreign_pool_use.load();
    ++ctx->totals.frames;
    ctx->totals.bricks_uploaded += R.stats.n_uploaded;
    ctx->totals.bytes_uploaded += R.stats.bytes_uploaded;
    ctx->totals.launches += R.launches;
    return LV_OK;
}

extern "C" lv_status lv_get_totals(lv_ctx* ctx, lv_ctx_totals* out)
{
    if (!ctx || !out)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    *out = ctx->totals;
    return LV_OK;
}

extern "C" lv_status lv_frame_histogram(lv_ctx* ctx, uint32_t n_bins, float range_lo,
                                       float range_hi, uint64_t* accumulated)
{
    if (!ctx || !accumulated)
        return LV_EINVAL;
    std::vector<uint64_t> ids;
    lv_volume* vol = nullptr;
    {
        std::lock_guard<std::mutex> lock(ctx->mutex);
        if (!ctx->renderer || !ctx->renderer->have_last || !ctx->renderer->last_vol)
            return fail(ctx, LV_EINVAL, "no frame rendered (or its volume is gone)");
        Renderer& R = *ctx->renderer;
        LV_CUDA(ctx, cudaSetDevice(ctx->device));
        LV_CUDA(ctx, cudaStreamSynchronize(R.last_stream));
        vol = R.last_vol;
        const lv_render_desc& d = R.last_desc;
        /* the frame's bricks: every pass's of a multi-pass frame, else the
         * rendering set (entries dropped for an ancestor are invalid ids) */
        std::vector<uint64_t> set;
        if (R.passes)
        {
            const uint64_t* hp = R.h_pass.as<uint64_t>();
            set.assign(hp, hp + R.h_counters.as<uint32_t>()[FC_WORDS + LV_SEL_WRITTEN]);
        }
        else
        {
            const uint32_t n = std::min<uint32_t>(R.h_counters.as<uint32_t>()[FC_RENDERED],
                                                  uint32_t(R.visible_capacity));
            set.resize(n);
            if (n)
                LV_CUDA(ctx, cudaMemcpy(set.data(), R.render_ids.ptr, sizeof(uint64_t) * n,
                                        cudaMemcpyDeviceToHost));
        }
        /* HistogramFilter::isCenterInViewport (HistogramFilter.cpp:44-76): a
         * brick counts when its centre projects into the rendered rect, the
         * frame's own borders pushed out to infinity; half-open, so a centre
         * on an edge two rects share counts in one of them */
        const bool whole = !(d.rect[2] && d.rect[3]);
        const uint32_t x0 = whole ? 0 : d.rect[0], y0 = whole ? 0 : d.rect[1];
        const uint32_t w = whole ? d.width : d.rect[2], h = whole ? d.height : d.rect[3];
        const float inf = std::numeric_limits<float>::infinity();
        const float xlo = x0 == 0 ? -inf : 2.0f * float(x0) / float(d.width) - 1.0f;
        const float xhi = x0 + w == d.width ? inf : 2.0f * float(x0 + w) / float(d.width) - 1.0f;
        const float ylo = y0 == 0 ? -inf : 2.0f * float(y0) / float(d.height) - 1.0f;
        const float yhi = y0 + h == d.height ? inf : 2.0f * float(y0 + h) / float(d.height) - 1.0f;
        const float* mv = d.camera.modelview;
        const float* pj = d.camera.projection;
        for (uint64_t id : set)
        {
            if (id == kInvalidNode)
                continue;
            float c[3], e[4], q[4];
            node_centre(vol->info, id, c);
            for (int r = 0; r < 4; ++r)
                e[r] = mv[r] * c[0] + mv[4 + r] * c[1] + mv[8 + r] * c[2] + mv[12 + r];
            for (int r = 0; r < 4; ++r)
                q[r] = pj[r] * e[0] + pj[4 + r] * e[1] + pj[8 + r] * e[2] + pj[12 + r] * e[3];
            const float nx = q[0] / q[3], ny = q[1] / q[3];
            if (nx >= xlo && nx < xhi && ny >= ylo && ny < yhi)
                ids.push_back(id);
        }
    }
    return lv_histogram(vol, ids.data(), uint32_t(ids.size()), n_bins, range_lo, range_hi,
                        nullptr, accumulated);
}

extern "C" lv_status lv_last_stats(lv_ctx* ctx, lv_frame_stats* out)
{
    if (!ctx || !out)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (!ctx->renderer || !ctx->renderer->have_last)
        return fail(ctx, LV_EINVAL, "no frame rendered");
    Renderer& R = *ctx->renderer;
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    LV_CUDA(ctx, cudaStreamSynchronize(R.last_stream));
    const uint32_t* hc = R.h_counters.as<uint32_t>();
    const uint32_t* sel = hc + FC_WORDS;
    lv_frame_stats s = R.stats;
    s.n_visible = sel[LV_SEL_WRITTEN];
    s.n_visited = sel[LV_SEL_VISITED];
    s.n_rendered = hc[FC_KEPT];
    s.n_available = hc[FC_AVAILABLE];
    s.n_not_available = hc[FC_NOT_AVAILABLE];
    s.max_level = hc[FC_MAX_LEVEL] ? hc[FC_MAX_LEVEL] - 1u : 0u;
    s.samples_per_ray = hc[FC_SAMPLES_PER_RAY];
    s.n_samples = uint64_t(hc[FC_SAMPLES_LO]) | (uint64_t(hc[FC_SAMPLES_HI]) << 32);
    s.n_launches = R.launches;
    s.error_flags = hc[FC_ERROR];
    s.n_passes = 1;
    if (cudaEventElapsedTime(&s.select_ms, R.t_sel0, R.t_sel1) != cudaSuccess ||
        cudaEventElapsedTime(&s.raycast_ms, R.t_ray0, R.t_ray1) != cudaSuccess)
    {
        cudaGetLastError(); /* do not leave the error for the next launch check */
        s.select_ms = s.raycast_ms = 0.f;
    }
    if (R.passes)
    {
        const lv_frame_stats& P = R.pass_stats;
        s.n_rendered = P.n_rendered;
        s.n_available = P.n_available;
        s.n_not_available = P.n_not_available;
        s.max_level = P.max_level;
        s.samples_per_ray = P.samples_per_ray;
        s.n_samples = P.n_samples;
        s.raycast_ms = P.raycast_ms;
        s.error_flags = P.error_flags;
        s.n_passes = P.n_passes;
    }
    *out = s;
    if (sel[LV_SEL_OVERFLOW] == 2u)
    {
        out->error_flags = 4u;
        return fail(ctx, LV_EDEVICE, "the selection's grid barrier gave up waiting");
    }
    if (hc[FC_ERROR])
        return fail(ctx, hc[FC_ERROR] == 1 ? LV_ENOMEM : LV_EDEVICE,
                    hc[FC_ERROR] == 1 ? "rendering set overflowed its buffer"
                                      : "a device index check failed (access skipped)");
    return LV_OK;
}
