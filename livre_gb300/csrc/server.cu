/*
 * Render server with continuous batching.
 *
 * Requests (volume, transfer function, camera, viewport, LOD threshold,
 * output buffer) are queued by lv_server_submit from any thread. A server
 * thread repeatedly:
 *   1. completes the batch that finished on the device (unpins its bricks,
 *      stamps latencies, wakes waiters);
 *   2. takes up to max_batch queued requests (FIFO), runs one multi-view LOD
 *      selection for them on its own stream and scratch (overlapping the batch
 *      still rendering), and admits them in order while the brick pool can
 *      hold their missing bricks (free slots plus resident bricks that no
 *      admitted request pins); admitted requests' visible bricks are pinned
 *      and their misses streamed on the upload stream;
 *   3. renders the admitted requests as one lv_batch_render (all bricks
 *      resident, so each result equals the same request rendered alone).
 * Four lv_batch objects take turns, so step 2 for the next batch runs while the
 * previous one renders. Mode LV_SERVE_PLAIN instead renders every request
 * alone with lv_render (synchronous residency), the per-request baseline.
 *
 * The reference serves frames through Equalizer channels, one view per
 * channel and frame (livre/eq/Channel.cpp:283-336); there is no
 * counterpart to batching requests across volumes.
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <memory>
#include <deque>
#include <thread>
#include <unordered_map>
#include <vector>

#include "lv_runtime.h"

namespace
{
using namespace lv;

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Req
{
    uint64_t ticket = 0;
    lv_request r{};
    double t_submit = 0, t_admit = 0, t_done = 0;
    lv_status status = LV_OK;
    uint32_t batch_size = 0;
    lv_frame_stats stats{};
    bool done = false;
    std::vector<uint64_t> pinned; /* node indices of r.volume */
};

/* Completion time written by a host function queued after the batch. */
struct DoneClock
{
    std::atomic<double> t{0.0};
};

void CUDART_CB stamp_done(void* p)
{
    static_cast<DoneClock*>(p)->t.store(now_ms());
}

struct Inflight
{
    lv_batch* batch = nullptr;
    /* tickets, not Req pointers: a request completed early by its view's
     * hook may be collected (and freed) by lv_server_wait before the batch
     * ends */
    std::vector<uint64_t> tickets;
    std::vector<std::pair<lv_volume*, std::vector<uint64_t>>> pins;
    lv_status status = LV_OK;
    cudaEvent_t ev = nullptr;
    std::shared_ptr<DoneClock> clock;
};

struct lv_server_hook
{
    lv_server* S;
    int batch;
};
} // namespace

/* Batches in flight at once: a batch is admitted and launched while up to
 * kSlots - 1 earlier ones still render (each later one a priority level
 * below them), so a heavy batch does not hold back the requests queued
 * behind it. */
constexpr int kSlots = lv::kBatchPriorityLevels;

struct lv_server
{
    lv_ctx* ctx = nullptr;
    lv_server_config cfg{};
    std::thread th;
    std::mutex m;
    std::condition_variable cv, cv_done;
    std::deque<Req*> queue;
    std::unordered_map<uint64_t, Req*> reqs;
    uint64_t next_ticket = 1;
    bool stop = false;
    lv_batch* batches[kSlots] = {};
    int cur = 0;
    std::deque<Inflight> inflight;
    std::vector<cudaEvent_t> free_events;
    cudaStream_t sel_stream = nullptr;
    /* one launch stream per batch object: consecutive batches overlap */
    cudaStream_t launch_stream[kSlots] = {};
    lv_server_hook hooks[kSlots];
    std::vector<uint64_t> current[kSlots]; /* tickets of the views in flight per batch object */
    cudaEvent_t uploads_done = nullptr;
    cudaEvent_t sel_t0 = nullptr, sel_t1 = nullptr; /* admission selection timing */
    /* dry-run selection buffers */
    SelectScratch sel;
    DeviceBuffer vis, res, views;
    PinnedBuffer h_vis, h_res, h_views;
    uint64_t vis_stride = 0;
    /* counters */
    uint64_t n_done = 0, n_batches = 0;
    lv_server_profile prof{};
};

namespace
{
void complete(lv_server* S, Inflight& f)
{
    double t = now_ms();
    if (f.clock && f.clock->t.load() > 0.0)
        t = f.clock->t.load();
    const uint32_t n = uint32_t(f.tickets.size());
    std::vector<lv_frame_stats> st(n);
    float batch_ms = 0.f, ray_ms = 0.f;
    if (f.batch && n)
        lv_batch_stats(f.batch, st.data(), n, &batch_ms, &ray_ms);
    {
        std::lock_guard<std::mutex> lk(S->ctx->mutex);
        for (auto& vp : f.pins)
        {
            lv_volume* v = vp.first;
            for (uint64_t idx : vp.second)
                if (v->pins[idx] && --v->pins[idx] == 0 && v->host_table[idx] >= 0)
                    --S->ctx->pool->pinned_count[v->slot_units];
        }
        f.pins.clear();
    }
    std::lock_guard<std::mutex> lk(S->m);
    S->prof.device_ms += batch_ms;
    S->prof.raycast_ms += ray_ms;
    S->prof.requests += n;
    for (uint32_t i = 0; i < n; ++i)
    {
        auto it = S->reqs.find(f.tickets[i]);
        if (it == S->reqs.end() || it->second->done)
            continue; /* completed by its view's hook */
        Req* r = it->second;
        r->t_done = t;
        r->stats = st[i];
        if (r->status == LV_OK)
            r->status = f.status;
        if (r->status == LV_OK && st[i].error_flags)
            r->status = LV_EDEVICE;
        r->done = true;
        ++S->n_done;
    }
    if (f.ev)
        S->free_events.push_back(f.ev);
    S->cv_done.notify_all();
}

/* A view of a per-view-kernel batch is complete (CUDA host-function
 * thread): its request is done, with the view's own statistics. */
void view_done(void* user, uint32_t view, const uint32_t* words)
{
    const lv_server_hook* h = static_cast<const lv_server_hook*>(user);
    lv_server* S = h->S;
    const double t = now_ms();
    std::lock_guard<std::mutex> lk(S->m);
    const std::vector<uint64_t>& cur = S->current[h->batch];
    if (view >= cur.size())
        return;
    auto it = S->reqs.find(cur[view]);
    if (it == S->reqs.end() || it->second->done)
        return;
    Req* r = it->second;
    batch_decode_stats(words, r->stats);
    if (r->stats.error_flags)
        r->status = LV_EDEVICE;
    r->t_done = t;
    r->done = true;
    ++S->n_done;
    S->cv_done.notify_all();
}

void add_time(lv_server* S, double lv_server_profile::*field, double ms)
{
    std::lock_guard<std::mutex> lk(S->m);
    S->prof.*field += ms;
}

/* Blocks until an in-flight batch finishes (server thread). */
void wait_batch(lv_server* S, cudaEvent_t ev)
{
    const double t0 = now_ms();
    cudaEventSynchronize(ev);
    add_time(S, &lv_server_profile::wait_ms, now_ms() - t0);
}

void fail_request(lv_server* S, Req* r, lv_status st)
{
    std::lock_guard<std::mutex> lk(S->m);
    r->status = st;
    r->t_admit = r->t_done = now_ms();
    r->done = true;
    ++S->n_done;
    S->cv_done.notify_all();
}

/* The admission selection's per-view constants from mapped page-locked
 * host memory, by a kernel rather than a copy: a copy would queue on the
 * copy engine behind the batches' own parameter copies, each waiting for
 * its stream. */
__global__ void views_from_host_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                       uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

/* An admission selection's result words and visible ids (the first
 * WRITTEN of each view's list) to mapped page-locked host memory, one CTA
 * per view. A kernel rather than copies: under load the copy engine holds
 * the batches' read-backs, each waiting for its ray cast, and a copy queued
 * behind them waits as long. */
__global__ void selection_to_host_kernel(const uint32_t* __restrict__ res,
                                         const uint64_t* __restrict__ vis, uint32_t stride,
                                         uint32_t* h_res, uint64_t* h_vis)
{
    const uint32_t v = blockIdx.x;
    const uint32_t* r = res + LV_SELECT_RESULT_WORDS * v;
    for (uint32_t i = threadIdx.x; i < LV_SELECT_RESULT_WORDS; i += blockDim.x)
        h_res[LV_SELECT_RESULT_WORDS * v + i] = r[i];
    const uint32_t k = min(r[LV_SEL_WRITTEN], stride);
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x)
        h_vis[uint64_t(stride) * v + i] = vis[uint64_t(stride) * v + i];
    __threadfence_system();
}

/* Dry-run selection of the candidates; returns the visible ids per view. */
lv_status dry_run(lv_server* S, const std::vector<Req*>& cand,
                  std::vector<std::vector<uint64_t>>& visible)
{
    lv_ctx* ctx = S->ctx;
    const uint32_t n = uint32_t(cand.size());
    uint64_t stride = 64, frontier = 0;
    for (Req* r : cand)
    {
        stride = std::max(stride, r->r.volume->n_nodes);
        frontier += max_frontier(r->r.volume->info);
    }
    cudaStream_t s = S->sel_stream;
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    lv_status st = reserve_frontier(ctx, S->sel, frontier, s);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, S->vis.reserve(stride * n * 8));
    LV_CUDA(ctx, S->h_vis.reserve(stride * n * 8));
    S->vis_stride = stride;
    LV_CUDA(ctx, S->res.reserve(sizeof(uint32_t) * LV_SELECT_RESULT_WORDS * n));
    LV_CUDA(ctx, S->h_res.reserve(sizeof(uint32_t) * LV_SELECT_RESULT_WORDS * n));
    LV_CUDA(ctx, S->views.reserve(sizeof(LodView) * n));
    LV_CUDA(ctx, S->h_views.reserve(sizeof(LodView) * n));
    LodView* hv = S->h_views.as<LodView>();
    uint32_t roots = 0, depth = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        const lv_request& q = cand[i]->r;
        lv_lod_params lod = q.desc.lod;
        if (lod.window_height == 0)
            lod.window_height = q.desc.height;
        st = make_lod_view(ctx, q.volume->info, q.desc.camera, lod, hv[i]);
        if (st != LV_OK)
            return st;
        hv[i].out_ids = S->vis.as<uint64_t>() + stride * i;
        hv[i].capacity = uint32_t(stride);
        hv[i].result = S->res.as<uint32_t>() + LV_SELECT_RESULT_WORDS * i;
        hv[i].root_offset = roots;
        roots += q.volume->info.root_blocks[0] * q.volume->info.root_blocks[1] *
                 q.volume->info.root_blocks[2];
        depth = std::max(depth, q.volume->info.depth);
    }
    LV_CUDA(ctx, cudaEventRecord(S->sel_t0, s));
    {
        const uint32_t words = uint32_t(sizeof(LodView) * n / 4);
        views_from_host_kernel<<<(words + 255) / 256, 256, 0, s>>>(
            static_cast<const uint32_t*>(S->h_views.dev), S->views.as<uint32_t>(), words);
        LV_CUDA(ctx, cudaGetLastError());
    }
    st = enqueue_selection(ctx, S->sel, S->views.as<LodView>(), n, roots, depth, s);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaEventRecord(S->sel_t1, s));
    selection_to_host_kernel<<<n, 256, 0, s>>>(S->res.as<uint32_t>(), S->vis.as<uint64_t>(),
                                               uint32_t(stride),
                                               static_cast<uint32_t*>(S->h_res.dev),
                                               static_cast<uint64_t*>(S->h_vis.dev));
    LV_CUDA(ctx, cudaGetLastError());
    LV_CUDA(ctx, cudaEventSynchronize(S->sel_t1));
    const double t_kernels = now_ms();
    float dev_ms = 0.f;
    if (cudaEventElapsedTime(&dev_ms, S->sel_t0, S->sel_t1) != cudaSuccess)
        cudaGetLastError();
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    visible.assign(n, {});
    const uint32_t* hr = S->h_res.as<uint32_t>();
    for (uint32_t i = 0; i < n; ++i)
    {
        const uint32_t k = hr[LV_SELECT_RESULT_WORDS * i + LV_SEL_WRITTEN];
        const uint64_t* p = S->h_vis.as<uint64_t>() + stride * i;
        visible[i].assign(p, p + k);
    }
    add_time(S, &lv_server_profile::select_device_ms, dev_ms);
    add_time(S, &lv_server_profile::select_ids_ms, now_ms() - t_kernels);
    return LV_OK;
}

/* Slots a brick of `units` can take: free, never used, or evictable. */
uint64_t available_units(lv_ctx* ctx, uint32_t units)
{
    Pool& P = *ctx->pool;
    uint64_t avail = (P.capacity_units - P.bump) / units;
    auto fl = P.free_by_units.find(units);
    if (fl != P.free_by_units.end())
        avail += fl->second.size();
    const uint64_t res = P.resident_count[units], pin = P.pinned_count[units];
    return avail + (res > pin ? res - pin : 0);
}

/* Admits a FIFO prefix of the candidates; streams their misses, pins them. */
void admit(lv_server* S, std::vector<Req*>& cand, std::vector<Req*>& admitted,
           std::vector<Req*>& rejected)
{
    std::vector<std::vector<uint64_t>> vis;
    const double t0 = now_ms();
    lv_status st = dry_run(S, cand, vis);
    add_time(S, &lv_server_profile::select_ms, now_ms() - t0);
    if (st != LV_OK)
    {
        rejected = cand;
        return;
    }
    lv_ctx* ctx = S->ctx;
    for (size_t i = 0; i < cand.size(); ++i)
    {
        Req* r = cand[i];
        lv_volume* v = r->r.volume;
        if (v->pins.size() != v->n_nodes)
            v->pins.assign(v->n_nodes, 0);
        Pool& P = *ctx->pool;
        std::vector<uint64_t> missing, idxs, missing_idx;
        for (uint64_t id : vis[i])
        {
            const uint64_t idx = node_index(v->level_offset, v->info.root_blocks, id);
            idxs.push_back(idx);
            if (v->host_table[idx] < 0)
            {
                missing.push_back(id);
                missing_idx.push_back(idx);
            }
        }
        const uint64_t capacity = P.capacity_units / v->slot_units;
        if (vis[i].size() > capacity)
        {
            r->status = LV_ENOMEM; /* can never fit */
            rejected.push_back(r);
            continue;
        }
        /* pin first, so streaming this request's misses cannot evict its
         * own resident bricks */
        for (uint64_t idx : idxs)
            if (v->pins[idx]++ == 0 && v->host_table[idx] >= 0)
                ++P.pinned_count[v->slot_units];
        auto unpin = [&]() {
            for (uint64_t idx : idxs)
                if (--v->pins[idx] == 0 && v->host_table[idx] >= 0)
                    --P.pinned_count[v->slot_units];
        };
        if (!missing.empty() && missing.size() > available_units(ctx, v->slot_units))
        {
            unpin();
            break; /* FIFO: wait for in-flight requests to release bricks */
        }
        uint32_t loaded = 0;
        uint64_t bytes = 0;
        const double t1 = now_ms();
        st = stream_bricks(ctx, v, missing.data(), uint32_t(missing.size()), 0xFFFFFFFFu,
                           S->sel_stream, loaded, bytes);
        add_time(S, &lv_server_profile::stream_ms, now_ms() - t1);
        /* bricks that became resident while pinned now count as pinned */
        for (uint64_t idx : missing_idx)
            if (v->host_table[idx] >= 0 && v->pins[idx] > 0)
                ++P.pinned_count[v->slot_units];
        if (st != LV_OK)
        {
            unpin();
            r->status = st;
            rejected.push_back(r);
            continue;
        }
        r->pinned = idxs;
        r->t_admit = now_ms();
        admitted.push_back(r);
    }
}

void loop_batched(lv_server* S)
{
    lv_ctx* ctx = S->ctx;
    cudaSetDevice(ctx->device);
    for (;;)
    {
        std::vector<Req*> cand;
        {
            std::unique_lock<std::mutex> lk(S->m);
            /* complete finished batches */
            while (!S->inflight.empty() && cudaEventQuery(S->inflight.front().ev) == cudaSuccess)
            {
                Inflight f = S->inflight.front();
                S->inflight.pop_front();
                lk.unlock();
                complete(S, f);
                lk.lock();
            }
            if (S->queue.empty())
            {
                if (!S->inflight.empty())
                {
                    Inflight f = S->inflight.front();
                    S->inflight.pop_front();
                    lk.unlock();
                    wait_batch(S, f.ev);
                    complete(S, f);
                    continue;
                }
                if (S->stop)
                    return;
                S->cv.wait(lk, [&] { return S->stop || !S->queue.empty(); });
                continue;
            }
            if (S->inflight.size() >= kSlots)
            {
                Inflight f = S->inflight.front();
                S->inflight.pop_front();
                lk.unlock();
                wait_batch(S, f.ev);
                complete(S, f);
                continue;
            }
            uint64_t pixels = 0;
            for (size_t i = 0; i < S->queue.size() && cand.size() < S->cfg.max_batch; ++i)
            {
                const lv_render_desc& d = S->queue[i]->r.desc;
                const uint64_t p = d.rect[2] && d.rect[3] ? uint64_t(d.rect[2]) * d.rect[3]
                                                          : uint64_t(d.width) * d.height;
                if (!cand.empty() && S->cfg.max_pixels && pixels + p > S->cfg.max_pixels)
                    break;
                pixels += p;
                cand.push_back(S->queue[i]);
            }
        }
        std::vector<Req*> admitted, rejected;
        {
            std::lock_guard<std::mutex> lk(ctx->mutex);
            ++ctx->foreign_pool_use; /* its batches read pool slots */
            admit(S, cand, admitted, rejected);
            if (!admitted.empty())
                cudaEventRecord(S->uploads_done, S->sel_stream);
        }
        {
            std::lock_guard<std::mutex> lk(S->m);
            for (Req* r : admitted)
                S->queue.erase(std::find(S->queue.begin(), S->queue.end(), r));
            for (Req* r : rejected)
                S->queue.erase(std::find(S->queue.begin(), S->queue.end(), r));
        }
        for (Req* r : rejected)
            fail_request(S, r, r->status == LV_OK ? LV_EDEVICE : r->status);
        if (admitted.empty())
        {
            /* nothing fits until an in-flight batch releases bricks */
            std::unique_lock<std::mutex> lk(S->m);
            if (!S->inflight.empty())
            {
                Inflight f = S->inflight.front();
                S->inflight.pop_front();
                lk.unlock();
                wait_batch(S, f.ev);
                complete(S, f);
            }
            else if (!rejected.size())
            {
                /* pool too small for the head request even when idle */
                Req* r = S->queue.front();
                S->queue.pop_front();
                lk.unlock();
                fail_request(S, r, LV_EAGAIN);
            }
            continue;
        }
        std::vector<lv_batch_view> bv(admitted.size());
        for (size_t i = 0; i < admitted.size(); ++i)
        {
            bv[i].volume = admitted[i]->r.volume;
            bv[i].tf = admitted[i]->r.tf;
            bv[i].desc = admitted[i]->r.desc;
            bv[i].desc.max_uploads = 0;
            bv[i].d_rgba = admitted[i]->r.d_rgba;
            admitted[i]->batch_size = uint32_t(admitted.size());
        }
        const int bi = S->cur;
        lv_batch* b = S->batches[bi];
        S->cur = (S->cur + 1) % kSlots;
        cudaStream_t ls = S->launch_stream[bi];
        Inflight f;
        f.batch = b;
        for (Req* r : admitted)
        {
            f.tickets.push_back(r->ticket);
            f.pins.emplace_back(r->r.volume, std::move(r->pinned));
            r->pinned.clear();
        }
        {
            /* the batch object's previous launch (and its hooks) ended
             * before this one is enqueued: lv_batch_render waits for it */
            std::lock_guard<std::mutex> lk(S->m);
            S->current[bi] = f.tickets;
        }
        /* one priority level below each batch still rendering: the oldest
         * requests keep the SM slots first */
        int level;
        {
            std::lock_guard<std::mutex> lk(S->m);
            level = int(S->inflight.size());
        }
        batch_set_priority_level(b, level);
        cudaStreamWaitEvent(ls, S->uploads_done, 0);
        const double t_launch = now_ms();
        const lv_status st = lv_batch_render(b, bv.data(), uint32_t(bv.size()), ls);
        add_time(S, &lv_server_profile::launch_ms, now_ms() - t_launch);
        {
            std::lock_guard<std::mutex> lk(S->m);
            if (!S->free_events.empty())
            {
                f.ev = S->free_events.back();
                S->free_events.pop_back();
            }
        }
        if (!f.ev)
            cudaEventCreateWithFlags(&f.ev, cudaEventDisableTiming);
        f.clock = std::make_shared<DoneClock>();
        cudaLaunchHostFunc(ls, stamp_done, f.clock.get());
        cudaEventRecord(f.ev, ls);
        if (st != LV_OK)
        {
            f.status = st;
            f.batch = nullptr;
        }
        std::lock_guard<std::mutex> lk(S->m);
        S->inflight.push_back(std::move(f));
        ++S->n_batches;
    }
}

void loop_plain(lv_server* S)
{
    cudaSetDevice(S->ctx->device);
    for (;;)
    {
        Req* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->m);
            S->cv.wait(lk, [&] { return S->stop || !S->queue.empty(); });
            if (S->queue.empty())
                return;
            r = S->queue.front();
            S->queue.pop_front();
        }
        r->t_admit = now_ms();
        r->batch_size = 1;
        lv_render_desc d = r->r.desc;
        d.synchronous = 1;
        const double t0 = now_ms();
        lv_status st = lv_render(S->ctx, r->r.volume, r->r.tf, &d, r->r.d_rgba,
                                 S->launch_stream[0]);
        if (st == LV_OK)
            st = lv_last_stats(S->ctx, &r->stats); /* synchronises */
        std::lock_guard<std::mutex> lk(S->m);
        S->prof.launch_ms += now_ms() - t0;
        S->prof.device_ms += r->stats.select_ms + r->stats.raycast_ms;
        S->prof.raycast_ms += r->stats.raycast_ms;
        ++S->prof.requests;
        r->status = st;
        r->t_done = now_ms();
        r->done = true;
        ++S->n_done;
        ++S->n_batches;
        S->cv_done.notify_all();
    }
}
} // namespace

extern "C" lv_status lv_server_create(lv_ctx* ctx, const lv_server_config* cfg, lv_server** out)
{
    if (!ctx || !cfg || !out || cfg->max_batch == 0)
        return fail(ctx, LV_EINVAL, "invalid server configuration");
    {
        std::lock_guard<std::mutex> lk(ctx->mutex);
        LV_CUDA(ctx, cudaSetDevice(ctx->device));
        lv_status st = ensure_renderer(ctx);
        if (st != LV_OK)
            return st;
        if (!ctx->pool)
            return fail(ctx, LV_EINVAL, "create the volumes before the server");
    }
    lv_server* S = new lv_server();
    S->ctx = ctx;
    S->cfg = *cfg;
    /* admission selections take the next free SM slots ahead of batch work */
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (cudaStreamCreateWithPriority(&S->sel_stream, cudaStreamNonBlocking, hi_prio) !=
            cudaSuccess ||
        cudaEventCreateWithFlags(&S->uploads_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&S->sel_t0) != cudaSuccess || cudaEventCreate(&S->sel_t1) != cudaSuccess)
    {
        delete S;
        return fail(ctx, LV_EDEVICE, "server streams");
    }
    for (int i = 0; i < kSlots; ++i)
        if (cudaStreamCreateWithFlags(&S->launch_stream[i], cudaStreamNonBlocking) != cudaSuccess)
        {
            delete S;
            return fail(ctx, LV_EDEVICE, "server streams");
        }
    for (int i = 0; i < kSlots; ++i)
    {
        lv_status st = lv_batch_create(ctx, &S->batches[i]);
        if (st != LV_OK)
        {
            delete S;
            return st;
        }
        lv_batch_config bc;
        lv_batch_get_config(S->batches[i], &bc);
        bc.use_graph = cfg->use_graph;
        if (cfg->tile_w)
        {
            bc.tile_w = cfg->tile_w;
            bc.tile_h = cfg->tile_h;
            bc.ctas_per_sm = cfg->ctas_per_sm ? cfg->ctas_per_sm : bc.ctas_per_sm;
        }
        lv_batch_set_config(S->batches[i], &bc);
        S->hooks[i] = lv_server_hook{S, i};
        batch_set_view_hook(S->batches[i], view_done, &S->hooks[i]);
    }
    S->th = std::thread(cfg->mode == LV_SERVE_PLAIN ? loop_plain : loop_batched, S);
    *out = S;
    return LV_OK;
}

extern "C" lv_status lv_server_submit(lv_server* S, const lv_request* req, uint64_t* ticket)
{
    if (!S || !req || !ticket || !req->volume || !req->tf || !req->d_rgba ||
        req->volume->ctx != S->ctx || req->tf->ctx != S->ctx || !req->desc.width ||
        !req->desc.height)
        return LV_EINVAL;
    Req* r = new Req();
    r->r = *req;
    r->t_submit = now_ms();
    std::lock_guard<std::mutex> lk(S->m);
    if (S->stop)
    {
        delete r;
        return LV_EINVAL;
    }
    if (S->cfg.max_queue && S->queue.size() >= S->cfg.max_queue)
    {
        delete r;
        return LV_EAGAIN;
    }
    r->ticket = S->next_ticket++;
    S->reqs[r->ticket] = r;
    S->queue.push_back(r);
    *ticket = r->ticket;
    S->cv.notify_one();
    return LV_OK;
}

extern "C" lv_status lv_server_wait(lv_server* S, uint64_t ticket, uint32_t timeout_ms,
                                    lv_request_result* out)
{
    if (!S || !out)
        return LV_EINVAL;
    std::unique_lock<std::mutex> lk(S->m);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end())
        return LV_ENOTFOUND;
    Req* r = it->second;
    if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; }))
        return LV_ETIMEDOUT;
    out->status = r->status;
    out->latency_ms = r->t_done - r->t_submit;
    out->queue_ms = r->t_admit - r->t_submit;
    out->batch_size = r->batch_size;
    out->stats = r->stats;
    S->reqs.erase(it);
    delete r;
    return LV_OK;
}

extern "C" lv_status lv_server_get_profile(lv_server* S, lv_server_profile* out)
{
    if (!S || !out)
        return LV_EINVAL;
    uint64_t captures = 0;
    for (lv_batch* b : S->batches)
    {
        uint64_t c = 0;
        if (b && lv_batch_graph_stats(b, &c, nullptr, nullptr) == LV_OK)
            captures += c;
    }
    std::lock_guard<std::mutex> lk(S->m);
    *out = S->prof;
    out->batches = S->n_batches;
    out->graph_captures = captures;
    return LV_OK;
}

extern "C" lv_status lv_server_counters(lv_server* S, uint64_t* completed, uint64_t* batches,
                                        uint64_t* queued)
{
    if (!S)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lk(S->m);
    if (completed)
        *completed = S->n_done;
    if (batches)
        *batches = S->n_batches;
    if (queued)
        *queued = S->queue.size();
    return LV_OK;
}

extern "C" void lv_server_destroy(lv_server* S)
{
    if (!S)
        return;
    {
        std::lock_guard<std::mutex> lk(S->m);
        S->stop = true;
        S->cv.notify_all();
    }
    if (S->th.joinable())
        S->th.join();
    cudaSetDevice(S->ctx->device);
    for (auto& f : S->inflight)
    {
        cudaEventSynchronize(f.ev);
        for (cudaStream_t ls : S->launch_stream)
            cudaStreamSynchronize(ls); /* host functions done */
        complete(S, f);
    }
    for (int i = 0; i < kSlots; ++i)
        lv_batch_destroy(S->batches[i]);
    for (cudaEvent_t e : S->free_events)
        cudaEventDestroy(e);
    for (auto& kv : S->reqs)
        delete kv.second;
    if (S->sel_stream)
        cudaStreamDestroy(S->sel_stream);
    for (cudaStream_t ls : S->launch_stream)
        if (ls)
            cudaStreamDestroy(ls);
    if (S->uploads_done)
        cudaEventDestroy(S->uploads_done);
    if (S->sel_t0)
        cudaEventDestroy(S->sel_t0);
    if (S->sel_t1)
        cudaEventDestroy(S->sel_t1);
    delete S;
}
