/*
 * Host runtime shared by the livre_gb300 translation units: device buffers,
 * the context (streams, scratch, pinned staging), error handling.
 */
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

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

/* Owning page-locked host buffer that only grows. */
struct PinnedBuffer
{
    void* ptr = nullptr;
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
        bytes = 0;
    }
    cudaError_t reserve(size_t n)
    {
        if (n <= bytes)
            return cudaSuccess;
        release();
        cudaError_t e = cudaHostAlloc(&ptr, n < 256 ? 256 : n, cudaHostAllocDefault);
        if (e == cudaSuccess)
            bytes = n < 256 ? 256 : n;
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
};

struct Pool;
struct Renderer;

} // namespace lv

struct lv_ctx
{
    int device = 0;
    std::string error;
    cudaStream_t upload_stream = nullptr;
    lv::SelectScratch sel;
    lv::Pool* pool = nullptr;
    lv::Renderer* renderer = nullptr;
    size_t pool_bytes = size_t(3072) << 20;
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
                        cudaStream_t stream);

/* Frontier size needed for a full traversal of a volume. */
uint64_t max_frontier(const lv_volume_info& vol);

/* Applies the sort-last range slice of SelectVisibles::visitPost to one
 * view (restores DFS order first). Synchronises `stream`. */
lv_status range_slice(lv_ctx* ctx, const lv_volume_info& vol,
                      const float range[2], uint64_t* d_ids, uint32_t* d_result,
                      cudaStream_t stream);

} // namespace lv
