/*
 * Per-brick value histograms on the device.
 *
 * Restates HistogramObject (livre/lib/cache/HistogramObject.cpp:30-224) and
 * the accumulation of HistogramFilter::execute (livre/lib/pipeline/
 * HistogramFilter.cpp:78-149) for one full viewport:
 *  - only the brick's own voxels count (the overlap is skipped);
 *  - each count is weighted by the number of finest-level voxels one voxel of
 *    the brick stands for, (2^(depth - 1 - level))^3;
 *  - the bin of value v over n bins and the data range [lo, hi] is
 *    floor((v - lo) * (n - 1) / (hi - lo)), clamped to [0, n - 1]; for uint8
 *    with 256 bins over [0, 255] this is the reference's bin = v. (The
 *    reference's integer bin width for 16-bit data divides by zero or writes
 *    past its bins for small or large ranges; the same formula is used for
 *    every type here.)
 * One CTA per brick builds the histogram in shared memory from the brick in
 * the HBM pool, then adds it (64-bit) to the per-brick and accumulated
 * outputs.
 */
#include <algorithm>
#include <vector>

#include "lv_runtime.h"

namespace
{
using namespace lv;

struct HistJob
{
    uint64_t offset; /* brick byte offset in the pool */
    uint64_t scale;  /* finest voxels per brick voxel */
};

template <int DT>
__global__ void __launch_bounds__(256)
    histogram_kernel(const uint8_t* __restrict__ pool, const HistJob* __restrict__ jobs,
                     uint32_t N0, uint32_t N1, uint32_t N2, uint32_t O0, uint32_t O1,
                     uint32_t O2, uint32_t dt, uint32_t u8_stride, uint32_t n_bins, float lo,
                     float scale_bins,
                     unsigned long long* __restrict__ per_brick,
                     unsigned long long* __restrict__ acc)
{
    extern __shared__ uint32_t bins[];
    for (uint32_t b = threadIdx.x; b < n_bins; b += blockDim.x)
        bins[b] = 0;
    __syncthreads();
    const HistJob job = jobs[blockIdx.x];
    const uint8_t* brick = pool + job.offset;
    const uint32_t B0 = N0 - 2 * O0, B1 = N1 - 2 * O1, B2 = N2 - 2 * O2;
    const uint32_t total = B0 * B1 * B2;
    for (uint32_t i = threadIdx.x; i < total; i += blockDim.x)
    {
        const uint32_t x = i % B0 + O0, y = (i / B0) % B1 + O1, z = i / (B0 * B1) + O2;
        const uint32_t idx = (z * N1 + y) * N0 + x;
        float v;
        if (DT == LV_DT_UINT16)
            v = float(reinterpret_cast<const uint16_t*>(brick)[idx]);
        else if (DT == LV_DT_UINT8)
            v = float(brick[u8_stride * idx]); /* 4: voxel quads, the element's byte 0 */
        else /* kDtAny: the voxel type `dt` */
            switch (dt)
            {
            case LV_DT_INT8: v = float(reinterpret_cast<const int8_t*>(brick)[idx]); break;
            case LV_DT_INT16: v = float(reinterpret_cast<const int16_t*>(brick)[idx]); break;
            case LV_DT_UINT32:
                v = __uint2float_rn(reinterpret_cast<const uint32_t*>(brick)[idx]);
                break;
            case LV_DT_INT32:
                v = __int2float_rn(reinterpret_cast<const int32_t*>(brick)[idx]);
                break;
            default: v = reinterpret_cast<const float*>(brick)[idx]; break;
            }
        const float f = floorf((v - lo) * scale_bins);
        const int bin = int(fminf(fmaxf(f, 0.0f), float(n_bins - 1)));
        atomicAdd(&bins[bin], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < n_bins; b += blockDim.x)
    {
        const unsigned long long c = (unsigned long long)bins[b] * job.scale;
        if (per_brick)
            per_brick[uint64_t(blockIdx.x) * n_bins + b] = c;
        if (c)
            atomicAdd(&acc[b], c);
    }
}
} // namespace

extern "C" lv_status lv_histogram(lv_volume* vol, const uint64_t* ids, uint32_t n,
                                  uint32_t n_bins, float range_lo, float range_hi,
                                  uint64_t* per_brick, uint64_t* accumulated)
{
    if (!vol || (n && !ids) || !accumulated || n_bins < 2 || n_bins > 8192 ||
        !(range_hi > range_lo))
        return LV_EINVAL;
    lv_ctx* ctx = vol->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->upload_stream;
    std::fill(accumulated, accumulated + n_bins, uint64_t(0));
    if (n == 0)
        return LV_OK;
    /* the bricks must be resident: load the missing ones (nothing in flight
     * is protected beyond this call) */
    uint32_t loaded = 0;
    uint64_t bytes = 0;
    lv_status st = stream_bricks(ctx, vol, ids, n, ctx->renderer->frame + 1u, s, loaded, bytes);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    std::vector<HistJob> jobs(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        const uint64_t id = ids[i];
        const uint32_t L = nid_level(id);
        if (L >= vol->info.depth)
            return fail(ctx, LV_EINVAL, "node id outside the volume");
        const uint64_t idx = node_index(vol->level_offset, vol->info.root_blocks, id);
        if (idx >= vol->n_nodes || vol->host_table[idx] < 0)
            return fail(ctx, LV_ENOTFOUND, "brick not resident (no data for the node)");
        const uint64_t side = uint64_t(1) << (vol->info.depth - 1u - L);
        jobs[i].offset = uint64_t(vol->host_table[idx]) * kSlotUnit;
        jobs[i].scale = side * side * side;
    }
    DeviceBuffer djobs, dout, dacc;
    LV_CUDA(ctx, djobs.reserve(sizeof(HistJob) * n));
    LV_CUDA(ctx, dacc.reserve(sizeof(uint64_t) * n_bins));
    if (per_brick)
        LV_CUDA(ctx, dout.reserve(sizeof(uint64_t) * n_bins * n));
    LV_CUDA(ctx, cudaMemcpyAsync(djobs.ptr, jobs.data(), sizeof(HistJob) * n,
                                 cudaMemcpyHostToDevice, s));
    LV_CUDA(ctx, cudaMemsetAsync(dacc.ptr, 0, sizeof(uint64_t) * n_bins, s));
    const float scale_bins = float(n_bins - 1) / (range_hi - range_lo);
    const size_t smem = sizeof(uint32_t) * n_bins;
    const auto& I = vol->info;
    auto kernel = I.dtype == LV_DT_UINT16  ? histogram_kernel<LV_DT_UINT16>
                  : I.dtype == LV_DT_UINT8 ? histogram_kernel<LV_DT_UINT8>
                                           : histogram_kernel<kDtAny>;
    kernel<<<n, 256, smem, s>>>(ctx->pool->arena.as<uint8_t>(), djobs.as<HistJob>(),
                                I.max_block[0], I.max_block[1], I.max_block[2], I.overlap[0],
                                I.overlap[1], I.overlap[2], I.dtype, vol->stage_off ? 4u : 1u,
                                n_bins, range_lo, scale_bins,
                                per_brick ? dout.as<unsigned long long>() : nullptr,
                                dacc.as<unsigned long long>());
    LV_CUDA(ctx, cudaGetLastError());
    LV_CUDA(ctx, cudaMemcpyAsync(accumulated, dacc.ptr, sizeof(uint64_t) * n_bins,
                                 cudaMemcpyDeviceToHost, s));
    if (per_brick)
        LV_CUDA(ctx, cudaMemcpyAsync(per_brick, dout.ptr, sizeof(uint64_t) * n_bins * n,
                                     cudaMemcpyDeviceToHost, s));
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    return LV_OK;
}
