/*
 * Synthetic blob volume generator on the device.
 *
 * A voxel at level-L coordinate g (clamped to the level's extent) holds
 * round(255 * clamp(sum_i a_i exp(-|x - c_i|^2 / (2 sigma_i^2)))) + noise,
 * with x = (g + 0.5) * 2^(depth-1-L) in finest-level voxel units, blobs cut
 * off at 6 sigma and noise U[-k, k] from a SplitMix64 hash of
 * (seed, L, g). Bricks are (block + 2 * overlap)^3 voxels, x fastest, like
 * the MemoryUnit a DataSourcePlugin returns (livre/data/MemoryUnit.h:33-167).
 *
 * Every float operation is an explicit round-to-nearest intrinsic in a fixed
 * order, and exp is evaluated by a fixed polynomial, so the bytes do not
 * depend on the compiler or on the device math library.
 */
#include <cmath>
#include <vector>

#include "lv_runtime.h"

namespace lv
{
struct Blob
{
    float cx, cy, cz, inv2s2, cut2, amp;
};

namespace
{
inline uint64_t splitmix_next(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline float unit24(uint64_t r)
{
    return float(r >> 40) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* e^x for x <= 0: 2^(x log2 e) = 2^n * 2^f, 2^f by its degree-7 Taylor
 * series (coefficients (ln 2)^k / k!) in Horner form. */
__device__ __forceinline__ float exp_neg(float x)
{
    if (x < -80.0f)
        return 0.0f;
    const float y = __fmul_rn(x, 1.44269504f);
    const float n = floorf(y);
    const float f = __fsub_rn(y, n);
    float p = 1.52527338e-05f;
    p = __fadd_rn(__fmul_rn(p, f), 0.000154035304f);
    p = __fadd_rn(__fmul_rn(p, f), 0.00133335581f);
    p = __fadd_rn(__fmul_rn(p, f), 0.00961812911f);
    p = __fadd_rn(__fmul_rn(p, f), 0.0555041087f);
    p = __fadd_rn(__fmul_rn(p, f), 0.240226507f);
    p = __fadd_rn(__fmul_rn(p, f), 0.693147182f);
    p = __fadd_rn(__fmul_rn(p, f), 1.0f);
    const float scale = __int_as_float((int(n) + 127) << 23);
    return __fmul_rn(p, scale);
}

struct GenParams
{
    uint32_t N[3];
    uint32_t B[3];
    uint32_t O[3];
    uint32_t voxels[3];
    uint32_t depth;
    uint32_t n_blobs;
    uint32_t noise;
    uint32_t dtype;
    uint64_t seed;
    uint64_t brick_bytes;
};

/* One block per brick: candidate blobs into shared memory, then voxels. */
__global__ void __launch_bounds__(256)
    blob_brick_kernel(GenParams P, const Blob* __restrict__ blobs,
                      const uint64_t* __restrict__ ids, uint8_t* __restrict__ out,
                      const uint64_t* __restrict__ offsets)
{
    extern __shared__ uint32_t cand[];
    __shared__ uint32_t n_cand;
    const uint64_t id = ids[blockIdx.x];
    uint8_t* dst = out + (offsets ? offsets[blockIdx.x]
                                  : uint64_t(blockIdx.x) * P.brick_bytes);
    const uint32_t L = nid_level(id);
    const uint32_t shift = P.depth - 1u - L;
    const uint32_t s = 1u << shift;
    const float fs = __uint2float_rn(s);
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    int32_t base[3], VL[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        VL[a] = int32_t((P.voxels[a] + s - 1u) >> shift);
        base[a] = int32_t(pos[a] * P.B[a]) - int32_t(P.O[a]);
    }
    if (threadIdx.x == 0)
        n_cand = 0;
    __syncthreads();
    /* conservative prefilter; the exact per-voxel cut-off decides */
    for (uint32_t b = threadIdx.x; b < P.n_blobs; b += blockDim.x)
    {
        const Blob bl = blobs[b];
        const float c[3] = {bl.cx, bl.cy, bl.cz};
        float d2 = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            int32_t lo = max(base[a], 0);
            int32_t hi = min(base[a] + int32_t(P.N[a]) - 1, VL[a] - 1);
            lo = min(lo, VL[a] - 1);
            hi = max(hi, 0);
            const float flo = (float(lo) + 0.5f) * fs - 1.0f;
            const float fhi = (float(hi) + 0.5f) * fs + 1.0f;
            float dd = 0.0f;
            if (c[a] < flo)
                dd = flo - c[a];
            else if (c[a] > fhi)
                dd = c[a] - fhi;
            d2 += dd * dd;
        }
        if (d2 < bl.cut2 * 1.01f + 1.0f)
        {
            const uint32_t k = atomicAdd(&n_cand, 1u);
            cand[k] = b;
        }
    }
    __syncthreads();
    /* restore index order so the sum runs over blobs in ascending index */
    if (threadIdx.x == 0)
    {
        const uint32_t n = n_cand;
        for (uint32_t i = 1; i < n; ++i)
        {
            const uint32_t v = cand[i];
            uint32_t j = i;
            while (j > 0 && cand[j - 1] > v)
            {
                cand[j] = cand[j - 1];
                --j;
            }
            cand[j] = v;
        }
    }
    __syncthreads();
    const uint32_t nc = n_cand;
    const uint32_t total = P.N[0] * P.N[1] * P.N[2];
    for (uint32_t idx = threadIdx.x; idx < total; idx += blockDim.x)
    {
        const uint32_t i = idx % P.N[0];
        const uint32_t j = (idx / P.N[0]) % P.N[1];
        const uint32_t k = idx / (P.N[0] * P.N[1]);
        const int32_t g0 = min(max(base[0] + int32_t(i), 0), VL[0] - 1);
        const int32_t g1 = min(max(base[1] + int32_t(j), 0), VL[1] - 1);
        const int32_t g2 = min(max(base[2] + int32_t(k), 0), VL[2] - 1);
        const float x = __fmul_rn(__fadd_rn(__int2float_rn(g0), 0.5f), fs);
        const float y = __fmul_rn(__fadd_rn(__int2float_rn(g1), 0.5f), fs);
        const float z = __fmul_rn(__fadd_rn(__int2float_rn(g2), 0.5f), fs);
        float acc = 0.0f;
        for (uint32_t c = 0; c < nc; ++c)
        {
            const Blob bl = blobs[cand[c]];
            const float dx = __fsub_rn(x, bl.cx);
            const float dy = __fsub_rn(y, bl.cy);
            const float dz = __fsub_rn(z, bl.cz);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                       __fmul_rn(dz, dz));
            if (d2 < bl.cut2)
                acc = __fadd_rn(acc, __fmul_rn(bl.amp, exp_neg(-__fmul_rn(d2, bl.inv2s2))));
        }
        const float v = fminf(fmaxf(acc, 0.0f), 1.0f);
        int32_t noise = 0;
        if (P.noise)
        {
            const uint64_t M = 0x100000001B3ull;
            uint64_t key = P.seed;
            key = key * M + L;
            key = key * M + uint32_t(g0);
            key = key * M + uint32_t(g1);
            key = key * M + uint32_t(g2);
            noise = int32_t(mix64(key) % (2u * P.noise + 1u)) - int32_t(P.noise);
        }
        if (P.dtype == LV_DT_UINT16)
        {
            int32_t q = int32_t(floorf(__fadd_rn(__fmul_rn(v, 65535.0f), 0.5f))) + noise * 257;
            q = min(max(q, 0), 65535);
            reinterpret_cast<uint16_t*>(dst)[idx] = uint16_t(q);
        }
        else
        {
            int32_t q = int32_t(floorf(__fadd_rn(__fmul_rn(v, 255.0f), 0.5f))) + noise;
            q = min(max(q, 0), 255);
            dst[idx] = uint8_t(q);
        }
    }
}
} // namespace

std::vector<Blob> make_blobs(const lv_volume_info& v, const lv_blob_desc& d)
{
    std::vector<Blob> blobs(d.n_blobs);
    uint64_t s = d.seed;
    for (uint32_t i = 0; i < d.n_blobs; ++i)
    {
        Blob& b = blobs[i];
        b.cx = unit24(splitmix_next(s)) * float(v.voxels[0]);
        b.cy = unit24(splitmix_next(s)) * float(v.voxels[1]);
        b.cz = unit24(splitmix_next(s)) * float(v.voxels[2]);
        const float sigma = 8.0f + 24.0f * unit24(splitmix_next(s));
        b.amp = 0.3f + 0.7f * unit24(splitmix_next(s));
        b.inv2s2 = 1.0f / (2.0f * sigma * sigma);
        const float c = 6.0f * sigma;
        b.cut2 = c * c;
    }
    return blobs;
}

/* Launches the generator for n bricks: brick i of ids goes to
 * out + offsets[i] (device array) or, when offsets is null, to
 * out + i * brick_bytes. */
lv_status launch_blob_bricks(lv_ctx* ctx, const lv_volume_info& v,
                             const lv_blob_desc& d, const Blob* d_blobs,
                             const uint64_t* d_ids, uint32_t n, uint8_t* out,
                             const uint64_t* d_offsets, cudaStream_t stream)
{
    if (v.dtype != LV_DT_UINT8 && v.dtype != LV_DT_UINT16)
        return fail(ctx, LV_EINVAL, "blob volumes are uint8 or uint16");
    GenParams P;
    for (int a = 0; a < 3; ++a)
    {
        P.N[a] = v.max_block[a];
        P.O[a] = v.overlap[a];
        P.B[a] = v.max_block[a] - 2u * v.overlap[a];
        P.voxels[a] = v.voxels[a];
    }
    P.depth = v.depth;
    P.n_blobs = d.n_blobs;
    P.noise = d.noise;
    P.dtype = v.dtype;
    P.seed = d.seed;
    P.brick_bytes = uint64_t(P.N[0]) * P.N[1] * P.N[2] *
                    (v.dtype == LV_DT_UINT16 ? 2u : 1u);
    if (n == 0)
        return LV_OK;
    const size_t smem = sizeof(uint32_t) * (d.n_blobs ? d.n_blobs : 1);
    if (smem > 48 * 1024)
        return fail(ctx, LV_EINVAL, "too many blobs (max 12288)");
    blob_brick_kernel<<<n, 256, smem, stream>>>(P, d_blobs, d_ids, out, d_offsets);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

} // namespace lv

extern "C" lv_status lv_blob_generate(lv_ctx* ctx, const lv_volume_info* info,
                                      const lv_blob_desc* blob,
                                      const uint64_t* ids, uint32_t n,
                                      void* d_out, void* stream)
{
    using namespace lv;
    if (!ctx || !info || !blob || (n && (!ids || !d_out)))
        return fail(ctx, LV_EINVAL, "null argument");
    if (info->depth == 0)
        return fail(ctx, LV_EINVAL, "volume info not filled");
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const std::vector<Blob> blobs = make_blobs(*info, *blob);
    DeviceBuffer dblobs, dids;
    LV_CUDA(ctx, dblobs.reserve(sizeof(Blob) * (blobs.size() + 1)));
    LV_CUDA(ctx, dids.reserve(sizeof(uint64_t) * (n + 1)));
    LV_CUDA(ctx, cudaMemcpyAsync(dblobs.ptr, blobs.data(), sizeof(Blob) * blobs.size(),
                                 cudaMemcpyHostToDevice, s));
    LV_CUDA(ctx, cudaMemcpyAsync(dids.ptr, ids, sizeof(uint64_t) * n,
                                 cudaMemcpyHostToDevice, s));
    lv_status st = launch_blob_bricks(ctx, *info, *blob, dblobs.as<Blob>(),
                                      dids.as<uint64_t>(), n,
                                      static_cast<uint8_t*>(d_out), nullptr, s);
    if (st != LV_OK)
        return st;
    /* the temporaries are freed on return: finish before that */
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    return LV_OK;
}
