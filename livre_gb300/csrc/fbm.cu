/*
 * Procedural fBm volume: fractal Brownian motion over improved Perlin noise
 * (K. Perlin, "Improving Noise", SIGGRAPH 2002: quintic fade, 12 edge
 * gradients picked by the low 4 bits of the hash, a 256-entry permutation
 * table repeated twice), `octaves` octaves of lacunarity and gain, mapped
 * linearly from [-1, 1] to the full range of the voxel type.
 *
 * The permutation is the identity shuffled by Fisher-Yates with SplitMix64
 * draws from the seed (j = draw mod (i + 1), i from 255 down to 1). A voxel
 * at level-L coordinate g (clamped to the level's extent, as the blob
 * volumes) samples the field at x = (g + 0.5) * 2^(depth-1-L) * frequency /
 * max(voxels), in finest-level voxel units scaled so that `frequency` noise
 * periods span the volume.
 *
 * Every float operation is IEEE single precision in a fixed order with no
 * contraction (the device code uses explicit round-to-nearest intrinsics,
 * the host code is built without FP contraction), so the host generator,
 * which a data-source plugin calls per brick, and the device generator,
 * which writes bricks straight into the pool, give the same bytes.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "lv_runtime.h"

namespace lv
{
namespace
{
inline uint64_t splitmix_draw(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Operations shared by the host and device generators: FADD/FMUL with
 * round-to-nearest and no fusion. */
struct HostOps
{
    static float add(float a, float b) { return a + b; }
    static float sub(float a, float b) { return a - b; }
    static float mul(float a, float b) { return a * b; }
};
struct DeviceOps
{
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
};

template <typename O>
__host__ __device__ __forceinline__ float fade(float t)
{
    /* t^3 (t (6 t - 15) + 10) */
    const float a = O::add(O::mul(t, O::sub(O::mul(t, 6.0f), 15.0f)), 10.0f);
    return O::mul(O::mul(O::mul(t, t), t), a);
}

template <typename O>
__host__ __device__ __forceinline__ float lerp(float t, float a, float b)
{
    return O::add(a, O::mul(t, O::sub(b, a)));
}

template <typename O>
__host__ __device__ __forceinline__ float grad(uint32_t h, float x, float y, float z)
{
    h &= 15u;
    const float u = h < 8u ? x : y;
    const float v = h < 4u ? y : (h == 12u || h == 14u ? x : z);
    return O::add((h & 1u) ? -u : u, (h & 2u) ? -v : v);
}

template <typename O>
__host__ __device__ __forceinline__ float noise3(const uint16_t* P, float x, float y, float z)
{
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const uint32_t X = uint32_t(int32_t(fx)) & 255u, Y = uint32_t(int32_t(fy)) & 255u,
                   Z = uint32_t(int32_t(fz)) & 255u;
    x = O::sub(x, fx);
    y = O::sub(y, fy);
    z = O::sub(z, fz);
    const float u = fade<O>(x), v = fade<O>(y), w = fade<O>(z);
    const uint32_t A = P[X] + Y, AA = P[A] + Z, AB = P[A + 1] + Z;
    const uint32_t B = P[X + 1] + Y, BA = P[B] + Z, BB = P[B + 1] + Z;
    const float x1 = O::sub(x, 1.0f), y1 = O::sub(y, 1.0f), z1 = O::sub(z, 1.0f);
    const float l00 = lerp<O>(u, grad<O>(P[AA], x, y, z), grad<O>(P[BA], x1, y, z));
    const float l10 = lerp<O>(u, grad<O>(P[AB], x, y1, z), grad<O>(P[BB], x1, y1, z));
    const float l01 = lerp<O>(u, grad<O>(P[AA + 1], x, y, z1), grad<O>(P[BA + 1], x1, y, z1));
    const float l11 = lerp<O>(u, grad<O>(P[AB + 1], x, y1, z1), grad<O>(P[BB + 1], x1, y1, z1));
    return lerp<O>(w, lerp<O>(v, l00, l10), lerp<O>(v, l01, l11));
}

template <typename O>
__host__ __device__ __forceinline__ float fbm(const uint16_t* P, const lv_fbm_params& f, float x,
                                              float y, float z)
{
    float sum = 0.0f, amp = 1.0f, freq = 1.0f;
    for (uint32_t o = 0; o < f.octaves; ++o)
    {
        sum = O::add(sum, O::mul(amp, noise3<O>(P, O::mul(x, freq), O::mul(y, freq),
                                                O::mul(z, freq))));
        amp = O::mul(amp, f.gain);
        freq = O::mul(freq, f.lacunarity);
    }
    return sum;
}

/* [-1, 1] -> [0, full scale], rounded half up */
template <typename O>
__host__ __device__ __forceinline__ uint32_t quantise(float v, float full)
{
    v = fminf(fmaxf(v, -1.0f), 1.0f);
    const float q = O::add(O::mul(O::mul(O::add(v, 1.0f), 0.5f), full), 0.5f);
    return uint32_t(floorf(q));
}

/* Per-brick sampling constants. */
struct FbmBrick
{
    int32_t base[3];   /* level coordinate of the brick's first voxel */
    int32_t last[3];   /* level extent - 1 */
    uint32_t N[3];
    float scale;       /* 2^(depth-1-L) * frequency / max(voxels) */
};

__host__ __device__ __forceinline__ FbmBrick brick_consts(const lv_volume_info& v,
                                                          const lv_fbm_params& f, uint64_t id)
{
    FbmBrick b;
    const uint32_t L = nid_level(id);
    const uint32_t shift = v.depth - 1u - L;
    const uint32_t s = 1u << shift;
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    uint32_t vmax = v.voxels[0];
    vmax = vmax > v.voxels[1] ? vmax : v.voxels[1];
    vmax = vmax > v.voxels[2] ? vmax : v.voxels[2];
    for (int a = 0; a < 3; ++a)
    {
        b.N[a] = v.max_block[a];
        const uint32_t B = v.max_block[a] - 2u * v.overlap[a];
        b.base[a] = int32_t(pos[a] * B) - int32_t(v.overlap[a]);
        b.last[a] = int32_t((v.voxels[a] + s - 1u) >> shift) - 1;
    }
    b.scale = float(s) * (f.frequency / float(vmax));
    return b;
}

template <typename O>
__host__ __device__ __forceinline__ float fbm_at(const uint16_t* P, const lv_fbm_params& f,
                                                 const FbmBrick& b, uint32_t i, uint32_t j,
                                                 uint32_t k)
{
    auto clampi = [](int32_t g, int32_t hi) { return g < 0 ? 0 : (g > hi ? hi : g); };
    const int32_t gi = clampi(b.base[0] + int32_t(i), b.last[0]);
    const int32_t gj = clampi(b.base[1] + int32_t(j), b.last[1]);
    const int32_t gk = clampi(b.base[2] + int32_t(k), b.last[2]);
    const float x = O::mul(O::add(float(gi), 0.5f), b.scale);
    const float y = O::mul(O::add(float(gj), 0.5f), b.scale);
    const float z = O::mul(O::add(float(gk), 0.5f), b.scale);
    return fbm<O>(P, f, x, y, z);
}

/* The gradient of corner hash h at a point, split into its x part and the
 * rest: grad(h, x, y, z) = add(sx * x, c) when the gradient has an x
 * component (h < 8, 12, 14; sx = +-1, c the signed other component), else
 * the constant c = grad(h, x, y, z) itself. add(a, b) = add(b, a) exactly
 * and +-1 * x is exact, so this is the same single rounding as grad<O>. */
struct CornerGrad
{
    float sx, c;
    bool has_x;
};

__device__ __forceinline__ CornerGrad corner_grad(uint32_t h, float y, float z)
{
    h &= 15u;
    CornerGrad g;
    if (h < 8u)
    {
        g.has_x = true;
        g.sx = (h & 1u) ? -1.0f : 1.0f;
        const float v = h < 4u ? y : z;
        g.c = (h & 2u) ? -v : v;
    }
    else if (h == 12u || h == 14u)
    {
        g.has_x = true;
        g.sx = (h & 2u) ? -1.0f : 1.0f;
        g.c = (h & 1u) ? -y : y;
    }
    else
    {
        g.has_x = false;
        g.sx = 0.0f;
        g.c = DeviceOps::add((h & 1u) ? -y : y, (h & 2u) ? -z : z);
    }
    return g;
}

__device__ __forceinline__ float corner_value(const CornerGrad& g, float x)
{
    return g.has_x ? DeviceOps::add(DeviceOps::mul(g.sx, x), g.c) : g.c;
}

/* One brick per blockIdx.y; each thread takes runs of R consecutive voxels
 * of a row (x), strided over blockIdx.x and the threads. Along a run only x
 * changes, so per octave the y and z lattice cells, fractions and fades are
 * computed once, and the eight corner hashes and the y / z parts of their
 * gradients only when the x cell changes; every voxel still gets the values
 * of fbm_at's operations (same roundings, same order), so the bytes equal the
 * host generator's. */
template <int R>
__global__ void __launch_bounds__(256)
    fbm_brick_kernel(lv_volume_info info, lv_fbm_params f, const uint16_t* __restrict__ perm,
                     const uint64_t* __restrict__ ids, const uint64_t* __restrict__ offsets,
                     uint8_t* __restrict__ out, uint64_t brick_bytes)
{
    using O = DeviceOps;
    __shared__ uint16_t P[512];
    for (uint32_t i = threadIdx.x; i < 512; i += blockDim.x)
        P[i] = perm[i];
    __syncthreads();
    const uint64_t id = ids[blockIdx.y];
    const FbmBrick b = brick_consts(info, f, id);
    uint8_t* dst = out + (offsets ? offsets[blockIdx.y] : uint64_t(blockIdx.y) * brick_bytes);
    const uint32_t runs_x = (b.N[0] + R - 1) / R;
    const uint32_t n_runs = runs_x * b.N[1] * b.N[2];
    const bool u16 = info.dtype == LV_DT_UINT16;
    const float full = u16 ? 65535.0f : 255.0f;
    auto clampi = [](int32_t g, int32_t hi) { return g < 0 ? 0 : (g > hi ? hi : g); };
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < n_runs;
         w += gridDim.x * blockDim.x)
    {
        /* neighbouring lanes take the same x run of neighbouring rows, so a
         * warp's lanes change x cell at the same voxel (no divergence) */
        const uint32_t j = w % b.N[1], rx = (w / b.N[1]) % runs_x, k = w / (runs_x * b.N[1]);
        const uint32_t i0 = rx * R;
        const uint32_t cnt = min(uint32_t(R), b.N[0] - i0);
        const int32_t gj = clampi(b.base[1] + int32_t(j), b.last[1]);
        const int32_t gk = clampi(b.base[2] + int32_t(k), b.last[2]);
        const float y = O::mul(O::add(float(gj), 0.5f), b.scale);
        const float z = O::mul(O::add(float(gk), 0.5f), b.scale);
        float xs[R], sum[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
        {
            const int32_t gi = clampi(b.base[0] + int32_t(i0 + r), b.last[0]);
            xs[r] = O::mul(O::add(float(gi), 0.5f), b.scale);
            sum[r] = 0.0f;
        }
        float amp = 1.0f, freq = 1.0f;
        for (uint32_t o = 0; o < f.octaves; ++o)
        {
            const float yv = O::mul(y, freq), zv = O::mul(z, freq);
            const float fy = floorf(yv), fz = floorf(zv);
            const uint32_t Y = uint32_t(int32_t(fy)) & 255u, Z = uint32_t(int32_t(fz)) & 255u;
            const float yf = O::sub(yv, fy), zf = O::sub(zv, fz);
            const float v = fade<O>(yf), wz = fade<O>(zf);
            const float y1 = O::sub(yf, 1.0f), z1 = O::sub(zf, 1.0f);
            uint32_t prevX = 0xFFFFFFFFu;
            /* corners (dx, dy, dz): g0 (0,0,0) g1 (1,0,0) g2 (0,1,0) g3 (1,1,0)
             * g4 (0,0,1) g5 (1,0,1) g6 (0,1,1) g7 (1,1,1) */
            CornerGrad g0{}, g1{}, g2{}, g3{}, g4{}, g5{}, g6{}, g7{};
#pragma unroll
            for (int r = 0; r < R; ++r)
            {
                if (uint32_t(r) < cnt)
                {
                    const float xv = O::mul(xs[r], freq);
                    const float fx = floorf(xv);
                    const uint32_t X = uint32_t(int32_t(fx)) & 255u;
                    if (X != prevX)
                    {
                        prevX = X;
                        const uint32_t A = P[X] + Y, AA = P[A] + Z, AB = P[A + 1] + Z;
                        const uint32_t B = P[X + 1] + Y, BA = P[B] + Z, BB = P[B + 1] + Z;
                        g0 = corner_grad(P[AA], yf, zf);
                        g1 = corner_grad(P[BA], yf, zf);
                        g2 = corner_grad(P[AB], y1, zf);
                        g3 = corner_grad(P[BB], y1, zf);
                        g4 = corner_grad(P[AA + 1], yf, z1);
                        g5 = corner_grad(P[BA + 1], yf, z1);
                        g6 = corner_grad(P[AB + 1], y1, z1);
                        g7 = corner_grad(P[BB + 1], y1, z1);
                    }
                    const float xf = O::sub(xv, fx);
                    const float u = fade<O>(xf);
                    const float x1 = O::sub(xf, 1.0f);
                    const float l00 = lerp<O>(u, corner_value(g0, xf), corner_value(g1, x1));
                    const float l10 = lerp<O>(u, corner_value(g2, xf), corner_value(g3, x1));
                    const float l01 = lerp<O>(u, corner_value(g4, xf), corner_value(g5, x1));
                    const float l11 = lerp<O>(u, corner_value(g6, xf), corner_value(g7, x1));
                    const float n = lerp<O>(wz, lerp<O>(v, l00, l10), lerp<O>(v, l01, l11));
                    sum[r] = O::add(sum[r], O::mul(amp, n));
                }
            }
            amp = O::mul(amp, f.gain);
            freq = O::mul(freq, f.lacunarity);
        }
        const uint64_t row = (uint64_t(k) * b.N[1] + j) * b.N[0] + i0;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (uint32_t(r) < cnt)
            {
                const uint32_t q = quantise<O>(sum[r], full);
                if (u16)
                    reinterpret_cast<uint16_t*>(dst)[row + r] = uint16_t(q);
                else
                    dst[row + r] = uint8_t(q);
            }
    }
}

bool valid_params(const lv_fbm_params& f)
{
    return f.octaves >= 1 && f.octaves <= 16 && f.frequency > 0.0f &&
           std::isfinite(f.frequency) && std::isfinite(f.gain) && std::isfinite(f.lacunarity);
}

/* Host generation of one brick over `threads` threads (z slabs). */
void fbm_brick_host(const lv_volume_info& info, const lv_fbm_params& f, const uint16_t* P,
                    uint64_t id, void* dst, uint32_t threads)
{
    const FbmBrick b = brick_consts(info, f, id);
    const bool u16 = info.dtype == LV_DT_UINT16;
    const float full = u16 ? 65535.0f : 255.0f;
    auto slab = [&](uint32_t k0, uint32_t k1) {
        for (uint32_t k = k0; k < k1; ++k)
            for (uint32_t j = 0; j < b.N[1]; ++j)
                for (uint32_t i = 0; i < b.N[0]; ++i)
                {
                    const uint32_t q = quantise<HostOps>(fbm_at<HostOps>(P, f, b, i, j, k), full);
                    const size_t idx = (size_t(k) * b.N[1] + j) * b.N[0] + i;
                    if (u16)
                        static_cast<uint16_t*>(dst)[idx] = uint16_t(q);
                    else
                        static_cast<uint8_t*>(dst)[idx] = uint8_t(q);
                }
    };
    threads = std::max(1u, std::min(threads, b.N[2]));
    if (threads == 1)
    {
        slab(0, b.N[2]);
        return;
    }
    std::vector<std::thread> pool;
    const uint32_t per = (b.N[2] + threads - 1) / threads;
    for (uint32_t t = 1; t < threads; ++t)
    {
        const uint32_t k0 = std::min(b.N[2], t * per), k1 = std::min(b.N[2], k0 + per);
        if (k0 < k1)
            pool.emplace_back(slab, k0, k1);
    }
    slab(0, std::min(b.N[2], per));
    for (auto& th : pool)
        th.join();
}

/* Host data source of an fBm volume (the LV_FBM_HOST placement). */
struct FbmSource
{
    lv_volume_info info;
    lv_fbm_params params;
    std::vector<uint16_t> perm;
    uint32_t threads;
};

int fbm_source_get(void* user, uint64_t id, void* dst, size_t bytes)
{
    const FbmSource* src = static_cast<const FbmSource*>(user);
    const lv_volume_info& v = src->info;
    if (nid_level(id) >= v.depth)
        return 1;
    const uint64_t need = uint64_t(v.max_block[0]) * v.max_block[1] * v.max_block[2] *
                          (v.dtype == LV_DT_UINT16 ? 2u : 1u);
    if (bytes < need)
        return 1;
    fbm_brick_host(v, src->params, src->perm.data(), id, dst, src->threads);
    return 0;
}

void fbm_source_free(void* user) { delete static_cast<FbmSource*>(user); }
} // namespace

std::vector<uint16_t> fbm_permutation(uint64_t seed)
{
    std::vector<uint16_t> p(512);
    for (uint32_t i = 0; i < 256; ++i)
        p[i] = uint16_t(i);
    uint64_t s = seed;
    for (uint32_t i = 255; i >= 1; --i)
    {
        const uint32_t j = uint32_t(splitmix_draw(s) % (i + 1u));
        std::swap(p[i], p[j]);
    }
    for (uint32_t i = 0; i < 256; ++i)
        p[256 + i] = p[i];
    return p;
}

lv_status launch_fbm_bricks(lv_ctx* ctx, const lv_volume_info& info, const lv_fbm_params& f,
                            const uint16_t* d_perm, const uint64_t* d_ids, uint32_t n,
                            uint8_t* out, const uint64_t* d_offsets, uint64_t brick_bytes,
                            cudaStream_t s)
{
    for (uint32_t first = 0; first < n; first += 65535u)
    {
        const uint32_t cnt = std::min(65535u, n - first);
        constexpr int R = 8;
        const uint32_t runs =
            (info.max_block[0] + R - 1) / R * info.max_block[1] * info.max_block[2];
        const dim3 grid(std::min(64u, (runs + 255u) / 256u), cnt);
        fbm_brick_kernel<R><<<grid, 256, 0, s>>>(info, f, d_perm, d_ids + first,
                                               d_offsets ? d_offsets + first : nullptr,
                                               d_offsets ? out : out + first * brick_bytes,
                                               brick_bytes);
        LV_CUDA(ctx, cudaGetLastError());
    }
    return LV_OK;
}

} // namespace lv

using namespace lv;

extern "C" lv_status lv_fbm_brick(const lv_volume_info* info, const lv_fbm_params* params,
                                  uint64_t node_id, void* dst, uint32_t n_threads)
{
    if (!info || !params || !dst || !valid_params(*params) || info->depth == 0 ||
        nid_level(node_id) >= info->depth ||
        (info->dtype != LV_DT_UINT8 && info->dtype != LV_DT_UINT16))
        return LV_EINVAL;
    const std::vector<uint16_t> P = fbm_permutation(params->seed);
    fbm_brick_host(*info, *params, P.data(), node_id, dst, n_threads ? n_threads : 1u);
    return LV_OK;
}

extern "C" lv_status lv_fbm_generate(lv_ctx* ctx, const lv_volume_info* info,
                                     const lv_fbm_params* params, const uint64_t* ids,
                                     uint32_t n, void* d_out, void* stream)
{
    if (!ctx || !info || !params || (n && (!ids || !d_out)) || !valid_params(*params) ||
        (info->dtype != LV_DT_UINT8 && info->dtype != LV_DT_UINT16))
        return fail(ctx, LV_EINVAL, "invalid fBm generation arguments");
    for (uint32_t i = 0; i < n; ++i)
        if (nid_level(ids[i]) >= info->depth)
            return fail(ctx, LV_EINVAL, "node id outside the volume");
    if (n == 0)
        return LV_OK;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const std::vector<uint16_t> P = fbm_permutation(params->seed);
    DeviceBuffer dperm, dids;
    LV_CUDA(ctx, dperm.reserve(sizeof(uint16_t) * P.size()));
    LV_CUDA(ctx, dids.reserve(sizeof(uint64_t) * n));
    LV_CUDA(ctx, cudaMemcpyAsync(dperm.ptr, P.data(), sizeof(uint16_t) * P.size(),
                                 cudaMemcpyHostToDevice, s));
    LV_CUDA(ctx, cudaMemcpyAsync(dids.ptr, ids, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, s));
    const uint64_t brick_bytes = uint64_t(info->max_block[0]) * info->max_block[1] *
                                 info->max_block[2] * (info->dtype == LV_DT_UINT16 ? 2u : 1u);
    lv_status st = launch_fbm_bricks(ctx, *info, *params, dperm.as<uint16_t>(),
                                     dids.as<uint64_t>(), n, static_cast<uint8_t*>(d_out),
                                     nullptr, brick_bytes, s);
    if (st != LV_OK)
        return st;
    /* the temporaries die at return */
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    return LV_OK;
}

extern "C" lv_status lv_volume_create_fbm(lv_ctx* ctx, const lv_volume_info* info,
                                          const lv_fbm_params* params, uint32_t placement,
                                          uint32_t host_threads, lv_volume** out)
{
    if (!ctx || !info || !params || !out)
        return fail(ctx, LV_EINVAL, "null argument");
    if (info->dtype != LV_DT_UINT8 && info->dtype != LV_DT_UINT16)
        return fail(ctx, LV_EINVAL, "fBm volumes are uint8 or uint16");
    if (!valid_params(*params))
        return fail(ctx, LV_EINVAL, "fBm: 1..16 octaves, a positive frequency");
    if (placement == LV_FBM_HOST)
    {
        /* one brick per fetch thread (the generator is re-entrant) */
        FbmSource* src = new FbmSource{*info, *params, fbm_permutation(params->seed), 1u};
        lv_status st = lv_volume_create(ctx, info, fbm_source_get, src, out);
        if (st != LV_OK)
        {
            delete src;
            return st;
        }
        (*out)->user_free = fbm_source_free;
        st = lv_volume_set_fetch_threads(*out, std::min(host_threads, 64u));
        if (st != LV_OK)
        {
            lv_volume_destroy(*out);
            *out = nullptr;
        }
        return st;
    }
    if (placement != LV_FBM_DEVICE)
        return fail(ctx, LV_EINVAL, "unknown fBm placement");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    lv_volume* v = new lv_volume();
    v->ctx = ctx;
    v->info = *info;
    v->fbm = *params;
    v->kind = SRC_FBM_DEVICE;
    lv_status st = volume_init(ctx, v);
    if (st != LV_OK)
    {
        delete v;
        return st;
    }
    const std::vector<uint16_t> P = fbm_permutation(params->seed);
    if (v->d_perm.reserve(sizeof(uint16_t) * P.size()) != cudaSuccess ||
        cudaMemcpy(v->d_perm.ptr, P.data(), sizeof(uint16_t) * P.size(),
                   cudaMemcpyHostToDevice) != cudaSuccess)
    {
        delete v;
        return fail(ctx, LV_ENOMEM, "fBm permutation table");
    }
    *out = v;
    return LV_OK;
}
